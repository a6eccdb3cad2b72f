// Property check of the persistent kernel's work queue (build_batch_items in
// finetools.jl_gb300/csrc/batch_queue.cpp), run on the host by
// tests/test_batch_queue.py.
//
// Random job sets (chunk counts, spans, rings, tiles, node ranges) are turned
// into queues, and the queues are executed by a discrete-event simulation of
// P persistent CTAs that take items in queue order, wait for the item's
// dependency counters and run for a random time.  Checked for every run:
//   - every item completes (no wait can block forever);
//   - an element item of chunk c of a job starts only after every reader of
//     its ring slot's previous chunk (gathers c - ring .. c - ring + span) has
//     completed;
//   - a gather item of chunk c starts only after the element items of chunks
//     c - span .. c have completed;
//   - every element of every job is covered by exactly one element item and
//     every gather-order node by exactly one gather item.
// Every other trial runs each job as slices of 1-3 chunks in successive
// launches (fresh counters per launch, the chunks' completion carried over),
// as the serving loop's rounds do; the same properties are checked across
// the launches.
// Prints "ok" and exits 0, or prints the first violation and exits 1.
#include <algorithm>
#include <cstdio>
#include <map>
#include <queue>
#include <random>
#include <vector>

#include "batch_host.h"

using namespace fegpu;

namespace {

using DoneMap = std::map<std::pair<int, int64_t>, int>;

// Runs one launch's items on P simulated CTAs; the per-chunk totals and done
// counts carry over between launches (a sliced job's earlier chunks ran in
// earlier launches on the same stream).
bool execute(std::mt19937_64 &rng, int P, const std::vector<BatchItem> &items, int ncounters,
             const std::vector<const fegpu_dofmap *> &dms, DoneMap &etotal, DoneMap &gtotal,
             DoneMap &edone, DoneMap &gdone) {
  const int n = static_cast<int>(items.size());
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 2; ++d)
      if (items[i].dep[d] >= ncounters || items[i].done >= ncounters)
        return std::printf("item %d: counter out of range\n", i), false;
  for (const auto &I : items) (I.kind == 0 ? etotal : gtotal)[{I.job, I.chunk}]++;
  std::vector<int> counters(ncounters, 0);
  std::vector<int> state(n, 0);  // 0 queued, 1 running, 2 done
  std::vector<double> finish(n, 0.0);
  std::vector<int> cta_item(P, -1);
  int next = 0, completed = 0;
  double now = 0.0;
  // item durations with a heavy tail, so that late stragglers overlap later stages
  std::uniform_real_distribution<double> unif(0.1, 3.0);
  auto dur = [&](std::mt19937_64 &g) { return (g() % 8 == 0 ? 40.0 : 1.0) * unif(g); };
  auto ready = [&](const BatchItem &I) {
    for (int d = 0; d < 2; ++d)
      if (I.dep[d] >= 0 && counters[I.dep[d]] < I.target[d]) return false;
    return true;
  };
  auto chunk_done = [&](DoneMap &done, DoneMap &total, int job, int64_t c) {
    return done[{job, c}] == total[{job, c}];
  };
  int guard = 0;
  while (completed < n) {
    if (++guard > 100 * n + 1000) return std::printf("no progress (deadlock)\n"), false;
    bool progressed = false;
    // idle CTAs take the next items in queue order; a CTA whose item is not
    // ready keeps it (it waits)
    for (int p = 0; p < P; ++p) {
      if (cta_item[p] < 0 && next < n) cta_item[p] = next++;
      const int i = cta_item[p];
      if (i >= 0 && state[i] == 0 && ready(items[i])) {
        const BatchItem &I = items[i];
        const fegpu_dofmap *dm = dms[I.job];
        if (I.kind == 0 && I.chunk >= dm->ring) {
          const int64_t prev = I.chunk - dm->ring;
          for (int64_t g = prev; g <= prev + dm->span && g < static_cast<int64_t>(dm->chunk_nodes.size()) - 1; ++g)
            if (!chunk_done(gdone, gtotal, I.job, g) || gtotal[{I.job, g}] == 0)
              return std::printf("element item of job %d chunk %lld overwrites the slot of "
                                 "chunk %lld while gather %lld runs\n",
                                 I.job, (long long)I.chunk, (long long)prev, (long long)g),
                     false;
        }
        if (I.kind == 1) {
          for (int64_t c = std::max<int64_t>(0, I.chunk - dm->span); c <= I.chunk; ++c)
            if (!chunk_done(edone, etotal, I.job, c) || etotal[{I.job, c}] == 0)
              return std::printf("gather of job %d chunk %lld starts before elements of "
                                 "chunk %lld\n",
                                 I.job, (long long)I.chunk, (long long)c),
                     false;
        }
        state[i] = 1;
        finish[i] = now + dur(rng);
        progressed = true;
      }
    }
    // advance to the next completion
    double t = 1e300;
    int who = -1;
    for (int p = 0; p < P; ++p) {
      const int i = cta_item[p];
      if (i >= 0 && state[i] == 1 && finish[i] < t) {
        t = finish[i];
        who = p;
      }
    }
    if (who < 0) {
      if (!progressed) return std::printf("deadlock: no running item\n"), false;
      continue;
    }
    now = t;
    const int i = cta_item[who];
    const BatchItem &I = items[i];
    state[i] = 2;
    counters[I.done]++;
    (I.kind == 0 ? edone : gdone)[{I.job, I.chunk}]++;
    cta_item[who] = -1;
    completed++;
  }
  return true;
}

// sliced = false: every job in one launch; true: every job cut into slices of
// 1 to 3 chunks run by successive launches (the serving loop's rounds)
bool run(std::mt19937_64 &rng, int njobs, int P, size_t budget, bool sliced) {
  std::vector<std::unique_ptr<fegpu_femm>> femms;
  std::vector<std::unique_ptr<fegpu_dofmap>> dmaps;
  std::vector<BatchJob> jobs(njobs);
  std::vector<const fegpu_dofmap *> dms;
  for (int j = 0; j < njobs; ++j) {
    auto fm = std::make_unique<fegpu_femm>();
    auto dm = std::make_unique<fegpu_dofmap>();
    const int nch = 1 + static_cast<int>(rng() % 9);
    const int64_t chunk = 1 + static_cast<int64_t>(rng() % 50);
    fm->nelem = (nch - 1) * chunk + 1 + static_cast<int64_t>(rng() % chunk);
    dm->femm = fm.get();
    dm->chunk = chunk;
    dm->span = static_cast<int>(rng() % 3);
    dm->ring = std::min(dm->span + 2, nch);
    dm->chunk_nodes.assign(1, 0);
    for (int c = 0; c < nch; ++c)
      dm->chunk_nodes.push_back(dm->chunk_nodes.back() + static_cast<int64_t>(rng() % 150));
    jobs[j].k.te = 1 + static_cast<int>(rng() % 9);
    jobs[j].elem_floats = 1 + static_cast<int64_t>(rng() % 2000);
    dms.push_back(dm.get());
    femms.push_back(std::move(fm));
    dmaps.push_back(std::move(dm));
  }
  DoneMap etotal, gtotal, edone, gdone;
  std::vector<BatchItem> all;
  if (!sliced) {
    std::vector<BatchItem> items;
    const int nc = build_batch_items(jobs, dms, budget, items);
    if (!execute(rng, P, items, nc, dms, etotal, gtotal, edone, gdone)) return false;
    all = items;
  } else {
    std::vector<int64_t> at(njobs, 0);
    for (;;) {
      std::vector<ChunkRange> ranges(njobs);
      bool any = false;
      for (int j = 0; j < njobs; ++j) {
        const int64_t nch = static_cast<int64_t>(dms[j]->chunk_nodes.size()) - 1;
        const int64_t c1 = std::min(nch, at[j] + 1 + static_cast<int64_t>(rng() % 3));
        ranges[j] = ChunkRange{at[j], c1};
        any = any || c1 > at[j];
        at[j] = c1;
      }
      if (!any) break;
      std::vector<BatchItem> items;
      const int nc = build_batch_items(jobs, dms, budget, items, &ranges);
      if (!execute(rng, P, items, nc, dms, etotal, gtotal, edone, gdone)) return false;
      all.insert(all.end(), items.begin(), items.end());
    }
  }
  // coverage
  for (int j = 0; j < njobs; ++j) {
    std::vector<int> ecov(dms[j]->femm->nelem, 0), ncov(dms[j]->chunk_nodes.back(), 0);
    for (const auto &I : all) {
      if (I.job != j) continue;
      auto &cov = I.kind == 0 ? ecov : ncov;
      for (int64_t x = I.b; x < I.e; ++x) cov[x]++;
    }
    for (int v : ecov)
      if (v != 1) return std::printf("job %d: element coverage %d\n", j, v), false;
    for (int v : ncov)
      if (v != 1) return std::printf("job %d: node coverage %d\n", j, v), false;
  }
  return true;
}

}  // namespace

int main() {
  std::mt19937_64 rng(12345);
  for (int trial = 0; trial < 1500; ++trial) {
    const int njobs = 1 + static_cast<int>(rng() % 6);
    const int P = std::vector<int>{1, 2, 3, 7, 64}[rng() % 5];
    const size_t budget = std::vector<size_t>{1, 4096, 1u << 20, 64u << 20}[rng() % 4];
    const bool sliced = trial % 2 == 1;
    if (!run(rng, njobs, P, budget, sliced)) {
      std::printf("trial %d failed (jobs %d, ctas %d, %s)\n", trial, njobs, P,
                  sliced ? "sliced" : "one launch");
      return 1;
    }
  }
  std::printf("ok\n");
  return 0;
}
