// Queue order of the persistent assembly kernel's work items (host only; see
// batch_host.h for the schedule and batch.cu for the kernel that runs it).
#include <algorithm>

#include "batch_host.h"

namespace fegpu {

int build_batch_items(const std::vector<BatchJob> &jobs,
                      const std::vector<const fegpu_dofmap *> &dms, size_t live_budget,
                      std::vector<BatchItem> &items, const std::vector<ChunkRange> *ranges) {
  const size_t njobs = jobs.size();
  items.clear();
  std::vector<int> base(njobs), nchunk(njobs);
  std::vector<int64_t> first(njobs, 0);
  int ncount = 0;
  for (size_t j = 0; j < njobs; ++j) {
    const int64_t all = static_cast<int64_t>(dms[j]->chunk_nodes.size()) - 1;
    if (ranges) {
      const ChunkRange r = (*ranges)[j];
      FEGPU_REQUIRE(0 <= r.c0 && r.c0 <= r.c1 && r.c1 <= std::max<int64_t>(all, 0),
                    "batch: chunk range outside the job");
      first[j] = r.c0;
      nchunk[j] = static_cast<int>(r.c1 - r.c0);
    } else {
      nchunk[j] = static_cast<int>(all);
    }
    base[j] = ncount;
    ncount += 2 * std::max(nchunk[j], 0);
  }
  std::vector<int> count(std::max(ncount, 1), 0);  // items per stage
  // counters: E(c) -> base + 2(c - first), G(c) -> base + 2(c - first) + 1.
  // A dependency on a stage before the job's first chunk (a slice continuing a
  // job run by an earlier launch on the same stream) is already met and is
  // left out.
  auto emit_stage = [&](size_t j, bool gather, int64_t c) {
    const BatchJob &J = jobs[j];
    const fegpu_dofmap *dm = dms[j];
    const int64_t c0 = first[j];
    auto ctr_of = [&](int64_t cc, bool g) { return base[j] + 2 * static_cast<int>(cc - c0) + (g ? 1 : 0); };
    const int ctr = ctr_of(c, gather);
    int dep[2] = {-1, -1}, target[2] = {0, 0};
    if (!gather) {
      if (c - 1 >= c0) dep[0] = ctr_of(c - 1, false);
      // the ring slot of chunk c last held chunk c - ring, read by gathers up
      // to G(c - ring + span)
      if (c >= dm->ring && c - dm->ring + dm->span >= c0)
        dep[1] = ctr_of(c - dm->ring + dm->span, true);
    } else {
      // G(c) reads the blocks of chunks c - span .. c; gathers complete in
      // order, so the wait of E(c + ring) above covers every reader of a slot
      dep[0] = ctr_of(c, false);
      if (c - 1 >= c0) dep[1] = ctr_of(c - 1, true);
    }
    for (int d = 0; d < 2; ++d)
      if (dep[d] >= 0) target[d] = count[dep[d]];
    auto push = [&](int kind, int64_t x0, int64_t x1) {
      items.push_back(BatchItem{static_cast<int>(j), kind, x0, x1, c, {dep[0], dep[1]},
                                {target[0], target[1]}, ctr, 0});
      count[ctr]++;
    };
    if (!gather) {
      const int64_t e0 = c * dm->chunk, e1 = std::min(dm->femm->nelem, (c + 1) * dm->chunk);
      for (int64_t x = e0; x < e1; x += J.k.te) push(0, x, std::min(e1, x + J.k.te));
      if (e0 >= e1) push(0, e0, e0);
    } else {
      const int64_t n0 = dm->chunk_nodes[c], n1 = dm->chunk_nodes[c + 1];
      for (int64_t x = n0; x < n1; x += kBatchGatherNodes)
        push(1, x, std::min(n1, x + kBatchGatherNodes));
      if (n0 >= n1) push(1, n0, n0);  // a stage without nodes still completes
    }
  };
  // per job the stage sequence E0, E1, G0, E2, G1, ..., E(n-1), G(n-2), G(n-1)
  auto stage_of = [&](size_t j, int k, bool &gather, int64_t &c) {
    const int n = nchunk[j];
    if (k == 0) {
      gather = false;
      c = 0;
    } else if (k == 2 * n - 1) {
      gather = true;
      c = n - 1;
    } else if (k % 2 == 1) {
      gather = false;
      c = (k + 1) / 2;
    } else {
      gather = true;
      c = k / 2 - 1;
    }
  };
  auto live_bytes = [&](size_t j) {
    const int64_t e = std::min<int64_t>(dms[j]->chunk, dms[j]->femm->nelem);
    return static_cast<size_t>(dms[j]->ring) * e * jobs[j].elem_floats * sizeof(float);
  };
  std::vector<size_t> window;
  std::vector<int> next(njobs, 0);
  size_t admitted = 0, live = 0;
  auto admit = [&]() {
    while (admitted < njobs && (window.size() < 2 || live + live_bytes(admitted) <= live_budget)) {
      if (nchunk[admitted] > 0) {
        window.push_back(admitted);
        live += live_bytes(admitted);
      }
      ++admitted;
    }
  };
  admit();
  while (!window.empty()) {
    std::vector<size_t> keep;
    for (size_t j : window) {
      bool gather;
      int64_t c;
      stage_of(j, next[j]++, gather, c);
      emit_stage(j, gather, first[j] + c);
      if (next[j] < 2 * nchunk[j]) keep.push_back(j);
      else live -= live_bytes(j);
    }
    window.swap(keep);
    admit();
  }
  FEGPU_REQUIRE(items.size() < (1u << 31), "batch: too many work items");
  return std::max(ncount, 1);
}

}  // namespace fegpu
