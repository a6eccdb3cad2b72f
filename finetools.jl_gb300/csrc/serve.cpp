// Serving loop: re-assembly requests on resident meshes, continuously batched
// on concurrent lanes, with bounded work per launch.
//
// A server keeps meshes resident on the device (connectivity, colouring, CSR
// pattern, gather plan, block ring, coefficient buffer, matrix values) and
// accepts requests that carry new per-element coefficients or new node
// coordinates for one of them.  A worker thread launches batches of the
// persistent assembly kernel (batch.cu) on `lanes` CUDA streams.  When a lane
// is free its next batch holds the next slice of every request running on it
// and the oldest waiting request of every mesh with none running, up to a job
// limit; a slice is at most slice_elements elements of a request's mesh, in
// whole chunks, so a 2 M-element mesh is assembled over several launches of
// its lane and cannot hold the lane for its whole assembly: requests that
// arrive meanwhile join the lane's next launch or start on another lane
// (continuous batching).  A request's slices run in order on its lane (its
// block ring carries over from one launch to the next).  A launch covers
// 1/(1 + lanes running) of the GPU: all of it when the others are idle.
// Requests of one mesh run in arrival order (at most one running per mesh).
//
// Admission: a mesh is added only if the device memory it still needs to be
// served (gather plan, block ring, coefficient and staging buffers) fits in
// the free memory, and, under a memory limit, if everything the server's
// meshes hold stays within it; otherwise the call returns FEGPU_ERR_MEMORY
// and the caller can remove a mesh and try again.  Meshes can be added and
// removed while requests stream.
//
// Precision: the lanes evaluate every request as the mixed-precision batch
// path.  A server set to FEGPU_FP64 or FEGPU_FP64_FAST instead runs each
// request by itself through the single-call form on the context's stream (the
// FP64 forms have no batched kernel), in arrival order.
//
// Completion times come from a host callback queued on the lane stream behind
// the kernel (cudaLaunchHostFunc), so latencies include queueing, the
// host-to-device copy of the request data and the assembly.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch_host.h"

using namespace fegpu;

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Page-locked host buffers recycled by size (request payloads, lane staging).
struct PinnedPool {
  std::mutex mu;
  std::multimap<size_t, void *> free_blocks;
  std::vector<void *> all;
  void *get(size_t bytes) {
    {
      std::lock_guard<std::mutex> lock(mu);
      auto it = free_blocks.lower_bound(bytes);
      if (it != free_blocks.end() && it->first <= 2 * bytes + 4096) {
        void *p = it->second;
        free_blocks.erase(it);
        return p;
      }
    }
    void *p = nullptr;
    FEGPU_CUDA(cudaMallocHost(&p, std::max<size_t>(bytes, 64) + sizeof(size_t)));
    *static_cast<size_t *>(p) = std::max<size_t>(bytes, 64);
    std::lock_guard<std::mutex> lock(mu);
    all.push_back(p);
    return p;
  }
  void put(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(mu);
    free_blocks.emplace(*static_cast<size_t *>(p), p);
  }
  static void *data(void *p) { return static_cast<char *>(p) + sizeof(size_t); }
  ~PinnedPool() {
    for (void *p : all) cudaFreeHost(p);
  }
};

constexpr int kReqPending = 0, kReqRunning = 1, kReqDone = 2, kReqFailed = 3,
              kReqCancelled = 4;

}  // namespace

struct fegpu_server {
  fegpu_context *ctx = nullptr;
  int nlanes = 2;
  int max_jobs = 64;
  double wait_s = 5.0;
  int64_t slice_elements = 16384;     // elements of one request per launch
  int precision = FEGPU_MIXED;
  int64_t mem_limit = 0;              // bytes the served meshes may hold (0: no limit)
  int64_t mem_held = 0;               // bytes they hold

  struct Mesh {
    fegpu_matrix *K = nullptr;
    int form = 0, code = 0, m = 3;
    BatchJob d{};
    std::unique_ptr<DevBuf> coef;     // coefficient values read by the kernel
    std::unique_ptr<DevBuf> ring;     // private ring when the dofmap is shared
    DevBuf xyz_stage;                 // column-major coordinates of an update
    int64_t coef_values = 0;          // doubles per coefficient update (0: constant)
    fegpu_coef cf{};                  // the coefficient (FP64 servers: host copy)
    std::vector<double> cf_host;
    int64_t bytes = 0;                // device bytes the mesh holds
    bool busy = false;                // a request of this mesh is in flight
    bool removed = false;
  };
  std::vector<std::unique_ptr<Mesh>> meshes;

  struct Request {
    int64_t mesh = 0;
    int kind = 0;
    void *payload = nullptr;          // pinned block
    size_t bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int state = kReqPending;
    int64_t next_chunk = 0;           // first chunk of its next slice
    int lane = -1;                    // the lane its slices run on
  };
  std::unordered_map<int64_t, Request> requests;
  std::deque<int64_t> pending;        // waiting, arrival order
  std::deque<int64_t> active;         // running (more slices to come), arrival order
  int64_t next_id = 0;

  struct Lane {
    cudaStream_t stream = nullptr;
    DevBuf d_jobs, d_items, d_counters, d_next, d_status;
    void *h_jobs = nullptr, *h_items = nullptr;  // pinned staging (pool blocks)
    int *h_status = nullptr;
    std::vector<int64_t> finishing;   // requests whose last slice is in this launch
    std::vector<int64_t> members;     // every request with a slice in this launch
    bool busy = false;
    fegpu_server *srv = nullptr;
  };
  std::vector<std::unique_ptr<Lane>> lanes;

  PinnedPool pool;
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool stop = false;
  bool hold = false;                  // launches paused (requests accumulate)
  std::string worker_error;
  int64_t batches = 0, jobs_run = 0;
};

namespace {

int64_t chunks_of(const fegpu_server::Mesh &M) {
  return std::max<int64_t>(static_cast<int64_t>(M.K->dm->chunk_nodes.size()) - 1, 0);
}

void lane_done(void *arg) {  // CUDA host callback: no CUDA calls here
  auto *R = static_cast<fegpu_server::Lane *>(arg);
  fegpu_server *s = R->srv;
  const double t = now_ms();
  std::lock_guard<std::mutex> lock(s->mu);
  const bool ok = *R->h_status == 0;
  // (a request failed by an earlier launch may already be collected: look up)
  if (!ok) {
    // every request with a slice in this launch is void; requests still
    // running lose their remaining slices
    for (int64_t id : R->members) {
      auto it = s->requests.find(id);
      if (it != s->requests.end() && it->second.state == kReqRunning) {
        it->second.state = kReqFailed;
        it->second.t_done = t;
        s->meshes[it->second.mesh]->busy = false;
      }
    }
    std::deque<int64_t> keep;
    for (int64_t id : s->active)
      if (s->requests[id].state == kReqRunning) keep.push_back(id);
    s->active.swap(keep);
  }
  for (int64_t id : R->finishing) {
    auto it = s->requests.find(id);
    if (it != s->requests.end() && it->second.state == kReqRunning) {
      it->second.state = kReqDone;
      it->second.t_done = t;
      s->meshes[it->second.mesh]->busy = false;
    }
  }
  // the payloads of requests that ended here were copied by this launch or an
  // earlier one of the lane: back to the pool for the next submissions
  for (int64_t id : R->members) {
    auto it = s->requests.find(id);
    if (it != s->requests.end() && it->second.state >= kReqDone) {
      s->pool.put(it->second.payload);
      it->second.payload = nullptr;
    }
  }
  R->finishing.clear();
  R->members.clear();
  R->busy = false;
  s->cv.notify_all();
}

// Lane buffers grow by half again when they must grow, so that steady traffic
// stops reallocating (cudaFree can stall behind the other lanes' work).
void grow(DevBuf &b, size_t n) {
  if (n > b.bytes) b.alloc(std::max(n, b.bytes + b.bytes / 2));
}

// One launch of a lane: uploads of the requests starting now, the items of
// every slice, the kernel on `share` of the GPU, the completion callback
// (worker thread, no lock held).
void launch_lane(fegpu_server *s, fegpu_server::Lane &R, const std::vector<int64_t> &ids,
                 const std::vector<ChunkRange> &ranges, const std::vector<char> &starts,
                 double share) {
  cudaStream_t st = R.stream;
  std::vector<BatchJob> jobs;
  std::vector<const fegpu_dofmap *> dms;
  for (size_t k = 0; k < ids.size(); ++k) {
    // the request and its mesh are looked up under the lock: a concurrent
    // submission or admission may grow the request map or the mesh list
    // (the objects themselves stay where they are)
    fegpu_server::Request *r;
    fegpu_server::Mesh *Mp;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      r = &s->requests[ids[k]];
      Mp = s->meshes[r->mesh].get();
    }
    fegpu_server::Mesh &M = *Mp;
    fegpu_femm *fm = M.K->dm->femm;
    if (starts[k]) {
      if (r->kind == FEGPU_REQUEST_COEF) {
        FEGPU_CUDA(cudaMemcpyAsync(M.coef->p, PinnedPool::data(r->payload), r->bytes,
                                   cudaMemcpyHostToDevice, st));
      } else {
        FEGPU_CUDA(cudaMemcpyAsync(M.xyz_stage.p, PinnedPool::data(r->payload), r->bytes,
                                   cudaMemcpyHostToDevice, st));
        pack_geometry(M.xyz_stage.as<double>(), fm->nnodes, fm->sdim, fm->xyz.as<double>(), st);
      }
    }
    jobs.push_back(M.d);
    dms.push_back(M.K->dm);
  }
  std::vector<BatchItem> items;
  const int ncount = build_batch_items(jobs, dms, 64u << 20, items, &ranges);
  const size_t smem = batch_smem_bytes(jobs, dms);
  const int nitems = static_cast<int>(items.size());
  const int grid = batch_grid(s->ctx->num_sms, smem, nitems, share);
  // staging: the lane's pinned blocks are free (its previous launch is done)
  const size_t jb = sizeof(BatchJob) * jobs.size(), ib = sizeof(BatchItem) * items.size();
  s->pool.put(R.h_jobs);
  s->pool.put(R.h_items);
  R.h_jobs = s->pool.get(jb);
  R.h_items = s->pool.get(ib);
  std::memcpy(PinnedPool::data(R.h_jobs), jobs.data(), jb);
  std::memcpy(PinnedPool::data(R.h_items), items.data(), ib);
  grow(R.d_jobs, jb);
  grow(R.d_items, ib);
  grow(R.d_counters, sizeof(int) * ncount);
  FEGPU_CUDA(cudaMemcpyAsync(R.d_jobs.p, PinnedPool::data(R.h_jobs), jb, cudaMemcpyHostToDevice, st));
  FEGPU_CUDA(cudaMemcpyAsync(R.d_items.p, PinnedPool::data(R.h_items), ib, cudaMemcpyHostToDevice, st));
  FEGPU_CUDA(cudaMemsetAsync(R.d_counters.p, 0, sizeof(int) * ncount, st));
  FEGPU_CUDA(cudaMemsetAsync(R.d_next.p, 0, sizeof(int), st));
  FEGPU_CUDA(cudaMemsetAsync(R.d_status.p, 0, sizeof(int), st));
  launch_batch_kernel(grid, smem, st, R.d_jobs.as<BatchJob>(), R.d_items.as<BatchItem>(), nitems,
                      R.d_next.as<int>(), R.d_counters.as<int>(), R.d_status.as<int>(), s->wait_s);
  FEGPU_CUDA(cudaMemcpyAsync(R.h_status, R.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FEGPU_CUDA(cudaLaunchHostFunc(st, lane_done, &R));
}

// One FP64 request through the single-call form (worker thread, no lock held).
void run_fp64(fegpu_server *s, int64_t id) {
  fegpu_server::Request *r;
  fegpu_server::Mesh *Mp;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    r = &s->requests[id];
    Mp = s->meshes[r->mesh].get();
  }
  fegpu_server::Mesh &M = *Mp;
  fegpu_femm *fm = M.K->dm->femm;
  fegpu_coef cf = M.cf;
  if (r->kind == FEGPU_REQUEST_COEF) {
    std::memcpy(M.cf_host.data(), PinnedPool::data(r->payload), r->bytes);
  } else {
    FEGPU_CUDA(cudaMemcpyAsync(M.xyz_stage.p, PinnedPool::data(r->payload), r->bytes,
                               cudaMemcpyHostToDevice, s->ctx->stream));
    pack_geometry(M.xyz_stage.as<double>(), fm->nnodes, fm->sdim, fm->xyz.as<double>(),
                  s->ctx->stream);
  }
  cf.data = M.cf_host.data();
  int st;
  if (M.form == F_DIFF_ISO) st = fegpu_bilform_diffusion(M.K, &cf, s->precision);
  else if (M.form == F_ELAST_ISO) st = fegpu_bilform_lin_elastic(M.K, &cf, s->precision);
  else st = fegpu_bilform_dot(M.K, &cf, M.m, 1, s->precision);
  if (st != FEGPU_OK) throw Error{st, fegpu_last_error()};
}

void worker_main(fegpu_server *s) {
  cudaSetDevice(s->ctx->device);
  for (;;) {
    fegpu_server::Lane *R = nullptr;
    double share = 1.0;
    std::vector<int64_t> ids;
    std::vector<ChunkRange> ranges;
    std::vector<char> starts;
    std::vector<int64_t> finishing;
    bool fp64 = false;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv.wait(lock, [&] {
        if (s->stop) return true;
        if (s->hold || (s->pending.empty() && s->active.empty())) return false;
        if (!s->pending.empty() && s->precision != FEGPU_MIXED) return true;
        for (auto &x : s->lanes) {
          if (x->busy) continue;
          // a free lane with work: a request running on it, or one waiting
          if (!s->pending.empty()) return true;
          const int li = static_cast<int>(&x - &s->lanes[0]);
          for (int64_t id : s->active)
            if (s->requests[id].lane == li) return true;
        }
        return false;
      });
      if (s->stop) return;
      fp64 = s->precision != FEGPU_MIXED;
      if (fp64) {
        // one request at a time, in arrival order
        const int64_t id = s->pending.front();
        s->pending.pop_front();
        auto &r = s->requests[id];
        r.state = kReqRunning;
        r.t_start = now_ms();
        ids.push_back(id);
      } else {
        // a free lane with a request running on it first (its next slice
        // waits for that lane), else the first free lane
        int li = -1;
        for (int64_t id : s->active) {
          const int l = s->requests[id].lane;
          if (!s->lanes[l]->busy) {
            li = l;
            break;
          }
        }
        for (int l = 0; li < 0 && l < s->nlanes; ++l)
          if (!s->lanes[l]->busy) li = l;
        R = s->lanes[li].get();
        // the launch takes its share of the GPU beside the lanes running now
        // (all of it when they are idle): persistent blocks keep their SMs
        // until the launch ends, so a launch sized for the whole GPU would
        // make the next lane's launch wait for it
        int running = 0;
        for (auto &x : s->lanes) running += x->busy ? 1 : 0;
        share = 1.0 / (1 + running);
        // the next slice of every request running on this lane, then the
        // oldest waiting request of each mesh with none running
        auto take_slice = [&](int64_t id, bool start) {
          auto &r = s->requests[id];
          const auto &M = *s->meshes[r.mesh];
          const int64_t nch = chunks_of(M);
          const int64_t per = std::max<int64_t>(1, s->slice_elements / std::max<int64_t>(
                                                                           M.K->dm->chunk, 1));
          const int64_t c0 = r.next_chunk, c1 = std::min(nch, c0 + per);
          ids.push_back(id);
          ranges.push_back(ChunkRange{c0, c1});
          starts.push_back(start ? 1 : 0);
          r.next_chunk = c1;
          if (c1 >= nch) finishing.push_back(id);
        };
        std::deque<int64_t> still;
        for (int64_t id : s->active) {
          const auto &r = s->requests[id];
          if (r.lane != li || static_cast<int>(ids.size()) >= s->max_jobs) {
            still.push_back(id);
            continue;
          }
          take_slice(id, false);
          if (r.next_chunk < chunks_of(*s->meshes[r.mesh])) still.push_back(id);
        }
        std::deque<int64_t> rest;
        for (int64_t id : s->pending) {
          auto &r = s->requests[id];
          auto &M = *s->meshes[r.mesh];
          if (static_cast<int>(ids.size()) < s->max_jobs && !M.busy) {
            M.busy = true;
            r.state = kReqRunning;
            r.t_start = now_ms();
            r.next_chunk = 0;
            r.lane = li;
            take_slice(id, true);
            if (r.next_chunk < chunks_of(M)) still.push_back(id);
          } else {
            rest.push_back(id);
          }
        }
        if (ids.empty()) {
          // every waiting request waits for its mesh: sleep until a launch ends
          s->cv.wait(lock);
          continue;
        }
        s->pending.swap(rest);
        s->active.swap(still);
        R->busy = true;
        R->finishing = finishing;
        R->members = ids;
      }
    }
    try {
      if (fp64) {
        run_fp64(s, ids[0]);
        std::lock_guard<std::mutex> lock(s->mu);
        auto &r = s->requests[ids[0]];
        r.state = kReqDone;
        r.t_done = now_ms();
        s->pool.put(r.payload);  // copied (coordinates: the stream synchronized)
        r.payload = nullptr;
        s->batches++;
        s->jobs_run++;
        s->cv.notify_all();
      } else {
        launch_lane(s, *R, ids, ranges, starts, share);
        std::lock_guard<std::mutex> lock(s->mu);
        s->batches++;
        s->jobs_run += static_cast<int64_t>(ids.size());
      }
    } catch (const Error &e) {
      std::lock_guard<std::mutex> lock(s->mu);
      s->worker_error = e.msg;
      for (int64_t id : ids) {
        auto &r = s->requests[id];
        r.state = kReqFailed;
        r.t_done = now_ms();
        s->meshes[r.mesh]->busy = false;
      }
      std::deque<int64_t> keep;
      for (int64_t id : s->active)
        if (s->requests[id].state == kReqRunning) keep.push_back(id);
      s->active.swap(keep);
      if (R) {
        R->finishing.clear();
        R->members.clear();
        R->busy = false;
      }
      s->cv.notify_all();
    }
  }
}

template <typename F>
int server_guard(F &&f) {
  try {
    f();
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc &) {
    set_error("host allocation failed");
    return FEGPU_ERR_MEMORY;
  } catch (const std::exception &e) {
    set_error(e.what());
    return FEGPU_ERR_STATE;
  }
}

// Device bytes of a mesh's femm, DOF map and matrix (already allocated by the
// caller), and what serving it adds: the gather plan (if not built yet), a
// private ring (dofmap shared with another served matrix), the coefficient
// buffer and the coordinate staging buffer.
int64_t resident_bytes(const fegpu_matrix *K) {
  const fegpu_dofmap *dm = K->dm;
  const fegpu_femm *fm = dm->femm;
  const int64_t E = fm->nelem, N = fm->nnodes, nne = fm->nne, ndn = dm->ndn;
  return 2 * E * nne * 4 + E * 4 + N * 32 +                      // femm
         (dm->ndof + 1) * 8 + dm->nnz * 4 + E * nne * nne * 2 +  // pattern, slot maps
         N * ndn * 4 + (N + 1) * 8 + dm->nnz * 8;                // DOFs, adjacency, values
}

int64_t serving_bytes(const fegpu_matrix *K, bool private_ring, int64_t coef_values) {
  const fegpu_dofmap *dm = K->dm;
  const fegpu_femm *fm = dm->femm;
  const int64_t E = fm->nelem, N = fm->nnodes, nne = fm->nne, ndn = dm->ndn;
  const int64_t block_floats = nne * (nne + 1) / 2 * ndn * ndn;
  int64_t ring_bytes = dm->ke.bytes;
  if (!dm->gather_ready) {
    // chunks of ~24 MB of blocks; the ring holds span + 2 of them (at most 4
    // on block meshes; counted as 4)
    const int64_t chunk = std::min<int64_t>(std::max<int64_t>(1024, (24ll << 20) / (block_floats * 4)),
                                            std::max<int64_t>(E, 1));
    ring_bytes = 4 * chunk * block_floats * 4;
  }
  int64_t b = 0;
  if (!dm->gather_ready)
    b += (N + 1) * 8 + E * nne * (4 + 1 + 4) + N * 4 + E * nne * nne * 2 + ring_bytes;
  if (private_ring) b += ring_bytes;
  b += coef_values * 8 + N * fm->sdim * 8;
  return b;
}

}  // namespace

extern "C" {

int fegpu_server_create(fegpu_context *ctx, int lanes, int max_jobs, fegpu_server **out) {
  return server_guard([&] {
    FEGPU_REQUIRE(ctx && out, "null handle");
    FEGPU_REQUIRE(lanes >= 1 && lanes <= 16, "server: 1 to 16 lanes");
    FEGPU_REQUIRE(max_jobs >= 1, "server: max_jobs must be positive");
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    auto s = std::make_unique<fegpu_server>();
    s->ctx = ctx;
    s->nlanes = lanes;
    s->max_jobs = max_jobs;
    // lanes at the highest stream priority: their blocks are scheduled ahead
    // of mesh admissions and other work on the context's stream
    int least = 0, greatest = 0;
    FEGPU_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    for (int i = 0; i < lanes; ++i) {
      auto L = std::make_unique<fegpu_server::Lane>();
      L->srv = s.get();
      FEGPU_CUDA(cudaStreamCreateWithPriority(&L->stream, cudaStreamNonBlocking, greatest));
      L->d_next.alloc(sizeof(int));
      L->d_status.alloc(sizeof(int));
      FEGPU_CUDA(cudaMallocHost(reinterpret_cast<void **>(&L->h_status), sizeof(int)));
      s->lanes.push_back(std::move(L));
    }
    fegpu_server *raw = s.release();
    raw->worker = std::thread(worker_main, raw);
    *out = raw;
  });
}

int fegpu_server_destroy(fegpu_server *s) {
  return server_guard([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->stop = true;
      s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    for (auto &L : s->lanes) {
      cudaStreamSynchronize(L->stream);
      cudaStreamDestroy(L->stream);
      cudaFreeHost(L->h_status);
      s->pool.put(L->h_jobs);
      s->pool.put(L->h_items);
    }
    for (auto &kv : s->requests) s->pool.put(kv.second.payload);
    delete s;
  });
}

int fegpu_server_set_precision(fegpu_server *s, int precision) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    FEGPU_REQUIRE(precision == FEGPU_MIXED || precision == FEGPU_FP64 ||
                      precision == FEGPU_FP64_FAST,
                  "unknown precision");
    std::lock_guard<std::mutex> lock(s->mu);
    FEGPU_REQUIRE(s->meshes.empty(), "server: set the precision before adding meshes");
    s->precision = precision;
  });
}

int fegpu_server_set_slice(fegpu_server *s, int64_t elements) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && elements >= 1, "server: a slice holds at least one element");
    std::lock_guard<std::mutex> lock(s->mu);
    s->slice_elements = elements;
  });
}

int fegpu_server_set_memory_limit(fegpu_server *s, int64_t bytes) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && bytes >= 0, "server: the memory limit must be >= 0");
    std::lock_guard<std::mutex> lock(s->mu);
    s->mem_limit = bytes;
  });
}

int fegpu_server_add_mesh(fegpu_server *s, fegpu_matrix *K, int form, const fegpu_coef *cf,
                          int m, int64_t *mesh_id) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && K && cf && cf->data && mesh_id, "null handle");
    fegpu_femm *fm = K->dm->femm;
    FEGPU_REQUIRE(fm->ctx == s->ctx, "server: the matrix belongs to another context");
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    FEGPU_CUDA(cudaSetDevice(s->ctx->device));
    int f;
    if (form == FEGPU_FORM_DIFFUSION) {
      f = F_DIFF_ISO;
      FEGPU_REQUIRE(K->dm->ndn == 1 && fm->sdim == fm->mdim,
                    "server: diffusion needs one DOF per node and sdim == mdim");
    } else if (form == FEGPU_FORM_LIN_ELASTIC) {
      f = F_ELAST_ISO;
      FEGPU_REQUIRE(K->dm->ndn == 3 && fm->mdim == 3 && fm->sdim == 3,
                    "server: elasticity on 3-D solids with three DOFs per node");
    } else if (form == FEGPU_FORM_DOT) {
      f = F_DOT;
      if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
      else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    } else {
      throw Error{FEGPU_ERR_ARG, "server: unknown form"};
    }
    const int code = batch_code(fm->etype, f, K->dm->ndn);
    FEGPU_REQUIRE(code >= 0, "server: this element type, form and DOF count are not served");
    fegpu_dofmap *dm = K->dm;
    bool shared = false;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      for (auto &o : s->meshes) {
        if (o->removed) continue;
        FEGPU_REQUIRE(o->K != K, "server: the matrix is already served");
        if (o->K->dm == dm) shared = true;
      }
    }
    int64_t coef_values = 0;
    if (cf->kind == FEGPU_COEF_ISO_LAME) coef_values = 2 * fm->nelem;
    else if (cf->kind == FEGPU_COEF_PER_QP) coef_values = static_cast<int64_t>(fm->npts) * fm->nelem;
    else if (cf->kind == FEGPU_COEF_PER_ELEMENT) coef_values = fm->nelem;
    // admission: what serving adds must fit in the free memory (a 256 MB
    // reserve kept), and under a limit everything the meshes hold
    const int64_t need = serving_bytes(K, shared, coef_values);
    const int64_t held = resident_bytes(K) + need;
    {
      size_t freeb = 0, total = 0;
      FEGPU_CUDA(cudaMemGetInfo(&freeb, &total));
      std::lock_guard<std::mutex> lock(s->mu);
      const int64_t room = static_cast<int64_t>(freeb) - (256ll << 20);
      const bool over_limit = s->mem_limit > 0 && s->mem_held + held > s->mem_limit;
      if (need > room || over_limit) {
        throw Error{FEGPU_ERR_MEMORY,
                    "server: not enough device memory to admit the mesh: it holds " +
                        std::to_string((held + (1ll << 20) - 1) >> 20) + " MiB, " +
                        std::to_string(static_cast<long long>(freeb >> 20)) + " MiB free" +
                        (s->mem_limit > 0
                             ? ", limit " + std::to_string(s->mem_limit >> 20) + " MiB of which " +
                                   std::to_string(s->mem_held >> 20) + " MiB held"
                             : std::string())};
      }
      s->mem_held += held;  // reserved now, so concurrent admissions see it
    }
    try {
      auto M = std::make_unique<fegpu_server::Mesh>();
      M->K = K;
      M->form = f;
      M->code = code;
      M->m = m;
      M->bytes = held;
      const int nne = fm->nne, ndn = dm->ndn;
      const int64_t elem_floats = static_cast<int64_t>(nne) * (nne + 1) / 2 * ndn * ndn;
      if (!dm->gather_ready) build_gather_plan(dm, static_cast<int>(elem_floats));
      float *ring = nullptr;
      if (shared) {
        M->ring = std::make_unique<DevBuf>();
        M->ring->alloc(dm->ke.bytes);
        ring = M->ring->as<float>();
      }
      make_batch_job(K, f, code, m, cf, 0, M->coef, ring, s->ctx->stream, M->d);
      M->coef_values = M->d.k.coef ? coef_values : 0;
      // the coefficient on the host: the FP64 forms take it by value
      const int64_t nvals = cf->kind == FEGPU_COEF_CONST ? cf->ncomp : coef_values;
      M->cf_host.assign(cf->data, cf->data + nvals);
      M->cf = *cf;
      M->xyz_stage.alloc(sizeof(double) * fm->nnodes * fm->sdim);
      FEGPU_CUDA(cudaStreamSynchronize(s->ctx->stream));
      std::lock_guard<std::mutex> lock(s->mu);
      *mesh_id = static_cast<int64_t>(s->meshes.size());
      s->meshes.push_back(std::move(M));
    } catch (...) {
      std::lock_guard<std::mutex> lock(s->mu);
      s->mem_held -= held;
      throw;
    }
  });
}

int fegpu_server_remove_mesh(fegpu_server *s, int64_t mesh_id) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::lock_guard<std::mutex> lock(s->mu);
    FEGPU_REQUIRE(mesh_id >= 0 && mesh_id < static_cast<int64_t>(s->meshes.size()) &&
                      !s->meshes[mesh_id]->removed,
                  "server: no such mesh");
    auto &M = *s->meshes[mesh_id];
    FEGPU_REQUIRE(!M.busy, "server: the mesh has a request in flight");
    for (int64_t id : s->pending)
      FEGPU_REQUIRE(s->requests[id].mesh != mesh_id, "server: the mesh has requests waiting");
    M.removed = true;
    M.coef.reset();
    M.ring.reset();
    M.xyz_stage.release();
    s->mem_held -= M.bytes;
  });
}

int fegpu_server_submit(fegpu_server *s, int64_t mesh_id, int kind, const double *data,
                        int64_t count, int64_t *request_id) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && data && request_id, "null handle");
    fegpu_server::Mesh *M;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      FEGPU_REQUIRE(mesh_id >= 0 && mesh_id < static_cast<int64_t>(s->meshes.size()) &&
                        !s->meshes[mesh_id]->removed,
                    "server: no such mesh");
      M = s->meshes[mesh_id].get();
      FEGPU_REQUIRE(s->worker_error.empty(), "server: " + s->worker_error);
    }
    const fegpu_femm *fm = M->K->dm->femm;
    if (kind == FEGPU_REQUEST_COEF) {
      FEGPU_REQUIRE(M->coef_values > 0,
                    "server: this mesh was added with a constant coefficient");
      FEGPU_REQUIRE(count == M->coef_values, "Size mismatch");
    } else if (kind == FEGPU_REQUEST_COORDS) {
      FEGPU_REQUIRE(count == fm->nnodes * fm->sdim, "Size mismatch");
    } else {
      throw Error{FEGPU_ERR_ARG, "server: unknown request kind"};
    }
    fegpu_server::Request r;
    r.mesh = mesh_id;
    r.kind = kind;
    r.bytes = sizeof(double) * count;
    r.payload = s->pool.get(r.bytes);
    std::memcpy(PinnedPool::data(r.payload), data, r.bytes);
    r.t_submit = now_ms();
    std::lock_guard<std::mutex> lock(s->mu);
    const int64_t id = s->next_id++;
    s->requests.emplace(id, r);
    s->pending.push_back(id);
    *request_id = id;
    s->cv.notify_all();
  });
}

int fegpu_server_cancel(fegpu_server *s, int64_t request_id) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->requests.find(request_id);
    FEGPU_REQUIRE(it != s->requests.end(), "server: no such request (or already collected)");
    if (it->second.state != kReqPending)
      throw Error{FEGPU_ERR_STATE, "server: the request is already running or done"};
    s->pending.erase(std::find(s->pending.begin(), s->pending.end(), request_id));
    s->pool.put(it->second.payload);
    it->second.payload = nullptr;
    it->second.state = kReqCancelled;
    it->second.t_done = now_ms();
    s->cv.notify_all();
  });
}

int fegpu_server_wait(fegpu_server *s, int64_t request_id, double *latency_ms) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request_id);
    FEGPU_REQUIRE(it != s->requests.end(), "server: no such request (or already collected)");
    s->cv.wait(lock, [&] { return it->second.state >= kReqDone; });
    const auto r = it->second;
    s->pool.put(r.payload);
    s->requests.erase(it);
    if (latency_ms) *latency_ms = r.t_done - r.t_submit;
    if (r.state == kReqCancelled)
      throw Error{FEGPU_ERR_STATE, "server: the request was cancelled"};
    if (r.state == kReqFailed)
      throw Error{FEGPU_ERR_DEVICE,
                  s->worker_error.empty()
                      ? "server: a work item of the request's launch waited past its time limit"
                      : "server: " + s->worker_error};
  });
}

int fegpu_server_hold(fegpu_server *s, int hold) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::lock_guard<std::mutex> lock(s->mu);
    s->hold = hold != 0;
    s->cv.notify_all();
  });
}

int fegpu_server_drain(fegpu_server *s) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::unique_lock<std::mutex> lock(s->mu);
    FEGPU_REQUIRE(!s->hold || (s->pending.empty() && s->active.empty()),
                  "server: drain while launches are held");
    s->cv.wait(lock, [&] {
      if (!s->pending.empty() || !s->active.empty()) return false;
      for (auto &L : s->lanes)
        if (L->busy) return false;
      for (auto &kv : s->requests)
        if (kv.second.state == kReqRunning) return false;
      return true;
    });
  });
}

int fegpu_server_stats(fegpu_server *s, int64_t *batches, int64_t *jobs, int64_t *pending) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::lock_guard<std::mutex> lock(s->mu);
    if (batches) *batches = s->batches;
    if (jobs) *jobs = s->jobs_run;
    if (pending) *pending = static_cast<int64_t>(s->pending.size());
  });
}

int fegpu_server_memory(fegpu_server *s, int64_t *free_bytes, int64_t *total_bytes) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    FEGPU_CUDA(cudaSetDevice(s->ctx->device));
    size_t f = 0, t = 0;
    FEGPU_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = static_cast<int64_t>(f);
    if (total_bytes) *total_bytes = static_cast<int64_t>(t);
  });
}

int fegpu_estimate_mesh_bytes(int etype, int64_t nelem, int64_t nnodes, int ndn,
                              int64_t *bytes) {
  return server_guard([&] {
    FEGPU_REQUIRE(bytes, "null handle");
    const int nne = nodes_per_elem(etype);
    FEGPU_REQUIRE(nne > 0 && nelem >= 0 && nnodes >= 0 && ndn >= 1 && ndn <= 3,
                  "estimate: bad element type or sizes");
    // average node degree (neighbours, the node itself included) of block
    // meshes of each type, rounded up: H8 24.5, H20 56.2, T10 28.3 measured
    int deg = 0;
    switch (etype) {
      case FEGPU_Q4: deg = 9; break;
      case FEGPU_H8: deg = 27; break;
      case FEGPU_H20: deg = 60; break;
      case FEGPU_T4: deg = 20; break;
      case FEGPU_T10: deg = 32; break;
    }
    const int64_t nnz = static_cast<int64_t>(ndn) * ndn * nnodes * deg;
    const int64_t E = nelem, N = nnodes;
    const int64_t block_floats = static_cast<int64_t>(nne) * (nne + 1) / 2 * ndn * ndn;
    const int64_t chunk = std::min<int64_t>(std::max<int64_t>(1024, (24ll << 20) / (block_floats * 4)),
                                            std::max<int64_t>(E, 1));
    const int64_t resident = 2 * E * nne * 4 + E * 4 + N * 32 + (N * ndn + 1) * 8 + nnz * 4 +
                             E * nne * nne * 2 + N * ndn * 4 + (N + 1) * 8 + nnz * 8;
    const int64_t serving = (N + 1) * 8 + E * nne * 9 + N * 4 + E * nne * nne * 2 +
                            4 * chunk * block_floats * 4 + 2 * E * 8 + N * 3 * 8;
    *bytes = resident + serving;
  });
}

int fegpu_server_mesh_bytes(fegpu_server *s, int64_t mesh_id, int64_t *bytes) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && bytes, "null handle");
    std::lock_guard<std::mutex> lock(s->mu);
    if (mesh_id < 0) {
      *bytes = s->mem_held;
      return;
    }
    FEGPU_REQUIRE(mesh_id < static_cast<int64_t>(s->meshes.size()) &&
                      !s->meshes[mesh_id]->removed,
                  "server: no such mesh");
    *bytes = s->meshes[mesh_id]->bytes;
  });
}

}  // extern "C"
