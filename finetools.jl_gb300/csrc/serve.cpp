// Serving loop: re-assembly requests on resident meshes, continuously batched.
//
// A server keeps meshes resident on the device (connectivity, colouring, CSR
// pattern, gather plan, block ring, coefficient buffer, matrix values) and
// accepts requests that carry new per-element coefficients or new node
// coordinates for one of them.  A worker thread forms batches from the
// pending requests -- the oldest request of every mesh that is not already on
// the GPU, up to a job limit -- and runs each batch as one launch of the
// persistent assembly kernel (batch.cu) on one of several lanes (CUDA
// streams).  Each lane's grid covers 1/lanes of the GPU, so a batch formed
// while others run starts at once and its work overlaps theirs; requests that
// arrive meanwhile wait only until a lane frees up (continuous batching, not a
// queue drained one batch at a time).  Requests on the same mesh run in
// arrival order (a mesh is in at most one batch at a time); the result of a
// request is the mesh's matrix as it stands when the request completes.
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

}  // namespace

struct fegpu_server {
  fegpu_context *ctx = nullptr;
  int nlanes = 1;
  int max_jobs = 64;
  double wait_s = 5.0;

  struct Mesh {
    fegpu_matrix *K = nullptr;
    int form = 0, code = 0, m = 3;
    BatchJob d{};
    std::unique_ptr<DevBuf> coef;     // coefficient values read by the kernel
    std::unique_ptr<DevBuf> ring;     // private ring when the dofmap is shared
    DevBuf xyz_stage;                 // column-major coordinates of an update
    int64_t coef_values = 0;          // doubles per coefficient update (0: constant)
    bool busy = false;                // in a batch on the GPU
  };
  std::vector<std::unique_ptr<Mesh>> meshes;

  struct Request {
    int64_t mesh = 0;
    int kind = 0;
    void *payload = nullptr;          // pinned block
    size_t bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int state = 0;                    // 0 pending, 1 running, 2 done, 3 failed
  };
  std::unordered_map<int64_t, Request> requests;
  std::deque<int64_t> pending;
  int64_t next_id = 0;

  struct Lane {
    cudaStream_t stream = nullptr;
    DevBuf d_jobs, d_items, d_counters, d_next, d_status;
    void *h_jobs = nullptr, *h_items = nullptr;  // pinned staging (pool blocks)
    int *h_status = nullptr;
    std::vector<int64_t> reqs;
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

void lane_done(void *arg) {  // CUDA host callback: no CUDA calls here
  auto *lane = static_cast<fegpu_server::Lane *>(arg);
  fegpu_server *s = lane->srv;
  const double t = now_ms();
  std::lock_guard<std::mutex> lock(s->mu);
  const bool ok = *lane->h_status == 0;
  for (int64_t id : lane->reqs) {
    auto &r = s->requests[id];
    r.t_done = t;
    r.state = ok ? 2 : 3;
    s->meshes[r.mesh]->busy = false;
  }
  lane->reqs.clear();
  lane->busy = false;
  s->cv.notify_all();
}

// Lane buffers grow by half again when they must grow, so that steady traffic
// stops reallocating (cudaFree can stall behind the other lanes' work).
void grow(DevBuf &b, size_t n) {
  if (n > b.bytes) b.alloc(std::max(n, b.bytes + b.bytes / 2));
}

// Stage one batch on a free lane and launch it (worker thread, no lock held).
void launch_lane(fegpu_server *s, fegpu_server::Lane &L, const std::vector<int64_t> &ids) {
  cudaStream_t st = L.stream;
  std::vector<BatchJob> jobs;
  std::vector<const fegpu_dofmap *> dms;
  for (int64_t id : ids) {
    fegpu_server::Request *r;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      r = &s->requests[id];
      r->t_start = now_ms();
    }
    fegpu_server::Mesh &M = *s->meshes[r->mesh];
    fegpu_femm *fm = M.K->dm->femm;
    if (r->kind == FEGPU_REQUEST_COEF) {
      FEGPU_CUDA(cudaMemcpyAsync(M.coef->p, PinnedPool::data(r->payload), r->bytes,
                                 cudaMemcpyHostToDevice, st));
    } else {
      FEGPU_CUDA(cudaMemcpyAsync(M.xyz_stage.p, PinnedPool::data(r->payload), r->bytes,
                                 cudaMemcpyHostToDevice, st));
      pack_geometry(M.xyz_stage.as<double>(), fm->nnodes, fm->sdim, fm->xyz.as<double>(), st);
    }
    jobs.push_back(M.d);
    dms.push_back(M.K->dm);
  }
  std::vector<BatchItem> items;
  const int ncount = build_batch_items(jobs, dms, 64u << 20, items);
  const size_t smem = batch_smem_bytes(jobs, dms);
  const int nitems = static_cast<int>(items.size());
  const int grid = batch_grid(s->ctx->num_sms, smem, nitems, 1.0 / s->nlanes);
  // staging: the lane's pinned blocks are free (the lane's previous batch is done)
  const size_t jb = sizeof(BatchJob) * jobs.size(), ib = sizeof(BatchItem) * items.size();
  s->pool.put(L.h_jobs);
  s->pool.put(L.h_items);
  L.h_jobs = s->pool.get(jb);
  L.h_items = s->pool.get(ib);
  std::memcpy(PinnedPool::data(L.h_jobs), jobs.data(), jb);
  std::memcpy(PinnedPool::data(L.h_items), items.data(), ib);
  grow(L.d_jobs, jb);
  grow(L.d_items, ib);
  grow(L.d_counters, sizeof(int) * ncount);
  FEGPU_CUDA(cudaMemcpyAsync(L.d_jobs.p, PinnedPool::data(L.h_jobs), jb, cudaMemcpyHostToDevice, st));
  FEGPU_CUDA(cudaMemcpyAsync(L.d_items.p, PinnedPool::data(L.h_items), ib, cudaMemcpyHostToDevice, st));
  FEGPU_CUDA(cudaMemsetAsync(L.d_counters.p, 0, sizeof(int) * ncount, st));
  FEGPU_CUDA(cudaMemsetAsync(L.d_next.p, 0, sizeof(int), st));
  FEGPU_CUDA(cudaMemsetAsync(L.d_status.p, 0, sizeof(int), st));
  launch_batch_kernel(grid, smem, st, L.d_jobs.as<BatchJob>(), L.d_items.as<BatchItem>(), nitems,
                      L.d_next.as<int>(), L.d_counters.as<int>(), L.d_status.as<int>(), s->wait_s);
  FEGPU_CUDA(cudaMemcpyAsync(L.h_status, L.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FEGPU_CUDA(cudaLaunchHostFunc(st, lane_done, &L));
}

void worker_main(fegpu_server *s) {
  cudaSetDevice(s->ctx->device);
  for (;;) {
    fegpu_server::Lane *lane = nullptr;
    std::vector<int64_t> ids;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv.wait(lock, [&] {
        if (s->stop) return true;
        if (s->hold || s->pending.empty()) return false;
        for (auto &L : s->lanes)
          if (!L->busy) return true;
        return false;
      });
      if (s->stop) return;
      for (auto &L : s->lanes)
        if (!L->busy) {
          lane = L.get();
          break;
        }
      // the oldest pending request of each mesh not on the GPU, in arrival order
      std::vector<int64_t> rest;
      std::vector<char> taken(s->meshes.size(), 0);
      for (int64_t id : s->pending) {
        auto &r = s->requests[id];
        if (static_cast<int>(ids.size()) < s->max_jobs && !s->meshes[r.mesh]->busy &&
            !taken[r.mesh]) {
          taken[r.mesh] = 1;
          ids.push_back(id);
          r.state = 1;
        } else {
          rest.push_back(id);
        }
      }
      if (ids.empty()) {
        // every pending request waits for its mesh: sleep until a lane completes
        s->cv.wait(lock);
        continue;
      }
      s->pending.assign(rest.begin(), rest.end());
      for (int64_t id : ids) s->meshes[s->requests[id].mesh]->busy = true;
      lane->busy = true;
      lane->reqs = ids;
    }
    try {
      launch_lane(s, *lane, ids);
      std::lock_guard<std::mutex> lock(s->mu);
      s->batches++;
      s->jobs_run += static_cast<int64_t>(ids.size());
    } catch (const Error &e) {
      std::lock_guard<std::mutex> lock(s->mu);
      s->worker_error = e.msg;
      for (int64_t id : ids) {
        auto &r = s->requests[id];
        r.state = 3;
        r.t_done = now_ms();
        s->meshes[r.mesh]->busy = false;
      }
      lane->reqs.clear();
      lane->busy = false;
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
    for (int i = 0; i < lanes; ++i) {
      auto L = std::make_unique<fegpu_server::Lane>();
      L->srv = s.get();
      FEGPU_CUDA(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
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
    auto M = std::make_unique<fegpu_server::Mesh>();
    M->K = K;
    M->form = f;
    M->code = code;
    M->m = m;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      for (auto &o : s->meshes) FEGPU_REQUIRE(o->K != K, "server: the matrix is already served");
    }
    fegpu_dofmap *dm = K->dm;
    const int nne = fm->nne, ndn = dm->ndn;
    const int64_t elem_floats = static_cast<int64_t>(nne) * (nne + 1) / 2 * ndn * ndn;
    if (!dm->gather_ready) build_gather_plan(dm, static_cast<int>(elem_floats));
    float *ring = nullptr;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      for (auto &o : s->meshes)
        if (o->K->dm == dm) {
          M->ring = std::make_unique<DevBuf>();
          M->ring->alloc(dm->ke.bytes);
          ring = M->ring->as<float>();
          break;
        }
    }
    make_batch_job(K, f, code, m, cf, 0, M->coef, ring, s->ctx->stream, M->d);
    if (M->d.k.coef) {
      int64_t width = cf->kind == FEGPU_COEF_ISO_LAME ? 2
                      : cf->kind == FEGPU_COEF_PER_QP ? fm->npts : 1;
      M->coef_values = width * fm->nelem;
    }
    M->xyz_stage.alloc(sizeof(double) * fm->nnodes * fm->sdim);
    FEGPU_CUDA(cudaStreamSynchronize(s->ctx->stream));
    std::lock_guard<std::mutex> lock(s->mu);
    *mesh_id = static_cast<int64_t>(s->meshes.size());
    s->meshes.push_back(std::move(M));
  });
}

int fegpu_server_submit(fegpu_server *s, int64_t mesh_id, int kind, const double *data,
                        int64_t count, int64_t *request_id) {
  return server_guard([&] {
    FEGPU_REQUIRE(s && data && request_id, "null handle");
    fegpu_server::Mesh *M;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      FEGPU_REQUIRE(mesh_id >= 0 && mesh_id < static_cast<int64_t>(s->meshes.size()),
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

int fegpu_server_wait(fegpu_server *s, int64_t request_id, double *latency_ms) {
  return server_guard([&] {
    FEGPU_REQUIRE(s, "null handle");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request_id);
    FEGPU_REQUIRE(it != s->requests.end(), "server: no such request (or already collected)");
    s->cv.wait(lock, [&] { return it->second.state >= 2; });
    const auto r = it->second;
    s->pool.put(r.payload);
    s->requests.erase(it);
    if (latency_ms) *latency_ms = r.t_done - r.t_submit;
    if (r.state == 3)
      throw Error{FEGPU_ERR_DEVICE,
                  s->worker_error.empty()
                      ? "server: a work item of the request's batch waited past its time limit"
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
    FEGPU_REQUIRE(!s->hold || s->pending.empty(), "server: drain while launches are held");
    s->cv.wait(lock, [&] {
      if (!s->pending.empty()) return false;
      for (auto &L : s->lanes)
        if (L->busy) return false;
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

}  // extern "C"
