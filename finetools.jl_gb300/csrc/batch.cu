// Many assemblies in one persistent launch (mixed element types and sizes).
//
// A batch holds jobs: (matrix, form, coefficient) triples whose matrices can
// belong to different meshes and element types.  Each job is the
// mixed-precision pipeline of the single-matrix path (FP32 element blocks into
// a ring, then the row gather) cut into stages: stage 2c = the element blocks
// of chunk c (items of one tile of elements each), stage 2c+1 = the row gather
// of the nodes whose last element lies in chunk c (items of a range of
// nodes).  The work queue interleaves the jobs stage by stage; one persistent
// kernel pulls items in queue order with an atomic counter, and an item of
// stage s first waits until every item of stage s-1 of its own job has
// completed (per-stage completion counters; release and acquire through
// __threadfence as in a grid-wide barrier).  Every dependency of an item sits
// earlier in the queue and has therefore been taken by a CTA that is running,
// so the waits end.  They are bounded all the same: a wait that exceeds its
// time budget sets the batch status word, every later item is skipped, and
// the host gets an error instead of a hang.
//
// Each CSR value is summed over its elements in element order whatever the
// schedule, so a job's matrix is the same alone, in any batch, and as the
// single-matrix FEGPU_MIXED result.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "batch_host.h"
#include "gather.cuh"
#include "mixed_fast.cuh"

namespace fegpu {

namespace {

static_assert(kBatchThreads == kMixedThreads, "element tiles fill the CTA");
static_assert(kBatchThreads == 32 * kGatherWarps, "gather warps fill the CTA");

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <int NNE, int NDN>
__device__ void batch_gather(const GArgs &g, int64_t b, int64_t e, unsigned char *smem) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wstride = gather_warp_stride(NDN, g.maxdeg);
  float *acc = reinterpret_cast<float *>(smem) + static_cast<size_t>(warp) * wstride;
  for (int64_t t = b + warp; t < e; t += kGatherWarps)
    gather_node<NNE, NDN, false, true>(g, g.nodes[t], acc, lane);
}

__device__ void elem_dispatch(const BatchJob &J, int64_t b, int64_t e, int64_t chunk,
                              unsigned char *smem) {
  const KArgs &a = J.k;
  // the gather reads the ring through a const pointer; this stage writes it
  float *ke = const_cast<float *>(J.g.ke) + (chunk % J.g.ring) * J.g.chunk * J.elem_floats;
  const int64_t e0 = chunk * J.g.chunk;
  const int ne = static_cast<int>(e - b);
  switch (J.code) {
    case BC_H8_DIFF: mixed_tile_fast<FEGPU_H8, F_DIFF_ISO, 1>(a, b, ne, smem, ke, e0); break;
    case BC_H20_DIFF: mixed_tile_fast<FEGPU_H20, F_DIFF_ISO, 1>(a, b, ne, smem, ke, e0); break;
    case BC_T4_DIFF: mixed_tile_fast<FEGPU_T4, F_DIFF_ISO, 1>(a, b, ne, smem, ke, e0); break;
    case BC_T10_DIFF: mixed_tile_fast<FEGPU_T10, F_DIFF_ISO, 1>(a, b, ne, smem, ke, e0); break;
    case BC_Q4_DIFF: mixed_tile_fast<FEGPU_Q4, F_DIFF_ISO, 1>(a, b, ne, smem, ke, e0); break;
    case BC_H8_ELAST: mixed_tile_fast<FEGPU_H8, F_ELAST_ISO, 3>(a, b, ne, smem, ke, e0); break;
    case BC_H20_ELAST: mixed_tile_fast<FEGPU_H20, F_ELAST_ISO, 3>(a, b, ne, smem, ke, e0); break;
    case BC_T4_ELAST: mixed_tile_fast<FEGPU_T4, F_ELAST_ISO, 3>(a, b, ne, smem, ke, e0); break;
    case BC_T10_ELAST: mixed_tile_fast<FEGPU_T10, F_ELAST_ISO, 3>(a, b, ne, smem, ke, e0); break;
    case BC_Q4_DOT1: mixed_tile_fast<FEGPU_Q4, F_DOT, 1>(a, b, ne, smem, ke, e0); break;
    case BC_Q4_DOT3: mixed_tile_fast<FEGPU_Q4, F_DOT, 3>(a, b, ne, smem, ke, e0); break;
    case BC_H8_DOT1: mixed_tile_fast<FEGPU_H8, F_DOT, 1>(a, b, ne, smem, ke, e0); break;
    case BC_H8_DOT3: mixed_tile_fast<FEGPU_H8, F_DOT, 3>(a, b, ne, smem, ke, e0); break;
    default: break;
  }
}

__device__ void gather_dispatch(const BatchJob &J, int64_t b, int64_t e, unsigned char *smem) {
  const bool three = J.ndn == 3;
  switch (J.etype) {
    case FEGPU_H8:
      three ? batch_gather<8, 3>(J.g, b, e, smem) : batch_gather<8, 1>(J.g, b, e, smem);
      break;
    case FEGPU_H20:
      three ? batch_gather<20, 3>(J.g, b, e, smem) : batch_gather<20, 1>(J.g, b, e, smem);
      break;
    case FEGPU_T4:
    case FEGPU_Q4:
      three ? batch_gather<4, 3>(J.g, b, e, smem) : batch_gather<4, 1>(J.g, b, e, smem);
      break;
    case FEGPU_T10:
      three ? batch_gather<10, 3>(J.g, b, e, smem) : batch_gather<10, 1>(J.g, b, e, smem);
      break;
    default: break;
  }
}

// The persistent kernel.  status: 0 ok, 1 a wait ran out of time.  withheld
// (>= 0): the completions of that counter are not published, so the items that
// wait on it run out of time (the failure path, exercised by a test).
__global__ void __launch_bounds__(kBatchThreads, 2) k_batch(const BatchJob *jobs,
                                                         const BatchItem *items, int nitems,
                                                         int *next, int *counters, int *status,
                                                         unsigned long long wait_ns,
                                                         int withheld) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item, s_go;
  for (;;) {
    __syncthreads();  // the previous item is done with shared memory
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) return;
    const BatchItem I = items[it];
    if (threadIdx.x == 0) {
      int go = *reinterpret_cast<volatile int *>(status) == 0;
      for (int d = 0; d < 2 && go; ++d) {
        if (I.dep[d] < 0) continue;
        const volatile int *ctr = counters + I.dep[d];
        const int target = I.target[d];
        if (*ctr < target) {
          const unsigned long long t0 = global_ns();
          long long spins = 0;
          while (*ctr < target) {
            __nanosleep(128);
            if ((++spins & 255) != 0) continue;
            if (*reinterpret_cast<volatile int *>(status) != 0) {  // another wait gave up
              go = 0;
              break;
            }
            // time budget, and an iteration cap in case the timer stalls
            if (global_ns() - t0 > wait_ns || spins > (1ll << 26)) {
              atomicExch(status, 1);
              go = 0;
              break;
            }
          }
        }
      }
      __threadfence();  // acquire: the producers' writes are visible
      s_go = go;
    }
    __syncthreads();
    if (s_go) {  // CTA-uniform
      const BatchJob &J = jobs[I.job];
      if (I.kind == 0) elem_dispatch(J, I.b, I.e, I.chunk, smem);
      else gather_dispatch(J, I.b, I.e, smem);
    }
    __syncthreads();
    if (threadIdx.x == 0 && I.done != withheld) {
      __threadfence();  // release this item's writes
      atomicAdd(&counters[I.done], 1);
    }
  }
}

}  // namespace

int batch_code(int etype, int form, int ndn) {
  if (form == F_DIFF_ISO && ndn == 1) {
    switch (etype) {
      case FEGPU_H8: return BC_H8_DIFF;
      case FEGPU_H20: return BC_H20_DIFF;
      case FEGPU_T4: return BC_T4_DIFF;
      case FEGPU_T10: return BC_T10_DIFF;
      case FEGPU_Q4: return BC_Q4_DIFF;
    }
  } else if (form == F_ELAST_ISO && ndn == 3) {
    switch (etype) {
      case FEGPU_H8: return BC_H8_ELAST;
      case FEGPU_H20: return BC_H20_ELAST;
      case FEGPU_T4: return BC_T4_ELAST;
      case FEGPU_T10: return BC_T10_ELAST;
    }
  } else if (form == F_DOT) {
    if (etype == FEGPU_Q4) return ndn == 1 ? BC_Q4_DOT1 : (ndn == 3 ? BC_Q4_DOT3 : -1);
    if (etype == FEGPU_H8) return ndn == 1 ? BC_H8_DOT1 : (ndn == 3 ? BC_H8_DOT3 : -1);
  }
  return -1;
}

static const char *const kCodeNames[BC_COUNT] = {
    "H8_diffusion",  "H20_diffusion", "T4_diffusion", "T10_diffusion", "Q4_diffusion",
    "H8_elasticity", "H20_elasticity", "T4_elasticity", "T10_elasticity",
    "Q4_dot1",       "Q4_dot3",        "H8_dot1",      "H8_dot3"};

const char *batch_code_name(int code) {
  return code >= 0 && code < BC_COUNT ? kCodeNames[code] : "unknown";
}

void launch_batch_kernel(int grid, size_t smem, cudaStream_t s, const BatchJob *jobs,
                         const BatchItem *items, int nitems, int *next, int *counters,
                         int *status, double wait_s, int withheld) {
  k_batch<<<grid, kBatchThreads, smem, s>>>(jobs, items, nitems, next, counters, status,
                                            static_cast<unsigned long long>(wait_s * 1e9),
                                            withheld);
  FEGPU_CUDA(cudaGetLastError());
}

int batch_grid(int num_sms, size_t smem, int nitems, double share) {
  // always the same (maximal) limit, so threads launching concurrently with
  // different needs cannot undercut each other's launches
  FEGPU_REQUIRE(smem <= kBatchMaxSmem, "batch: shared-memory need too large");
  FEGPU_CUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(kBatchMaxSmem)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kBatchThreads, smem));
  per_sm = std::max(per_sm, 1);
  const int full = num_sms * per_sm;
  const int g = static_cast<int>(full * std::min(1.0, std::max(share, 0.0)));
  return std::max(1, std::min(nitems, std::max(g, 1)));
}

size_t batch_smem_bytes(const std::vector<BatchJob> &jobs,
                        const std::vector<const fegpu_dofmap *> &dms) {
  size_t smem = 0;
  for (size_t j = 0; j < jobs.size(); ++j) {
    const fegpu_femm *fm = dms[j]->femm;
    smem = std::max(smem, tile_smem_bytes(fm->etype, jobs[j].form, fm->npts, jobs[j].k.te));
    smem = std::max(smem, sizeof(float) * gather_warp_stride(jobs[j].ndn, jobs[j].g.maxdeg) *
                              kGatherWarps);
  }
  FEGPU_REQUIRE(smem <= kBatchMaxSmem, "batch: shared-memory need above the per-CTA limit");
  return smem;
}

}  // namespace fegpu

using namespace fegpu;

struct fegpu_batch {
  fegpu_context *ctx = nullptr;
  struct Job {
    fegpu_matrix *K = nullptr;
    int form = 0, code = 0, m = 3;
    BatchJob d{};
    std::unique_ptr<DevBuf> coef;     // per-element / per-point coefficients
    std::unique_ptr<DevBuf> ring;     // private block ring (dofmap shared with another job)
  };
  std::vector<Job> jobs;
  std::map<int, int> tile;            // elements per tile by job kind (tuned or cached)
  DevBuf d_jobs, d_items, d_counters, d_next, d_status;
  int nitems = 0, ncounters = 0, grid = 0;
  size_t smem = 0;
  double wait_s = 5.0;                // time budget of one dependency wait
  int withheld = -1;                  // counter whose completions are withheld (test hook)
  bool dirty = true;                  // queue and graph must be rebuilt
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~fegpu_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

namespace fegpu {

// ---- job descriptors ----------------------------------------------------------
void make_batch_job(fegpu_matrix *K, int form, int code, int m, const fegpu_coef *cf, int te,
                    std::unique_ptr<DevBuf> &coef, float *ring, cudaStream_t s, BatchJob &out) {
  fegpu_dofmap *dm = K->dm;
  fegpu_femm *fm = dm->femm;
  const int nne = fm->nne, ndn = dm->ndn;
  const int64_t elem_floats = static_cast<int64_t>(nne) * (nne + 1) / 2 * ndn * ndn;
  if (!dm->gather_ready) build_gather_plan(dm, static_cast<int>(elem_floats));
  K->unsym = false;
  KArgs a = base_args(K, dm);
  a.conn = fm->conn_orig.as<int32_t>();
  a.measure_m = m;
  a.coef_kind = cf->kind;
  a.ncomp = cf->ncomp;
  int64_t width = 0;  // coefficient values per element
  if (form == F_ELAST_ISO) {
    if (cf->kind == FEGPU_COEF_CONST) {
      double lam, mu;
      FEGPU_REQUIRE(cf->ncomp == 36 && is_isotropic(cf->data, lam, mu),
                    "batch: elasticity needs an isotropic D or per-element (lambda, mu)");
      a.cconst[0] = lam;
      a.cconst[1] = mu;
    } else {
      FEGPU_REQUIRE(cf->kind == FEGPU_COEF_ISO_LAME && cf->ncomp == 2,
                    "batch: elasticity needs an isotropic D or per-element (lambda, mu)");
      width = 2;
    }
  } else {
    FEGPU_REQUIRE(cf->kind == FEGPU_COEF_CONST || cf->kind == FEGPU_COEF_PER_ELEMENT ||
                      cf->kind == FEGPU_COEF_PER_QP,
                  "batch: bad coefficient kind");
    const bool matrix_coef = form == F_DOT && ndn > 1 && cf->ncomp == ndn * ndn;
    FEGPU_REQUIRE(cf->ncomp == 1 || (matrix_coef && cf->kind == FEGPU_COEF_CONST),
                  "batch: scalar coefficients (or a constant ndn x ndn matrix for dot)");
    if (cf->kind == FEGPU_COEF_CONST) a.cconst[0] = cf->data[0];
    if (cf->kind == FEGPU_COEF_PER_ELEMENT) width = 1;
    if (cf->kind == FEGPU_COEF_PER_QP) width = fm->npts;
    if (form == F_DOT) {
      // element-matrix entry (k,p),(l,q) = N_k N_l c[p][q] (src/FEMMBaseModule.jl:1357-1361),
      // arranged as the symmetric assembler keeps it (lower triangle, mirrored)
      double c[9] = {0};
      if (matrix_coef) {
        for (int i = 0; i < ndn * ndn; ++i) c[i] = cf->data[i];
        a.coef_kind = kCoefNone;
      } else {
        for (int i = 0; i < ndn; ++i) c[i * ndn + i] = 1.0;
      }
      for (int i = 0; i < ndn; ++i)
        for (int j = 0; j < ndn; ++j) {
          a.cab[i * ndn + j] = c[j * ndn + i];
          a.cdiag[i * ndn + j] = c[std::max(i, j) * ndn + std::min(i, j)];
        }
    }
  }
  if (width > 0) {
    const int64_t n = width * fm->nelem;
    if (!coef) coef = std::make_unique<DevBuf>();
    coef->alloc(sizeof(double) * std::max<int64_t>(n, 1));
    if (n > 0 && cf->data)
      FEGPU_CUDA(cudaMemcpyAsync(coef->p, cf->data, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    a.coef = coef->as<double>();
  } else {
    a.coef = nullptr;
  }
  a.te = te > 0 ? std::min(te, max_fast_tile(fm->etype)) : mixed_tile_for(fm->etype, form, fm->npts);
  a.ke = nullptr;
  out.k = a;
  GArgs &g = out.g;
  std::memset(&g, 0, sizeof(g));
  g.n2e_ptr = dm->n2e_ptr.as<int64_t>();
  g.n2e_elem = dm->n2e_elem.as<int32_t>();
  g.n2e_loc = dm->n2e_loc.as<uint8_t>();
  g.n2e_slot = dm->n2e_slot.as<int32_t>();
  g.nodes = dm->gnodes.as<int32_t>();
  g.nptr = dm->nptr.as<int64_t>();
  g.pos = dm->pos_orig.as<uint16_t>();
  g.ke = ring ? ring : dm->ke.as<float>();
  g.chunk = dm->chunk;
  g.ring = dm->ring;
  g.dof = dm->dof.as<int32_t>();
  g.rowptr = dm->rowptr.as<int64_t>();
  g.colperm = dm->contiguous ? nullptr : dm->colperm.as<int32_t>();
  g.cpoff = dm->contiguous ? nullptr : dm->cpoff.as<int64_t>();
  g.val = K->val.as<double>();
  g.maxdeg = dm->maxdeg;
  g.check = out.k.check;
  g.nnz = dm->nnz;
  out.code = code;
  out.form = form;
  out.etype = fm->etype;
  out.ndn = ndn;
  out.elem_floats = elem_floats;
}

namespace {

void drop_graph(fegpu_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// (Re)build a job's descriptor: coefficient copy and private ring as needed.
void fill_job(fegpu_batch *b, size_t index, const fegpu_coef *cf) {
  fegpu_batch::Job &J = b->jobs[index];
  fegpu_dofmap *dm = J.K->dm;
  const int nne = dm->femm->nne, ndn = dm->ndn;
  const int64_t elem_floats = static_cast<int64_t>(nne) * (nne + 1) / 2 * ndn * ndn;
  if (!dm->gather_ready) build_gather_plan(dm, static_cast<int>(elem_floats));
  float *ring = nullptr;
  for (size_t j = 0; j < index; ++j)
    if (b->jobs[j].K->dm == dm) {  // the dofmap's ring is taken: use a private one
      if (!J.ring) J.ring = std::make_unique<DevBuf>();
      J.ring->alloc(dm->ke.bytes);
      ring = J.ring->as<float>();
      break;
    }
  const int te = b->tile.count(J.code) ? b->tile[J.code] : 0;
  make_batch_job(J.K, J.form, J.code, J.m, cf, te, J.coef, ring, b->ctx->stream, J.d);
}

void build_queue(fegpu_batch *b) {
  std::vector<BatchJob> dj;
  std::vector<const fegpu_dofmap *> dms;
  for (auto &J : b->jobs) {
    dj.push_back(J.d);
    dms.push_back(J.K->dm);
  }
  std::vector<BatchItem> items;
  const int ncount = build_batch_items(dj, dms, 64u << 20, items);
  b->smem = batch_smem_bytes(dj, dms);
  cudaStream_t st = b->ctx->stream;
  b->nitems = static_cast<int>(items.size());
  b->ncounters = ncount;
  b->d_items.alloc(sizeof(BatchItem) * std::max<size_t>(items.size(), 1));
  if (!items.empty())
    FEGPU_CUDA(cudaMemcpyAsync(b->d_items.p, items.data(), sizeof(BatchItem) * items.size(),
                               cudaMemcpyHostToDevice, st));
  b->d_jobs.alloc(sizeof(BatchJob) * std::max<size_t>(dj.size(), 1));
  if (!dj.empty())
    FEGPU_CUDA(cudaMemcpyAsync(b->d_jobs.p, dj.data(), sizeof(BatchJob) * dj.size(),
                               cudaMemcpyHostToDevice, st));
  b->d_counters.alloc(sizeof(int) * b->ncounters);
  b->d_next.alloc(sizeof(int));
  b->d_status.alloc(sizeof(int));
  b->grid = batch_grid(b->ctx->num_sms, b->smem, b->nitems, 1.0);
  FEGPU_CUDA(cudaStreamSynchronize(st));
  b->dirty = false;
}

// Stream work of one run: counter resets and the persistent launch.
void enqueue_batch(fegpu_batch *b, cudaStream_t st) {
  FEGPU_CUDA(cudaMemsetAsync(b->d_counters.p, 0, sizeof(int) * b->ncounters, st));
  FEGPU_CUDA(cudaMemsetAsync(b->d_next.p, 0, sizeof(int), st));
  FEGPU_CUDA(cudaMemsetAsync(b->d_status.p, 0, sizeof(int), st));
  launch_batch_kernel(b->grid, b->smem, st, b->d_jobs.as<BatchJob>(), b->d_items.as<BatchItem>(),
                      b->nitems, b->d_next.as<int>(), b->d_counters.as<int>(),
                      b->d_status.as<int>(), b->wait_s, b->withheld);
}

void check_status(fegpu_batch *b) {
  int status = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&status, b->d_status.p, sizeof(int), cudaMemcpyDeviceToHost,
                             b->ctx->stream));
  FEGPU_CUDA(cudaStreamSynchronize(b->ctx->stream));
  if (status != 0)
    throw Error{FEGPU_ERR_DEVICE,
                "batch: a work item waited past its time limit for its dependency; "
                "the matrices of this run are incomplete"};
}

template <typename F>
int batch_guard(F &&f) {
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

fegpu_batch::Job &job_at(fegpu_batch *b, int64_t job) {
  FEGPU_REQUIRE(job >= 0 && job < static_cast<int64_t>(b->jobs.size()), "batch: no such job");
  return b->jobs[static_cast<size_t>(job)];
}

}  // namespace
}  // namespace fegpu

extern "C" {

int fegpu_batch_create(fegpu_context *ctx, fegpu_batch **out) {
  return batch_guard([&] {
    FEGPU_REQUIRE(ctx && out, "null handle");
    auto *b = new fegpu_batch();
    b->ctx = ctx;
    *out = b;
  });
}

int fegpu_batch_destroy(fegpu_batch *b) {
  return batch_guard([&] {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
  });
}

int fegpu_batch_add(fegpu_batch *b, fegpu_matrix *K, int form, const fegpu_coef *cf, int m,
                    int64_t *job) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b && K && cf && cf->data, "null handle");
    fegpu_femm *fm = K->dm->femm;
    FEGPU_REQUIRE(fm->ctx == b->ctx, "batch: the matrix belongs to another context");
    FEGPU_CUDA(cudaSetDevice(b->ctx->device));
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    for (const auto &J : b->jobs)
      FEGPU_REQUIRE(J.K != K, "batch: the matrix already has a job in this batch");
    int f;
    if (form == FEGPU_FORM_DIFFUSION) {
      f = F_DIFF_ISO;
      FEGPU_REQUIRE(K->dm->ndn == 1 && fm->sdim == fm->mdim,
                    "batch: diffusion needs one DOF per node and sdim == mdim");
    } else if (form == FEGPU_FORM_LIN_ELASTIC) {
      f = F_ELAST_ISO;
      FEGPU_REQUIRE(K->dm->ndn == 3 && fm->mdim == 3 && fm->sdim == 3,
                    "batch: elasticity on 3-D solids with three DOFs per node");
    } else if (form == FEGPU_FORM_DOT) {
      f = F_DOT;
      if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
      else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    } else {
      throw Error{FEGPU_ERR_ARG, "batch: unknown form"};
    }
    const int code = batch_code(fm->etype, f, K->dm->ndn);
    FEGPU_REQUIRE(code >= 0, "batch: this element type, form and DOF count are not batched");
    fegpu_batch::Job J;
    J.K = K;
    J.form = f;
    J.code = code;
    J.m = m;
    b->jobs.push_back(std::move(J));
    try {
      fill_job(b, b->jobs.size() - 1, cf);
    } catch (...) {
      b->jobs.pop_back();
      throw;
    }
    b->dirty = true;
    drop_graph(b);
    if (job) *job = static_cast<int64_t>(b->jobs.size()) - 1;
  });
}

int fegpu_batch_set_coef(fegpu_batch *b, int64_t job, const fegpu_coef *cf) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b && cf && cf->data, "null handle");
    FEGPU_CUDA(cudaSetDevice(b->ctx->device));
    auto &J = job_at(b, job);
    const int te = J.d.k.te;
    fill_job(b, static_cast<size_t>(job), cf);
    J.d.k.te = te;  // keep the queue's tiling
    if (!b->dirty)  // queue and graph stay; refresh this job's descriptor in place
      FEGPU_CUDA(cudaMemcpyAsync(b->d_jobs.as<BatchJob>() + job, &J.d, sizeof(BatchJob),
                                 cudaMemcpyHostToDevice, b->ctx->stream));
    FEGPU_CUDA(cudaStreamSynchronize(b->ctx->stream));
  });
}

int fegpu_batch_launch(fegpu_batch *b) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    FEGPU_CUDA(cudaSetDevice(b->ctx->device));
    if (b->jobs.empty()) return;
    if (b->dirty) {
      drop_graph(b);
      build_queue(b);
    }
    cudaStream_t st = b->ctx->stream;
    if (!b->exec) {
      // the resets and the persistent launch are captured once and replayed
      FEGPU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue_batch(b, st);
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      FEGPU_CUDA(cudaStreamEndCapture(st, &b->graph));
      FEGPU_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    fegpu_context *ctx = b->ctx;
    for (const auto &J : b->jobs) await_export(J.K, st);  // outside the captured graph
    if (ctx->timing) FEGPU_CUDA(cudaEventRecord(ctx->ev0, st));
    FEGPU_CUDA(cudaGraphLaunch(b->exec, st));
    if (ctx->timing) FEGPU_CUDA(cudaEventRecord(ctx->ev1, st));
    ctx->launches += 1;
  });
}

int fegpu_batch_wait(fegpu_batch *b) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    FEGPU_CUDA(cudaSetDevice(b->ctx->device));
    if (b->jobs.empty() || b->dirty) return;
    fegpu_context *ctx = b->ctx;
    check_status(b);
    device_checks(ctx, ctx->stream);
    if (ctx->timing) {
      float ms = 0.f;
      FEGPU_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      ctx->kernel_ms += ms;
    }
  });
}

int fegpu_batch_run(fegpu_batch *b) {
  const int st = fegpu_batch_launch(b);
  return st != FEGPU_OK ? st : fegpu_batch_wait(b);
}

int fegpu_batch_withhold(fegpu_batch *b, int64_t job) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    FEGPU_REQUIRE(job >= -1 && job < static_cast<int64_t>(b->jobs.size()), "batch: no such job");
    int ctr = -1;
    if (job >= 0) {
      // completion counters: two per chunk of every job, jobs in order
      // (batch_queue.cpp); the job's first element stage is its first counter
      ctr = 0;
      for (int64_t j = 0; j < job; ++j)
        ctr += 2 * std::max<int>(0, static_cast<int>(b->jobs[j].K->dm->chunk_nodes.size()) - 1);
    }
    b->withheld = ctr;
    b->dirty = true;  // a captured kernel argument
    drop_graph(b);
  });
}

int fegpu_batch_set_wait_limit(fegpu_batch *b, double seconds) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    FEGPU_REQUIRE(seconds > 0.0 && seconds <= 3600.0, "batch: wait limit out of range");
    b->wait_s = seconds;
    b->dirty = true;  // the limit is a captured kernel argument
    drop_graph(b);
  });
}

// Autotuner: for every job kind without a tile size, time the job of that
// kind with the most elements alone (as a one-job batch) for each candidate
// tile and keep the fastest.  cache_path (may be null) holds lines
// "<kind> <elements per tile>": read first (known kinds are not re-timed),
// appended to after timing.
int fegpu_batch_tune(fegpu_batch *b, const char *cache_path) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    FEGPU_CUDA(cudaSetDevice(b->ctx->device));
    if (cache_path) {
      if (FILE *f = std::fopen(cache_path, "r")) {
        char name[64];
        int te;
        while (std::fscanf(f, "%63s %d", name, &te) == 2)
          for (int c = 0; c < BC_COUNT; ++c)
            if (std::strcmp(name, batch_code_name(c)) == 0 && te > 0 && te <= 4096)
              b->tile[c] = te;
        std::fclose(f);
      }
    }
    std::map<int, size_t> largest;
    for (size_t j = 0; j < b->jobs.size(); ++j) {
      const int c = b->jobs[j].code;
      if (b->tile.count(c)) continue;
      if (!largest.count(c) ||
          b->jobs[j].K->dm->femm->nelem > b->jobs[largest[c]].K->dm->femm->nelem)
        largest[c] = j;
    }
    cudaStream_t st = b->ctx->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FEGPU_CUDA(cudaEventCreate(&e0));
    FEGPU_CUDA(cudaEventCreate(&e1));
    try {
      for (auto &kv : largest) {
        const auto &J = b->jobs[kv.second];
        const fegpu_femm *fm = J.K->dm->femm;
        static const int cands[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128};
        float best = 3.0e38f;
        int best_te = J.d.k.te;
        for (int te : cands) {
          if (te > max_fast_tile(fm->etype) ||
              tile_smem_bytes(fm->etype, J.form, fm->npts, te) > 112 * 1024)
            break;
          fegpu_batch one;
          one.ctx = b->ctx;
          fegpu_batch::Job S;
          S.K = J.K;
          S.form = J.form;
          S.code = J.code;
          S.m = J.m;
          S.d = J.d;
          S.d.k.te = te;
          one.jobs.push_back(std::move(S));
          build_queue(&one);
          enqueue_batch(&one, st);  // warm-up
          check_status(&one);
          FEGPU_CUDA(cudaEventRecord(e0, st));
          for (int r = 0; r < 3; ++r) enqueue_batch(&one, st);
          FEGPU_CUDA(cudaEventRecord(e1, st));
          FEGPU_CUDA(cudaEventSynchronize(e1));
          check_status(&one);
          b->ctx->launches += 4;
          float ms = 0.f;
          FEGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          if (ms < best) {
            best = ms;
            best_te = te;
          }
        }
        b->tile[J.code] = best_te;
        if (cache_path) {
          if (FILE *f = std::fopen(cache_path, "a")) {
            std::fprintf(f, "%s %d\n", batch_code_name(J.code), best_te);
            std::fclose(f);
          }
        }
      }
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &J : b->jobs)
      if (b->tile.count(J.code)) J.d.k.te = b->tile[J.code];
    b->dirty = true;
    drop_graph(b);
  });
}

int fegpu_batch_tile(fegpu_batch *b, int64_t job, int *elements_per_tile) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b && elements_per_tile, "null handle");
    *elements_per_tile = job_at(b, job).d.k.te;
  });
}

int fegpu_batch_stats(fegpu_batch *b, int64_t *jobs, int64_t *items) {
  return batch_guard([&] {
    FEGPU_REQUIRE(b, "null handle");
    if (b->dirty && !b->jobs.empty()) {
      FEGPU_CUDA(cudaSetDevice(b->ctx->device));
      drop_graph(b);
      build_queue(b);
    }
    if (jobs) *jobs = static_cast<int64_t>(b->jobs.size());
    if (items) *items = b->nitems;
  });
}

}  // extern "C"
