// C-ABI entry points of libfegpu (declared in include/fegpu.h).
//
// Every function validates its arguments with the reference's own error
// conditions (AssemblyModule.assemble!/startassembly!, src/AssemblyModule.jl
// 265-273, 463, 511-524), converts Julia-layout host arrays into the device
// layout, and enqueues work on the context's stream.  Element-form launches
// are asynchronous with respect to the host; every copy-out synchronises.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "fegpu_internal.h"
#include "forms_dispatch.cuh"

namespace fegpu {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

template <typename F>
static int guarded(F &&f) {
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
  } catch (...) {
    set_error("unknown failure");
    return FEGPU_ERR_STATE;
  }
}

static void use_device(const fegpu_context *ctx) { FEGPU_CUDA(cudaSetDevice(ctx->device)); }

int launch_mixed(int etype, int form, const KArgs &a, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_Q4: return launch_mixed_q4(form, a, num_sms, s);
    case FEGPU_H8: return launch_mixed_h8(form, a, num_sms, s);
    case FEGPU_H20: return launch_mixed_h20(form, a, num_sms, s);
    case FEGPU_T4: return launch_mixed_t4(form, a, num_sms, s);
    case FEGPU_T10: return launch_mixed_t10(form, a, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

int launch_form(int etype, int form, int precision, int ndn, const KArgs &a, int num_sms,
                cudaStream_t s) {
  switch (etype) {
    case FEGPU_Q4: return launch_form_q4(form, precision, ndn, a, num_sms, s);
    case FEGPU_H8: return launch_form_h8(form, precision, ndn, a, num_sms, s);
    case FEGPU_H20: return launch_form_h20(form, precision, ndn, a, num_sms, s);
    case FEGPU_T4: return launch_form_t4(form, precision, ndn, a, num_sms, s);
    case FEGPU_T10: return launch_form_t10(form, precision, ndn, a, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

// Elements per tile: fill the shared-memory budget, but keep enough
// (element, point) work items for the 256 threads of a CTA.
int choose_tile(int etype, int form, int precision, int npts) {
  const int nne = nodes_per_elem(etype), mdim = manif_dim(etype);
  const bool grad = form <= F_ELAST_GEN;
  const int tsize = (precision == FEGPU_MIXED && grad) ? 4 : 8;
  // shared-memory budget per CTA: measured on T10 60^3 elasticity (FP64),
  // 82 KB (36 elements per tile) runs 1.05x faster than 72 KB (32) and 1.5x
  // faster than 100 KB (44): two CTAs per SM either way, but the larger
  // carve-out leaves the scatter's loads less L1
  const size_t budget = (etype == FEGPU_H20) ? 200 * 1024 : 82 * 1024;
  const SmemLayout one = smem_layout(nne, mdim, npts, 1, tsize, grad);
  const SmemLayout two = smem_layout(nne, mdim, npts, 2, tsize, grad);
  const size_t per = two.total - one.total;
  const size_t fixed = one.total > per ? one.total - per : 0;
  int te = static_cast<int>((budget - std::min(budget, fixed)) / std::max<size_t>(per, 1));
  const int want = std::max(1, (2 * kFormThreads + npts - 1) / npts);
  te = std::max(1, std::min(te, want));
  // FEGPU_FP64_TILE overrides the elements per tile of the FP64 colour
  // kernels (tuning; capped by the shared memory of one CTA)
  if (precision != FEGPU_MIXED) {
    if (const char *env = std::getenv("FEGPU_FP64_TILE")) {
      const int v = std::atoi(env);
      if (v > 0) {
        te = v;
        while (te > 1 && smem_layout(nne, mdim, npts, te, tsize, grad).total > 227 * 1024) --te;
      }
    }
  }
  return te;
}

int mixed_tile_for(int etype, int form, int npts, bool wide) {
  return default_tile(etype, form, npts, wide);
}
size_t mixed_smem_for(int etype, int form, int npts, int te) {
  return tile_smem_bytes(etype, form, npts, te);
}

size_t form_smem_bytes(int etype, int form, int precision, int npts, int te) {
  const bool grad = form <= F_ELAST_GEN;
  const int tsize = (precision == FEGPU_MIXED && grad) ? 4 : 8;
  return smem_layout(nodes_per_elem(etype), manif_dim(etype), npts, te, tsize, grad).total;
}

namespace {

__global__ void k_pack_xyz(const double *src, int64_t n, int sdim, double *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    dst[4 * i] = src[i];
    dst[4 * i + 1] = sdim > 1 ? src[n + i] : 0.0;
    dst[4 * i + 2] = sdim > 2 ? src[2 * n + i] : 0.0;
    dst[4 * i + 3] = 0.0;
  }
}

__global__ void k_gather_rows(const double *src, const int32_t *perm, int64_t nrows,
                              int64_t width, double *dst) {
  const int64_t total = nrows * width;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / width, c = t - r * width;
    dst[t] = src[static_cast<int64_t>(perm[r]) * width + c];
  }
}

int grid_of(int64_t n) {
  return static_cast<int>(std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 1 << 20));
}

// Per-call coefficient staging: device copy in colour order.
struct CoefStage {
  DevBuf raw, sorted;
};

void validate_conn(const int64_t *conn, int64_t nelem, int nne, int64_t nnodes,
                   std::vector<int32_t> &c0) {
  c0.resize(static_cast<size_t>(nelem) * nne);
  for (int64_t e = 0; e < nelem; ++e) {
    for (int a = 0; a < nne; ++a) {
      const int64_t n = conn[e * nne + a];
      FEGPU_REQUIRE(n >= 1, "connectivity: node number < 1");
      FEGPU_REQUIRE(n <= nnodes, "connectivity: node number > number of nodes");
      c0[e * nne + a] = static_cast<int32_t>(n - 1);
    }
    for (int a = 0; a < nne; ++a)
      for (int b = a + 1; b < nne; ++b)
        FEGPU_REQUIRE(c0[e * nne + a] != c0[e * nne + b],
                      "connectivity: an element lists a node twice");
  }
}

// Copies the caller's coefficient into KArgs (constant) or a device array in
// colour order (per element / per point).
void stage_coef(fegpu_femm *fm, const fegpu_coef *cf, int expect_ncomp, KArgs &a,
                CoefStage &st, bool colour_order = true) {
  FEGPU_REQUIRE(cf != nullptr && cf->data != nullptr, "coefficient: null data");
  a.coef_kind = cf->kind;
  a.ncomp = cf->ncomp;
  a.coef = nullptr;
  if (cf->kind == FEGPU_COEF_CONST) {
    FEGPU_REQUIRE(cf->ncomp >= 1 && cf->ncomp <= 36, "coefficient: too many components");
    for (int i = 0; i < cf->ncomp; ++i) a.cconst[i] = cf->data[i];
    return;
  }
  int64_t width = 0;
  if (cf->kind == FEGPU_COEF_PER_ELEMENT) width = cf->ncomp;
  else if (cf->kind == FEGPU_COEF_PER_QP) width = static_cast<int64_t>(cf->ncomp) * fm->npts;
  else if (cf->kind == FEGPU_COEF_ISO_LAME) width = 2;
  else throw Error{FEGPU_ERR_ARG, "coefficient: unknown kind"};
  (void)expect_ncomp;
  const int64_t n = fm->nelem * width;
  cudaStream_t s = fm->ctx->stream;
  st.raw.alloc(sizeof(double) * n);
  st.sorted.alloc(sizeof(double) * n);
  FEGPU_CUDA(cudaMemcpyAsync(st.raw.p, cf->data, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (!colour_order) {
    a.coef = st.raw.as<double>();
    return;
  }
  k_gather_rows<<<grid_of(n), 256, 0, s>>>(st.raw.as<double>(), fm->perm.as<int32_t>(),
                                           fm->nelem, width, st.sorted.as<double>());
  FEGPU_CUDA(cudaGetLastError());
  fm->ctx->launches++;
  a.coef = st.sorted.as<double>();
}

}  // namespace

void pack_geometry(const double *src_colmajor, int64_t nnodes, int sdim, double *xyz4,
                   cudaStream_t s) {
  if (nnodes <= 0) return;
  k_pack_xyz<<<grid_of(nnodes), 256, 0, s>>>(src_colmajor, nnodes, sdim, xyz4);
  FEGPU_CUDA(cudaGetLastError());
}

void await_export(fegpu_matrix *K, cudaStream_t s) {
  if (K && K->export_pending) FEGPU_CUDA(cudaStreamWaitEvent(s, K->exported, 0));
}

void device_checks(fegpu_context *ctx, cudaStream_t s) {
  if (!kDeviceChecks || !ctx->check_word.p) return;
  unsigned long long w = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&w, ctx->check_word.p, sizeof(w), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  if (w == 0) return;
  FEGPU_CUDA(cudaMemsetAsync(ctx->check_word.p, 0, sizeof(w), s));
  static const char *const kSites[] = {"?", "node number of an element", "CSR slot of the scatter",
                                       "CSR slot of the row gather", "vector entry"};
  const int site = static_cast<int>(w >> 56);
  throw Error{FEGPU_ERR_DEVICE,
              std::string("device index check: ") + kSites[site <= 4 ? site : 0] + " " +
                  std::to_string(static_cast<long long>(w & ((1ull << 56) - 1ull))) +
                  " out of range (the kernel skipped the access)"};
}

KArgs base_args(fegpu_matrix *K, fegpu_dofmap *dm) {
  fegpu_femm *fm = dm->femm;
  await_export(K, fm->ctx->stream);
  KArgs a;
  std::memset(&a, 0, sizeof(a));
  a.conn = fm->conn.as<int32_t>();
  a.xyz = fm->xyz.as<double>();
  a.tab = fm->tab.as<double>();
  a.tab32 = fm->tab32.as<float>();
  a.pos = dm->pos.as<uint16_t>();
  a.dof = dm->dof.as<int32_t>();
  a.rowptr = dm->rowptr.as<int64_t>();
  a.colperm = dm->contiguous ? nullptr : dm->colperm.as<int32_t>();
  a.cpoff = dm->contiguous ? nullptr : dm->cpoff.as<int64_t>();
  a.val = K ? K->val.as<double>() : nullptr;
  a.nnz = dm->nnz;
  a.nnodes = fm->nnodes;
  a.check = fm->ctx->check_word.as<unsigned long long>();  // null without device checks
  a.npts = fm->npts;
  a.sdim = fm->sdim;
  a.otherdim = fm->otherdim;
  a.axisym = fm->axisym;
  a.measure_m = 3;
  // mixed path: elements whose det J ratio over the points falls below this
  // take FP64 Jacobians.  T10 takes them always: its FP32 Jacobian sums ten
  // cancelling terms per entry, and FP64 geometry cuts the assembled T10 60^3
  // error from 1.2e-6 to 1.4e-7 (max |dK| / max |K|) for 17 % more time.
  // FEGPU_MIXED_FP64_GEOMETRY=1 / 0 forces FP64 geometry for every / only the
  // distorted elements of any type.
  // FP64 geometry in the mixed tiles: distorted elements (det_min / det_max
  // below 0.1) and curved T10 (an isoparametric T10 Jacobian entry sums ten
  // cancelling terms; a straight-sided T10 is affine and takes its exact
  // corner Jacobian in FP32).  FEGPU_MIXED_FP64_GEOMETRY=1: FP64 for every
  // element; =0: only for the distorted ones (isoparametric FP32 T10).
  a.distort_tol = 0.1;
  a.t10_affine = fm->etype == FEGPU_T10 ? 1 : 0;
  if (const char *env = std::getenv("FEGPU_MIXED_FP64_GEOMETRY")) {
    if (env[0] == '1') a.distort_tol = 2.0;
    else if (env[0] == '0') a.t10_affine = 0;
  }
  return a;
}

namespace {

void run_colours(fegpu_dofmap *dm, int form, int precision, KArgs &a) {
  fegpu_femm *fm = dm->femm;
  a.te = choose_tile(fm->etype, form, precision, fm->npts);
  const size_t smem = form_smem_bytes(fm->etype, form, precision, fm->npts, a.te);
  FEGPU_REQUIRE(smem <= 227 * 1024, "quadrature rule too large for the element kernel");
  fegpu_context *ctx = fm->ctx;
  const int ncol = static_cast<int>(fm->color_offsets.size()) - 1;
  if (ctx->timing) FEGPU_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  const int te_max = a.te;
  const bool fixed = std::getenv("FEGPU_FP64_TILE") != nullptr;
  // resident CTAs per SM of the colour kernels: two (registers), one when a
  // tile's shared memory leaves no room for a second
  const size_t smem_max = form_smem_bytes(fm->etype, form, precision, fm->npts, te_max);
  const int64_t slots =
      static_cast<int64_t>(ctx->num_sms) * (smem_max + 1024 <= 113 * 1024 ? 2 : 1);
  for (int c = 0; c < ncol; ++c) {
    a.e0 = fm->color_offsets[c];
    a.e1 = fm->color_offsets[c + 1];
    // elements per tile: the time of a colour goes as (waves of tiles over
    // the CTA slots) x (elements per tile), so pick the tile in
    // [te_max / 2, te_max] (at least 4) that minimises that product, ties to
    // the larger tile (T10 60^3, 32.4 k-element colours: 36 per tile, three
    // full waves, against four waves at 32); small colours get small tiles
    // (H8 20^3 diffusion, 1,000-element colours: 4 per tile, one wave)
    const int64_t n = a.e1 - a.e0;
    int best = te_max;
    if (!fixed) {
      int64_t best_cost = -1;
      for (int te = std::max(1, std::min(4, te_max)); te <= te_max; ++te) {
        if (te < te_max / 2 && (n + te - 1) / te > slots) continue;
        const int64_t waves = ((n + te - 1) / te + slots - 1) / slots;
        const int64_t cost = waves * te;
        if (best_cost < 0 || cost < best_cost || (cost == best_cost && te > best)) {
          best_cost = cost;
          best = te;
        }
      }
    }
    a.te = best;
    ctx->launches += launch_form(fm->etype, form, precision, dm->ndn, a, ctx->num_sms, ctx->stream);
  }
  a.te = te_max;
  if (ctx->timing) {
    FEGPU_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    FEGPU_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    FEGPU_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->kernel_ms += ms;
  }
}

// Mixed precision: element blocks in FP32 into the ring, then the row gather
// (gather.cu), chunk by chunk in element order.
void run_gather(fegpu_dofmap *dm, int form, KArgs &a) {
  fegpu_femm *fm = dm->femm;
  fegpu_context *ctx = fm->ctx;
  const int nne = fm->nne, ndn = dm->ndn;
  const int bs = ndn * ndn, nblk = nne * (nne + 1) / 2;
  if (!dm->gather_ready) build_gather_plan(dm, nblk * bs);
  a.conn = fm->conn_orig.as<int32_t>();
  a.te = default_tile(fm->etype, form, fm->npts, false);  // the single-call tile
  FEGPU_REQUIRE(tile_smem_bytes(fm->etype, form, fm->npts, a.te) <= 227 * 1024,
                "quadrature rule too large for the element kernel");
  GArgs g;
  std::memset(&g, 0, sizeof(g));
  g.n2e_ptr = dm->n2e_ptr.as<int64_t>();
  g.n2e_elem = dm->n2e_elem.as<int32_t>();
  g.n2e_loc = dm->n2e_loc.as<uint8_t>();
  g.n2e_slot = dm->n2e_slot.as<int32_t>();
  g.nodes = dm->gnodes.as<int32_t>();
  g.nptr = dm->nptr.as<int64_t>();
  g.pos = dm->pos_orig.as<uint16_t>();
  g.ke = dm->ke.as<float>();
  g.chunk = dm->chunk;
  g.ring = dm->ring;
  g.dof = dm->dof.as<int32_t>();
  g.rowptr = dm->rowptr.as<int64_t>();
  g.colperm = dm->contiguous ? nullptr : dm->colperm.as<int32_t>();
  g.cpoff = dm->contiguous ? nullptr : dm->cpoff.as<int64_t>();
  g.val = a.val;
  g.maxdeg = dm->maxdeg;
  g.check = a.check;
  g.nnz = dm->nnz;
  const int64_t nch = static_cast<int64_t>(dm->chunk_nodes.size()) - 1;
  // Element blocks on the side stream, gathers on the context stream: the
  // blocks of chunk c wait for the gather that last read their ring slot
  // (G(c - ring + span)) and for everything before this call; the gather of
  // chunk c waits for the blocks of chunk c.  Events are kept per ring slot.
  cudaStream_t s0 = ctx->stream;
  if (!ctx->side) FEGPU_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
  while (static_cast<int>(ctx->ev_blocks.size()) < dm->ring) {
    cudaEvent_t e1, e2;
    FEGPU_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
    FEGPU_CUDA(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
    ctx->ev_blocks.push_back(e1);
    ctx->ev_gather.push_back(e2);
  }
  // the element-block grid covers a share of the SMs' CTA slots, so the
  // gathers find room beside it (FEGPU_MIXED_BLOCK_SHARE overrides, 0..1)
  double share = 1.0;
  if (const char *env = std::getenv("FEGPU_MIXED_BLOCK_SHARE")) {
    const double v = std::atof(env);
    if (v > 0.0 && v <= 1.0) share = v;
  }
  const int block_sms = std::max(1, static_cast<int>(ctx->num_sms * share));
  if (!ctx->tc_status.p) {
    ctx->tc_status.alloc(sizeof(int));
    FEGPU_CUDA(cudaMemsetAsync(ctx->tc_status.p, 0, sizeof(int), s0));
  }
  a.status = ctx->tc_status.as<int>();
  if (ctx->timing) FEGPU_CUDA(cudaEventRecord(ctx->ev0, s0));
  FEGPU_CUDA(cudaEventRecord(ctx->ev_gather[0], s0));  // work before this call
  FEGPU_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_gather[0], 0));
  for (int64_t c = 0; c < nch; ++c) {
    const int slot = static_cast<int>(c % dm->ring);
    if (c >= dm->ring) {
      const int64_t reader = c - dm->ring + dm->span;  // last gather reading the slot
      FEGPU_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_gather[reader % dm->ring], 0));
    }
    a.e0 = c * dm->chunk;
    a.e1 = std::min(fm->nelem, (c + 1) * dm->chunk);
    a.ke = dm->ke.as<float>() + slot * dm->chunk * nblk * bs;
    ctx->launches += launch_mixed(fm->etype, form, a, block_sms, ctx->side);
    FEGPU_CUDA(cudaEventRecord(ctx->ev_blocks[slot], ctx->side));
    FEGPU_CUDA(cudaStreamWaitEvent(s0, ctx->ev_blocks[slot], 0));
    g.n0 = dm->chunk_nodes[c];
    g.n1 = dm->chunk_nodes[c + 1];
    ctx->launches += launch_gather(fm->etype, ndn, g, ctx->num_sms, s0);
    FEGPU_CUDA(cudaEventRecord(ctx->ev_gather[slot], s0));
  }
  if (ctx->timing) {
    FEGPU_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    FEGPU_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    FEGPU_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->kernel_ms += ms;
  }
  // the tensor-core element kernel reports a wait that ran out
  int st = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&st, ctx->tc_status.p, sizeof(int), cudaMemcpyDeviceToHost, s0));
  FEGPU_CUDA(cudaStreamSynchronize(s0));
  if (st != 0) {
    FEGPU_CUDA(cudaMemsetAsync(ctx->tc_status.p, 0, sizeof(int), s0));
    throw Error{FEGPU_ERR_DEVICE, "mixed path: tensor-core completion wait ran out"};
  }
}

void run_form(fegpu_dofmap *dm, int form, int precision, KArgs &a) {
  if (precision == FEGPU_MIXED && form <= F_ELAST_GEN) run_gather(dm, form, a);
  else run_colours(dm, form, precision, a);
}

void require_geometry(fegpu_femm *fm) {
  FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
}

}  // namespace

bool is_isotropic(const double *D, double &lam, double &mu) {
  const double a = D[0], b = D[1], c = D[3 * 6 + 3];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double expect;
      if (i < 3 && j < 3) expect = (i == j) ? a : b;
      else if (i == j) expect = c;
      else expect = 0.0;
      if (D[i * 6 + j] != expect) return false;
    }
  if (a != b + 2.0 * c) return false;
  lam = b;
  mu = c;
  return true;
}

bool iso_pattern(const double *D, double &d0, double &d1, double &d3) {
  d0 = D[0];
  d1 = D[1];
  d3 = D[3 * 6 + 3];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double expect;
      if (i < 3 && j < 3) expect = (i == j) ? d0 : d1;
      else if (i == j) expect = d3;
      else expect = 0.0;
      if (D[i * 6 + j] != expect) return false;
    }
  return true;
}

}  // namespace fegpu

using namespace fegpu;

extern "C" {

const char *fegpu_last_error(void) { return g_last_error.c_str(); }

int fegpu_context_create(int device, fegpu_context **out) {
  return guarded([&] {
    FEGPU_REQUIRE(out != nullptr, "null output handle");
    int ndev = 0;
    FEGPU_CUDA(cudaGetDeviceCount(&ndev));
    FEGPU_REQUIRE(device >= 0 && device < ndev, "no such CUDA device");
    FEGPU_CUDA(cudaSetDevice(device));
    auto *ctx = new fegpu_context();
    ctx->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      throw Error{FEGPU_ERR_CUDA, std::string("context: ") + cudaGetErrorString(e)};
    }
    try {
      noalloc_prepare(device);
      if (kDeviceChecks) {
        ctx->check_word.alloc(sizeof(unsigned long long));
        FEGPU_CUDA(cudaMemset(ctx->check_word.p, 0, sizeof(unsigned long long)));
      }
    } catch (...) {
      cudaStreamDestroy(ctx->stream);
      delete ctx;
      throw;
    }
    *out = ctx;
  });
}

int fegpu_context_stream(fegpu_context *ctx, void **stream) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx && stream, "null handle");
    *stream = static_cast<void *>(ctx->stream);
  });
}

int fegpu_context_timing(fegpu_context *ctx, int enable) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx, "null context");
    use_device(ctx);
    if (enable && !ctx->ev0) {
      FEGPU_CUDA(cudaEventCreate(&ctx->ev0));
      FEGPU_CUDA(cudaEventCreate(&ctx->ev1));
    }
    ctx->timing = enable != 0;
  });
}

int fegpu_context_kernel_stats(fegpu_context *ctx, double *kernel_ms, int64_t *launches,
                               int reset) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx, "null context");
    if (kernel_ms) *kernel_ms = ctx->kernel_ms;
    if (launches) *launches = ctx->launches;
    if (reset) {
      ctx->kernel_ms = 0.0;
      ctx->launches = 0;
    }
  });
}

int fegpu_context_device_checks(fegpu_context *ctx, int *enabled) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx && enabled, "null handle");
    *enabled = kDeviceChecks ? 1 : 0;
  });
}

int fegpu_context_destroy(fegpu_context *ctx) {
  return guarded([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (cudaEvent_t e : ctx->ev_blocks) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ev_gather) cudaEventDestroy(e);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->export_stream) {
      cudaStreamSynchronize(ctx->export_stream);
      cudaStreamDestroy(ctx->export_stream);
    }
    ctx->scratch.release();
    ctx->scratch2.release();
    cudaStreamDestroy(ctx->stream);
    delete ctx;
  });
}

int fegpu_context_synchronize(fegpu_context *ctx) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx, "null context");
    use_device(ctx);
    FEGPU_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int fegpu_femm_create(fegpu_context *ctx, int etype, int64_t nelem, const int64_t *conn,
                      int64_t nnodes, int npts, const double *Ns, const double *gradNparams,
                      const double *w, double otherdimension, fegpu_femm **out) {
  return guarded([&] {
    FEGPU_REQUIRE(ctx && out, "null handle");
    const int nne = nodes_per_elem(etype);
    FEGPU_REQUIRE(nne > 0, "unknown element type");
    FEGPU_REQUIRE(nelem >= 0 && nnodes > 0 && nnodes < (int64_t(1) << 31),
                  "bad element or node count");
    FEGPU_REQUIRE(nelem == 0 || conn, "null connectivity");
    FEGPU_REQUIRE(npts >= 1 && npts <= max_qp(etype), "unsupported number of quadrature points");
    FEGPU_REQUIRE(Ns && gradNparams && w, "null integration tables");
    FEGPU_REQUIRE(std::isfinite(otherdimension), "other dimension must be a finite number");
    use_device(ctx);
    const int mdim = manif_dim(etype);
    auto fm = std::make_unique<fegpu_femm>();
    fm->ctx = ctx;
    fm->etype = etype;
    fm->nne = nne;
    fm->mdim = mdim;
    fm->npts = npts;
    fm->nelem = nelem;
    fm->nnodes = nnodes;
    fm->otherdim = otherdimension;
    std::vector<int32_t> c0;
    validate_conn(conn, nelem, nne, nnodes, c0);
    const int64_t ncol = nelem > 0 ? greedy_element_coloring(nelem, nne, c0.data(), nnodes, fm->colors) : 0;
    // stable sort of the elements by colour
    std::vector<int64_t> off(ncol + 1, 0);
    for (int64_t e = 0; e < nelem; ++e) off[fm->colors[e]]++;
    for (int64_t c = 0; c < ncol; ++c) off[c + 1] += off[c];
    std::vector<int64_t> fill(off.begin(), off.end());
    std::vector<int32_t> perm(nelem), cs(static_cast<size_t>(nelem) * nne);
    for (int64_t e = 0; e < nelem; ++e) {
      const int64_t p = fill[fm->colors[e] - 1]++;
      perm[p] = static_cast<int32_t>(e);
      std::memcpy(&cs[p * nne], &c0[e * nne], sizeof(int32_t) * nne);
    }
    fm->color_offsets = off;
    fm->conn_host = c0;
    cudaStream_t s = ctx->stream;
    fm->conn_orig.alloc(sizeof(int32_t) * c0.size());
    fm->conn.alloc(sizeof(int32_t) * cs.size());
    fm->perm.alloc(sizeof(int32_t) * perm.size());
    if (nelem > 0) {
      FEGPU_CUDA(cudaMemcpyAsync(fm->conn_orig.p, c0.data(), sizeof(int32_t) * c0.size(),
                                 cudaMemcpyHostToDevice, s));
      FEGPU_CUDA(cudaMemcpyAsync(fm->conn.p, cs.data(), sizeof(int32_t) * cs.size(),
                                 cudaMemcpyHostToDevice, s));
      FEGPU_CUDA(cudaMemcpyAsync(fm->perm.p, perm.data(), sizeof(int32_t) * perm.size(),
                                 cudaMemcpyHostToDevice, s));
    }
    std::vector<double> tab(static_cast<size_t>(npts) * nne * (mdim + 1) + npts);
    std::memcpy(tab.data(), Ns, sizeof(double) * npts * nne);
    std::memcpy(tab.data() + npts * nne, gradNparams, sizeof(double) * npts * nne * mdim);
    std::memcpy(tab.data() + npts * nne * (mdim + 1), w, sizeof(double) * npts);
    fm->tab.alloc(sizeof(double) * tab.size());
    FEGPU_CUDA(cudaMemcpyAsync(fm->tab.p, tab.data(), sizeof(double) * tab.size(),
                               cudaMemcpyHostToDevice, s));
    std::vector<float> tab32(tab.size());  // N, dN, w in FP32
    for (size_t i = 0; i < tab32.size(); ++i) tab32[i] = static_cast<float>(tab[i]);
    fm->tab32.alloc(sizeof(float) * tab32.size());
    FEGPU_CUDA(cudaMemcpyAsync(fm->tab32.p, tab32.data(), sizeof(float) * tab32.size(),
                               cudaMemcpyHostToDevice, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
    *out = fm.release();
  });
}

int fegpu_femm_destroy(fegpu_femm *femm) {
  return guarded([&] {
    if (!femm) return;
    cudaSetDevice(femm->ctx->device);
    cudaStreamSynchronize(femm->ctx->stream);
    delete femm;
  });
}

int fegpu_femm_set_axisymmetric(fegpu_femm *fm, int axisymmetric) {
  return guarded([&] {
    FEGPU_REQUIRE(fm, "null handle");
    fm->axisym = axisymmetric ? 1 : 0;
  });
}

int fegpu_femm_set_geometry(fegpu_femm *fm, int sdim, const double *xyz) {
  return guarded([&] {
    FEGPU_REQUIRE(fm && xyz, "null handle");
    FEGPU_REQUIRE(sdim >= fm->mdim && sdim <= 3, "geometry: bad number of space dimensions");
    use_device(fm->ctx);
    cudaStream_t s = fm->ctx->stream;
    const int64_t n = fm->nnodes;
    fm->ctx->scratch2.alloc(sizeof(double) * n * sdim);
    FEGPU_CUDA(cudaMemcpyAsync(fm->ctx->scratch2.p, xyz, sizeof(double) * n * sdim,
                               cudaMemcpyHostToDevice, s));
    fm->xyz.alloc(sizeof(double) * 4 * n);
    k_pack_xyz<<<grid_of(n), 256, 0, s>>>(fm->ctx->scratch2.as<double>(), n, sdim,
                                          fm->xyz.as<double>());
    FEGPU_CUDA(cudaGetLastError());
    fm->ctx->launches++;
    fm->sdim = sdim;
    fm->has_geometry = true;
  });
}

int fegpu_femm_colors(fegpu_femm *fm, int64_t *colors, int64_t *ncolors) {
  return guarded([&] {
    FEGPU_REQUIRE(fm, "null handle");
    if (colors) std::memcpy(colors, fm->colors.data(), sizeof(int64_t) * fm->nelem);
    if (ncolors) *ncolors = static_cast<int64_t>(fm->color_offsets.size()) - 1;
  });
}

int fegpu_dofmap_create(fegpu_femm *fm, int ndn, const int64_t *dofnums, int64_t nalldofs,
                        fegpu_dofmap **out, int64_t *nnz) {
  return guarded([&] {
    FEGPU_REQUIRE(fm && out && dofnums, "null handle");
    FEGPU_REQUIRE(ndn >= 1 && ndn <= 3, "DOFs per node must be 1, 2 or 3");
    FEGPU_REQUIRE(nalldofs >= 1 && nalldofs < (int64_t(1) << 31), "bad number of DOFs");
    use_device(fm->ctx);
    const int64_t N = fm->nnodes;
    // nodes referenced by elements must carry valid, distinct DOF numbers
    std::vector<char> ref(N, 0);
    {
      std::vector<int32_t> c0(static_cast<size_t>(fm->nelem) * fm->nne);
      if (fm->nelem > 0)
        FEGPU_CUDA(cudaMemcpy(c0.data(), fm->conn_orig.p, sizeof(int32_t) * c0.size(),
                              cudaMemcpyDeviceToHost));
      for (int32_t n : c0) ref[n] = 1;
    }
    std::vector<int32_t> hdof(static_cast<size_t>(N) * ndn);
    std::vector<char> seen(nalldofs, 0);
    for (int64_t n = 0; n < N; ++n)
      for (int j = 0; j < ndn; ++j) {
        const int64_t d = dofnums[j * N + n];  // column-major nnodes x ndn
        if (ref[n]) {
          FEGPU_REQUIRE(d >= 1, "Row degree of freedom < 1");
          FEGPU_REQUIRE(d <= nalldofs, "Row degree of freedom > size");
          FEGPU_REQUIRE(!seen[d - 1], "a DOF number is used twice");
          seen[d - 1] = 1;
        }
        hdof[n * ndn + j] = (d >= 1 && d <= nalldofs) ? static_cast<int32_t>(d - 1) : 0;
      }
    auto dm = std::make_unique<fegpu_dofmap>();
    dm->femm = fm;
    dm->ndn = ndn;
    dm->ndof = nalldofs;
    if (fm->nelem == 0) {
      dm->nnz = 0;
      dm->rowptr.alloc(sizeof(int64_t) * (nalldofs + 1));
      FEGPU_CUDA(cudaMemset(dm->rowptr.p, 0, sizeof(int64_t) * (nalldofs + 1)));
      dm->colind.alloc(16);
      dm->pos.alloc(16);
      dm->dof.alloc(sizeof(int32_t) * hdof.size());
      FEGPU_CUDA(cudaMemcpy(dm->dof.p, hdof.data(), sizeof(int32_t) * hdof.size(),
                            cudaMemcpyHostToDevice));
    } else {
      build_pattern(dm.get(), hdof);
    }
    if (nnz) *nnz = dm->nnz;
    *out = dm.release();
  });
}

int fegpu_dofmap_destroy(fegpu_dofmap *dm) {
  return guarded([&] {
    if (!dm) return;
    cudaSetDevice(dm->femm->ctx->device);
    cudaStreamSynchronize(dm->femm->ctx->stream);
    delete dm;
  });
}

int fegpu_dofmap_copy_pattern(fegpu_dofmap *dm, int64_t *colptr, int64_t *rowval) {
  return guarded([&] {
    FEGPU_REQUIRE(dm && colptr && rowval, "null handle");
    use_device(dm->femm->ctx);
    copy_csc(dm->femm->ctx, dm, nullptr, 0, colptr, rowval, nullptr);
  });
}

int fegpu_matrix_create(fegpu_dofmap *dm, fegpu_matrix **out) {
  return guarded([&] {
    FEGPU_REQUIRE(dm && out, "null handle");
    use_device(dm->femm->ctx);
    auto K = std::make_unique<fegpu_matrix>();
    K->dm = dm;
    K->val.alloc(sizeof(double) * (dm->nnz + 1));
    FEGPU_CUDA(cudaMemsetAsync(K->val.p, 0, sizeof(double) * (dm->nnz + 1), dm->femm->ctx->stream));
    *out = K.release();
  });
}

int fegpu_matrix_destroy(fegpu_matrix *K) {
  return guarded([&] {
    if (!K) return;
    cudaSetDevice(K->dm->femm->ctx->device);
    cudaStreamSynchronize(K->dm->femm->ctx->stream);
    if (K->exported) cudaEventSynchronize(K->exported);  // a copy may still read val
    if (K->ready) cudaEventDestroy(K->ready);
    if (K->exported) cudaEventDestroy(K->exported);
    delete K;
  });
}

int fegpu_matrix_set_symmetric_assembly(fegpu_matrix *K, int symmetric) {
  return guarded([&] {
    FEGPU_REQUIRE(K, "null handle");
    K->symm_asm = symmetric != 0;
  });
}

static void zero_matrix(fegpu_matrix *K) {
  FEGPU_CUDA(cudaMemsetAsync(K->val.p, 0, sizeof(double) * K->dm->nnz, K->dm->femm->ctx->stream));
}

int fegpu_bilform_diffusion(fegpu_matrix *K, const fegpu_coef *cf, int precision) {
  return guarded([&] {
    FEGPU_REQUIRE(K && cf, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    use_device(fm->ctx);
    require_geometry(fm);
    FEGPU_REQUIRE(dm->ndn == 1, "diffusion: the field must have one DOF per node");
    FEGPU_REQUIRE(fm->sdim == fm->mdim, "diffusion: the element must fill the space");
    FEGPU_REQUIRE(precision == FEGPU_FP64 || precision == FEGPU_MIXED ||
                      precision == FEGPU_FP64_FAST,
                  "unknown precision");
    const int md = fm->mdim;
    int form;
    if (cf->ncomp == 1) {
      form = F_DIFF_ISO;
      FEGPU_REQUIRE(cf->kind != FEGPU_COEF_ISO_LAME, "diffusion: bad coefficient kind");
    } else {
      FEGPU_REQUIRE(cf->ncomp == md * md, "diffusion: coefficient must be scalar or mdim x mdim");
      FEGPU_REQUIRE(cf->kind == FEGPU_COEF_CONST || cf->kind == FEGPU_COEF_PER_ELEMENT ||
                        cf->kind == FEGPU_COEF_PER_QP,
                    "diffusion: a matrix coefficient must be constant, per element or per point");
      form = F_DIFF_GEN;
    }
    K->unsym = false;
    KArgs a = base_args(K, dm);
    CoefStage st;
    const bool exact = precision == FEGPU_FP64;
    const bool gather = precision == FEGPU_MIXED || exact;
    stage_coef(fm, cf, cf->ncomp, a, st, !gather);
    if (exact) {
      if (fm->nelem > 0) run_exact(dm, form, a, K->symm_asm);
      else zero_matrix(K);
    } else {
      if (!gather) zero_matrix(K);
      if (fm->nelem > 0) run_form(dm, form, precision, a);
    }
    FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));  // st owns the staged data
    device_checks(fm->ctx, fm->ctx->stream);
  });
}

int fegpu_bilform_lin_elastic(fegpu_matrix *K, const fegpu_coef *cf, int precision) {
  return guarded([&] {
    FEGPU_REQUIRE(K && cf, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    use_device(fm->ctx);
    require_geometry(fm);
    FEGPU_REQUIRE(fm->mdim == 3 && fm->sdim == 3, "lin_elastic: 3-D solid elements only");
    FEGPU_REQUIRE(dm->ndn == 3, "lin_elastic: the field must have three DOFs per node");
    FEGPU_REQUIRE(precision == FEGPU_FP64 || precision == FEGPU_MIXED ||
                      precision == FEGPU_FP64_FAST,
                  "unknown precision");
    K->unsym = false;
    KArgs a = base_args(K, dm);
    CoefStage st;
    int form;
    if (precision == FEGPU_FP64) {
      // reference order: the 6x6 D entries themselves (an isotropic pattern
      // skips D's zeros), per-element (lambda, mu) pairs formed into D's
      // entries on the device as the 6x6 D is formed
      if (cf->kind == FEGPU_COEF_ISO_LAME) {
        form = F_ELAST_ISO;
        stage_coef(fm, cf, 2, a, st, false);
      } else if (cf->kind == FEGPU_COEF_CONST && cf->ncomp == 36) {
        double d0, d1, d3;
        if (iso_pattern(cf->data, d0, d1, d3)) {
          form = F_ELAST_ISO;
          a.coef_kind = FEGPU_COEF_CONST;
          a.ncomp = 3;
          a.cconst[0] = d0;
          a.cconst[1] = d1;
          a.cconst[2] = d3;
        } else {
          form = F_ELAST_GEN;
          stage_coef(fm, cf, 36, a, st, false);
        }
      } else if ((cf->kind == FEGPU_COEF_PER_ELEMENT || cf->kind == FEGPU_COEF_PER_QP) &&
                 cf->ncomp == 36) {
        form = F_ELAST_GEN;
        stage_coef(fm, cf, 36, a, st, false);
      } else {
        throw Error{FEGPU_ERR_ARG,
                    "lin_elastic: coefficient must be a 6x6 D (constant, per element or per "
                    "point) or per-element (lambda, mu)"};
      }
      if (fm->nelem > 0) run_exact(dm, form, a, K->symm_asm);
      else zero_matrix(K);
      FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));
      device_checks(fm->ctx, fm->ctx->stream);
      return;
    }
    const bool gather = precision == FEGPU_MIXED;
    if (cf->kind == FEGPU_COEF_ISO_LAME) {
      form = F_ELAST_ISO;
      stage_coef(fm, cf, 2, a, st, !gather);
    } else if (cf->kind == FEGPU_COEF_CONST && cf->ncomp == 36) {
      double lam, mu;
      if (is_isotropic(cf->data, lam, mu)) {
        form = F_ELAST_ISO;
        a.coef_kind = FEGPU_COEF_CONST;
        a.ncomp = 2;
        a.cconst[0] = lam;
        a.cconst[1] = mu;
      } else {
        form = F_ELAST_GEN;
        stage_coef(fm, cf, 36, a, st, !gather);
      }
    } else if (cf->kind == FEGPU_COEF_PER_ELEMENT && cf->ncomp == 36) {
      form = F_ELAST_GEN;
      stage_coef(fm, cf, 36, a, st, !gather);
    } else if (cf->kind == FEGPU_COEF_PER_QP) {
      // these paths apply D to the element's point-summed gradient products,
      // which needs one D per element
      throw Error{FEGPU_ERR_ARG,
                  "lin_elastic: a D that varies over the points of an element needs precision "
                  "FEGPU_FP64"};
    } else {
      throw Error{FEGPU_ERR_ARG,
                  "lin_elastic: coefficient must be a 6x6 D (constant or per element) or "
                  "per-element (lambda, mu)"};
    }
    if (!gather) zero_matrix(K);
    if (fm->nelem > 0) run_form(dm, form, precision, a);
    FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    device_checks(fm->ctx, fm->ctx->stream);
  });
}

// bilform_div_grad (src/FEMMBaseModule.jl:1672-1723): block (a, b) of the
// element matrix is mu (g_a . g_b I + g_b g_a^T) summed over the points, i.e.
// the isotropic elasticity block with lambda = 0 and mu = the viscosity; the
// element kernels of bilform_lin_elastic evaluate it.
int fegpu_bilform_div_grad(fegpu_matrix *K, const fegpu_coef *cf, int precision) {
  return guarded([&] {
    FEGPU_REQUIRE(K && cf && cf->data, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    use_device(fm->ctx);
    require_geometry(fm);
    FEGPU_REQUIRE(fm->mdim == 3 && fm->sdim == 3 && dm->ndn == 3,
                  "div_grad: 3-D elements with a three-component field");
    FEGPU_REQUIRE(precision == FEGPU_FP64 || precision == FEGPU_MIXED ||
                      precision == FEGPU_FP64_FAST,
                  "unknown precision");
    // FP64: the colour kernels of the elasticity form (lambda = 0), whose
    // element blocks are the div_grad blocks in another association
    if (precision == FEGPU_FP64) precision = FEGPU_FP64_FAST;
    FEGPU_REQUIRE(cf->ncomp == 1, "div_grad: the viscosity must be a scalar");
    K->unsym = false;
    KArgs a = base_args(K, dm);
    CoefStage st;
    const bool gather = precision == FEGPU_MIXED;
    if (cf->kind == FEGPU_COEF_CONST) {
      a.coef_kind = FEGPU_COEF_CONST;
      a.ncomp = 2;
      a.cconst[0] = 0.0;
      a.cconst[1] = cf->data[0];
    } else if (cf->kind == FEGPU_COEF_PER_ELEMENT) {
      std::vector<double> lame(static_cast<size_t>(2 * fm->nelem));
      for (int64_t e = 0; e < fm->nelem; ++e) {
        lame[2 * e] = 0.0;
        lame[2 * e + 1] = cf->data[e];
      }
      const fegpu_coef pairs{FEGPU_COEF_ISO_LAME, 2, lame.data()};
      stage_coef(fm, &pairs, 2, a, st, !gather);
      FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));  // lame leaves scope
    } else {
      throw Error{FEGPU_ERR_ARG, "div_grad: viscosity constant or per element"};
    }
    if (!gather) zero_matrix(K);
    if (fm->nelem > 0) run_form(dm, F_ELAST_ISO, precision, a);
    FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    device_checks(fm->ctx, fm->ctx->stream);
  });
}

int fegpu_bilform_dot(fegpu_matrix *K, const fegpu_coef *cf, int m, int symmetric, int precision) {
  return guarded([&] {
    FEGPU_REQUIRE(K && cf, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    use_device(fm->ctx);
    require_geometry(fm);
    const int ndn = dm->ndn;
    if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
    else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    (void)precision;  // the dot form is always evaluated in FP64
    KArgs a = base_args(K, dm);
    a.measure_m = m;
    CoefStage st;
    double c[9] = {0};
    if (cf->ncomp == 1) {
      stage_coef(fm, cf, 1, a, st);
      const double sc = cf->kind == FEGPU_COEF_CONST ? cf->data[0] : 1.0;
      if (cf->kind == FEGPU_COEF_CONST) a.coef_kind = FEGPU_COEF_CONST;
      for (int i = 0; i < ndn; ++i) c[i * ndn + i] = sc;
      if (cf->kind == FEGPU_COEF_ISO_LAME) throw Error{FEGPU_ERR_ARG, "dot: bad coefficient kind"};
    } else {
      FEGPU_REQUIRE(cf->ncomp == ndn * ndn, "dot: coefficient must be ndn x ndn");
      FEGPU_REQUIRE(cf->kind == FEGPU_COEF_CONST, "dot: a matrix coefficient must be constant");
      for (int i = 0; i < ndn * ndn; ++i) c[i] = cf->data[i];
      a.coef_kind = FEGPU_COEF_CONST;
    }
    K->unsym = false;
    if (!symmetric)
      for (int i = 0; i < ndn; ++i)
        for (int j = 0; j < ndn; ++j)
          if (c[i * ndn + j] != c[j * ndn + i]) K->unsym = true;
    // element-matrix entry (k,p),(l,q) is N_k N_l c[p][q] (src/FEMMBaseModule.jl:1357-1361);
    // the symmetric assembler keeps its lower triangle by local index and mirrors it.
    for (int i = 0; i < ndn; ++i)
      for (int j = 0; j < ndn; ++j) {
        if (symmetric) {
          a.cab[i * ndn + j] = c[j * ndn + i];
          a.cba[j * ndn + i] = c[j * ndn + i];
          a.cdiag[i * ndn + j] = c[std::max(i, j) * ndn + std::min(i, j)];
        } else {
          a.cab[i * ndn + j] = c[i * ndn + j];
          a.cba[j * ndn + i] = c[j * ndn + i];
          a.cdiag[i * ndn + j] = c[i * ndn + j];
        }
      }
    zero_matrix(K);
    if (fm->nelem > 0) run_colours(dm, F_DOT, FEGPU_FP64, a);
    FEGPU_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    device_checks(fm->ctx, fm->ctx->stream);
  });
}

int fegpu_linform_dot(fegpu_dofmap *dm, const fegpu_coef *f, int m, double *F) {
  return guarded([&] {
    FEGPU_REQUIRE(dm && f && F, "null handle");
    fegpu_femm *fm = dm->femm;
    use_device(fm->ctx);
    require_geometry(fm);
    if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
    else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    FEGPU_REQUIRE(f->ncomp == dm->ndn, "linform_dot: the force must have ndn components");
    FEGPU_REQUIRE(f->kind != FEGPU_COEF_ISO_LAME, "linform_dot: bad coefficient kind");
    KArgs a = base_args(nullptr, dm);
    a.measure_m = m;
    CoefStage st;
    stage_coef(fm, f, dm->ndn, a, st);
    DevBuf vec;
    vec.alloc(sizeof(double) * dm->ndof);
    cudaStream_t s = fm->ctx->stream;
    FEGPU_CUDA(cudaMemsetAsync(vec.p, 0, sizeof(double) * dm->ndof, s));
    a.val = vec.as<double>();
    a.nnz = dm->ndof;
    if (fm->nelem > 0) run_colours(dm, F_LIN, FEGPU_FP64, a);
    device_checks(fm->ctx, s);
    FEGPU_CUDA(cudaMemcpyAsync(F, vec.p, sizeof(double) * dm->ndof, cudaMemcpyDeviceToHost, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
  });
}

int fegpu_matrix_nnz(fegpu_matrix *K, int drop_zeros, int64_t *nnz) {
  return guarded([&] {
    FEGPU_REQUIRE(K && nnz, "null handle");
    use_device(K->dm->femm->ctx);
    *nnz = drop_zeros ? count_nonzeros(K->dm->femm->ctx, K->dm, K->val.as<double>()) : K->dm->nnz;
  });
}

int fegpu_matrix_copy_csc(fegpu_matrix *K, int drop_zeros, int64_t *colptr, int64_t *rowval,
                          double *nzval) {
  return guarded([&] {
    FEGPU_REQUIRE(K && colptr && rowval && nzval, "null handle");
    use_device(K->dm->femm->ctx);
    if (K->unsym) {  // CSC of an unsymmetric matrix: the values read by columns
      DevBuf t;
      t.alloc(sizeof(double) * std::max<int64_t>(K->dm->nnz, 1));
      transpose_values(K->dm, K->val.as<double>(), t.as<double>(), K->dm->femm->ctx->stream);
      copy_csc(K->dm->femm->ctx, K->dm, t.as<double>(), drop_zeros, colptr, rowval, nzval);
    } else {
      copy_csc(K->dm->femm->ctx, K->dm, K->val.as<double>(), drop_zeros, colptr, rowval, nzval);
    }
  });
}

int fegpu_matrix_copy_block_csc(fegpu_matrix *K, int64_t row0, int64_t row1, int64_t col0,
                                int64_t col1, int drop_zeros, int64_t *nnz, int64_t *colptr,
                                int64_t *rowval, double *nzval) {
  return guarded([&] {
    FEGPU_REQUIRE(K && nnz, "null handle");
    const fegpu_dofmap *dm = K->dm;
    FEGPU_REQUIRE(0 <= row0 && row0 <= row1 && row1 <= dm->ndof, "The ff block has too many rows");
    FEGPU_REQUIRE(0 <= col0 && col0 <= col1 && col1 <= dm->ndof,
                  "The ff block has too many columns");
    FEGPU_REQUIRE((colptr == nullptr) == (rowval == nullptr) && (rowval == nullptr) == (nzval == nullptr),
                  "colptr, rowval and nzval: all or none");
    fegpu_context *ctx = dm->femm->ctx;
    use_device(ctx);
    DevBuf t;
    const double *v = K->val.as<double>();
    if (K->unsym) {
      t.alloc(sizeof(double) * std::max<int64_t>(dm->nnz, 1));
      transpose_values(dm, K->val.as<double>(), t.as<double>(), ctx->stream);
      v = t.as<double>();
    }
    *nnz = copy_block_csc(ctx, dm, v, row0, row1, col0, col1, drop_zeros, colptr, rowval,
                          nzval);
  });
}

int fegpu_matrix_copy_values(fegpu_matrix *K, double *nzval) {
  return guarded([&] {
    FEGPU_REQUIRE(K && nzval, "null handle");
    fegpu_context *ctx = K->dm->femm->ctx;
    use_device(ctx);
    FEGPU_CUDA(cudaMemcpyAsync(nzval, K->val.p, sizeof(double) * K->dm->nnz,
                               cudaMemcpyDeviceToHost, ctx->stream));
    FEGPU_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int fegpu_matrix_copy_values_async(fegpu_matrix *K, double *nzval) {
  return guarded([&] {
    FEGPU_REQUIRE(K && nzval, "null handle");
    fegpu_context *ctx = K->dm->femm->ctx;
    use_device(ctx);
    if (!ctx->export_stream)
      FEGPU_CUDA(cudaStreamCreateWithFlags(&ctx->export_stream, cudaStreamNonBlocking));
    if (!K->ready) FEGPU_CUDA(cudaEventCreateWithFlags(&K->ready, cudaEventDisableTiming));
    if (!K->exported) FEGPU_CUDA(cudaEventCreateWithFlags(&K->exported, cudaEventDisableTiming));
    FEGPU_CUDA(cudaEventRecord(K->ready, ctx->stream));
    FEGPU_CUDA(cudaStreamWaitEvent(ctx->export_stream, K->ready, 0));
    FEGPU_CUDA(cudaMemcpyAsync(nzval, K->val.p, sizeof(double) * K->dm->nnz,
                               cudaMemcpyDeviceToHost, ctx->export_stream));
    FEGPU_CUDA(cudaEventRecord(K->exported, ctx->export_stream));
    K->export_pending = true;
  });
}

int fegpu_matrix_wait_export(fegpu_matrix *K) {
  return guarded([&] {
    FEGPU_REQUIRE(K, "null handle");
    use_device(K->dm->femm->ctx);
    if (K->export_pending) FEGPU_CUDA(cudaEventSynchronize(K->exported));
  });
}

int fegpu_matrix_spmv(fegpu_matrix *K, const double *x, double *y) {
  return guarded([&] {
    FEGPU_REQUIRE(K && x && y, "null handle");
    fegpu_context *ctx = K->dm->femm->ctx;
    use_device(ctx);
    const int64_t n = K->dm->ndof;
    DevBuf dx, dy;
    dx.alloc(sizeof(double) * n);
    dy.alloc(sizeof(double) * n);
    FEGPU_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    spmv(K->dm, K->val.as<double>(), dx.as<double>(), dy.as<double>(), ctx->stream);
    FEGPU_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    FEGPU_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
