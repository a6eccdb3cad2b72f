// Reference-order FP64 assembly: plan, row gather and orchestration (the
// element blocks are k_blocks_exact of exact.cuh, instantiated per element
// type in forms_<type>.cu).
//
// The gather sums each CSR entry over the incident elements in element order
// with separately rounded FP64 adds, in two buckets that are the reference's
// S(r, c) and S(c, r) (SysmatAssemblerSparseSymm's assemble! keeps the lower
// triangle by local index; sparse() sums duplicates in input order;
// makematrix! returns S + S' with the diagonal halved,
// src/AssemblyModule.jl:500-583).  An empty bucket starts as -0.0, which the
// first addition replaces exactly, so every stored value is the reference's
// value bit for bit; exact zeros are left out at export (drop_zeros) as the
// reference's sparse `+` leaves them out.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "exact.cuh"
#include "forms_dispatch.cuh"

namespace fegpu {
namespace {

constexpr int kExactGatherWarps = 8;
}  // namespace
int exact_tile(int etype, int form, int npts);
namespace {

// doubles of shared memory per warp: the node's NDN rows, one or two buckets
__host__ __device__ inline int exact_warp_stride(int ndn, int maxdeg, bool sym) {
  return (sym ? 2 : 1) * ndn * maxdeg * ndn;
}

template <int NNE, int NDN, bool SYM>
__device__ __forceinline__ void gather_node_exact(const GArgs &g, int32_t A, double *acc,
                                                  int lane) {
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int BS = NDN * NDN;
  constexpr int NTASK = NNE * NDN;  // (b, j): node of the element, column component
  constexpr int NSLOT = (NTASK + 31) / 32;
  const int cmax = g.maxdeg * NDN;
  const int cols = static_cast<int>(g.nptr[A + 1] - g.nptr[A]) * NDN;
  double *lo = acc;                // S(r, c): local row index >= local column index
  double *up = acc + NDN * cmax;   // S(c, r) (symmetric assembly only)
  for (int c = lane; c < cols; c += 32)
#pragma unroll
    for (int i = 0; i < NDN; ++i) {
      lo[i * cmax + c] = -0.0;
      if (SYM) up[i * cmax + c] = -0.0;
    }
  int tb[NSLOT], tj[NSLOT], trow[NSLOT];
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const int task = min(lane + 32 * s, NTASK - 1);
    tb[s] = task / NDN;
    tj[s] = task - tb[s] * NDN;
    trow[s] = tb[s] * NNE - tb[s] * (tb[s] - 1) / 2 - tb[s];  // pair(b, x) = trow + x, x >= b
  }
  __syncwarp();
  const int64_t qa = g.n2e_ptr[A], qz = g.n2e_ptr[A + 1];
  int self = 0;  // position of A in its own neighbour list (its diagonal)
  if constexpr (NDN == 1) {
    // one row per node (diffusion): element by element (the pipelined loop
    // below made H8 20^3 slower, 0.140 against 0.13 ms)
    for (int64_t q = qa; q < qz; ++q) {
      const int32_t e = g.n2e_elem[q];
      const int a = g.n2e_loc[q];
      const int32_t ch = static_cast<int32_t>(g.chunk);
      const int32_t ce = e / ch;
      const int64_t slot = static_cast<int64_t>(ce % g.ring) * ch + (e - ce * ch);
      const double *kb = g.ke64 + slot * NBLK * BS;
      const uint16_t *pe = g.pos + (static_cast<int64_t>(e) * NNE + a) * NNE;
      if (q == qa) self = pe[a];
      const int rowa = a * NNE - a * (a - 1) / 2 - a;
#pragma unroll
      for (int s = 0; s < NSLOT; ++s) {
        if (lane + 32 * s >= NTASK) break;
        const int b = tb[s];
        const bool upper = a <= b;
        const double v = kb[upper ? rowa + b : trow[s] + a];
        double *dst = (SYM && a < b) ? up : lo;
        dst += pe[b];
        *dst = __dadd_rn(*dst, v);
      }
      __syncwarp();
    }
  } else {
  // One incident element's contributions to this lane's tasks: the block
  // values and their columns, loaded one element ahead of the sums (the
  // loads of element k+1 are in flight while element k's sums run; with the
  // diagonal entries formed apart below, the gather waits on these loads
  // rather than on the FP64 pipe: T10 60^3 29.2 -> 28.4 ms).
  struct Pending {
    double v[NSLOT][NDN];
    int col[NSLOT];
    int a;
  };
  const int32_t ch = static_cast<int32_t>(g.chunk);
  auto fetch = [&](int32_t e, int a, Pending &P) {
    const int32_t ce = e / ch;
    const int64_t slot = static_cast<int64_t>(ce % g.ring) * ch + (e - ce * ch);
    const double *kb = g.ke64 + slot * NBLK * BS;
    const uint16_t *pe = g.pos + (static_cast<int64_t>(e) * NNE + a) * NNE;
    const int rowa = a * NNE - a * (a - 1) / 2 - a;
    P.a = a;
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      P.col[s] = 0;
#pragma unroll
      for (int i = 0; i < NDN; ++i) P.v[s][i] = 0.0;
      if (lane + 32 * s < NTASK) {
        const int b = tb[s], j = tj[s];
        const bool upper = a <= b;  // block (a, b) stored; else (b, a), transposed
        const double *blk = kb + (upper ? rowa + b : trow[s] + a) * BS + (upper ? j : j * NDN);
        const int step = upper ? NDN : 1;
        P.col[s] = pe[b] * NDN + j;
#pragma unroll
        for (int i = 0; i < NDN; ++i) P.v[s][i] = blk[i * step];
      }
    }
  };
  // the incident elements in element order, 32 at a time (one per lane)
  for (int64_t q0 = qa; q0 < qz; q0 += 32) {
    const int m = static_cast<int>(qz - q0 < 32 ? qz - q0 : 32);
    const int32_t my_e = lane < m ? g.n2e_elem[q0 + lane] : 0;
    const int my_a = lane < m ? g.n2e_loc[q0 + lane] : 0;
    Pending cur, nxt;
    {
      const int32_t e0 = __shfl_sync(0xffffffffu, my_e, 0);
      const int a0 = __shfl_sync(0xffffffffu, my_a, 0);
      fetch(e0, a0, cur);
      if (q0 == qa) self = g.pos[(static_cast<int64_t>(e0) * NNE + a0) * NNE + a0];
    }
    for (int k = 0; k < m; ++k) {
      const int32_t en = __shfl_sync(0xffffffffu, my_e, k + 1 < m ? k + 1 : k);
      const int an = __shfl_sync(0xffffffffu, my_a, k + 1 < m ? k + 1 : k);
      if (k + 1 < m) fetch(en, an, nxt);
      const int a = cur.a;
#pragma unroll
      for (int s = 0; s < NSLOT; ++s) {
        if (lane + 32 * s >= NTASK) break;
        const int b = tb[s], j = tj[s];
#pragma unroll
        for (int i = 0; i < NDN; ++i) {
          double *dst = lo;
          if (SYM && a * NDN + i < b * NDN + j) dst = up;
          dst += i * cmax + cur.col[s];
          *dst = __dadd_rn(*dst, cur.v[s][i]);
        }
      }
      __syncwarp();
      cur = nxt;
    }
  }
  }
  int64_t base[NDN];
#pragma unroll
  for (int i = 0; i < NDN; ++i) base[i] = g.rowptr[g.dof[A * NDN + i]];
  // S + S', and (S + S) / 2 on the diagonal.  With three rows per node the
  // diagonal entries are formed apart by the first three lanes (a select
  // between the two forms issues all three FP64 operations for every value:
  // T10 60^3 29.4 -> 29.3 ms, H20 40^3 30.1 -> 29.6 ms); with one row per
  // node (diffusion) the select stays: H8 20^3 showed no difference beyond
  // its run-to-run spread.
  constexpr bool APART = SYM && NDN == 3;
  for (int c = lane; c < cols; c += 32) {
    const int64_t off = g.colperm ? g.colperm[g.cpoff[A] * NDN + c] : c;
#pragma unroll
    for (int i = 0; i < NDN; ++i) {
      const double l = lo[i * cmax + c];
      double v = l;
      if (APART) {
        if (c == self * NDN + i) continue;
        v = __dadd_rn(l, up[i * cmax + c]);
      } else if (SYM) {
        v = (c == self * NDN + i) ? __dmul_rn(__dadd_rn(l, l), 0.5) : __dadd_rn(l, up[i * cmax + c]);
      }
      if (dcheck(g.check, CK_GATHER, base[i] + off, g.nnz)) g.val[base[i] + off] = v;
    }
  }
  if (APART && lane < NDN) {
    const int i = lane, c = self * NDN + i;
    int64_t bi = base[0];  // base[i] without indexing the array by a lane value
#pragma unroll
    for (int k = 1; k < NDN; ++k) bi = i == k ? base[k] : bi;
    const int64_t off = g.colperm ? g.colperm[g.cpoff[A] * NDN + c] : c;
    const double l = lo[i * cmax + c];
    const double v = __dmul_rn(__dadd_rn(l, l), 0.5);
    if (dcheck(g.check, CK_GATHER, bi + off, g.nnz)) g.val[bi + off] = v;
  }
  __syncwarp();
}

template <int NNE, int NDN, bool SYM>
__global__ void __launch_bounds__(kExactGatherWarps * 32) k_gather_exact(const GArgs g) {
  extern __shared__ __align__(16) double xsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *acc = xsm + static_cast<size_t>(warp) * exact_warp_stride(NDN, g.maxdeg, SYM);
  for (int64_t t = g.n0 + static_cast<int64_t>(blockIdx.x) * kExactGatherWarps + warp; t < g.n1;
       t += static_cast<int64_t>(gridDim.x) * kExactGatherWarps)
    gather_node_exact<NNE, NDN, SYM>(g, g.nodes[t], acc, lane);
}

template <int NNE, int NDN, bool SYM>
int launch_gx(const GArgs &g, int num_sms, cudaStream_t s) {
  const int64_t n = g.n1 - g.n0;
  if (n <= 0) return 0;
  const size_t smem =
      sizeof(double) * static_cast<size_t>(exact_warp_stride(NDN, g.maxdeg, SYM)) * kExactGatherWarps;
  FEGPU_REQUIRE(smem <= 227 * 1024, "node degree too large for the row gather");
  auto kern = k_gather_exact<NNE, NDN, SYM>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kExactGatherWarps * 32,
                                                           smem));
  per_sm = std::max(per_sm, 1);
  const int64_t ctas = (n + kExactGatherWarps - 1) / kExactGatherWarps;
  const int grid = static_cast<int>(std::min<int64_t>(ctas, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kExactGatherWarps * 32, smem, s>>>(g);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

template <int NNE>
int launch_gx_nne(int ndn, bool sym, const GArgs &g, int num_sms, cudaStream_t s) {
  if (ndn == 1) return sym ? launch_gx<NNE, 1, true>(g, num_sms, s) : launch_gx<NNE, 1, false>(g, num_sms, s);
  return sym ? launch_gx<NNE, 3, true>(g, num_sms, s) : launch_gx<NNE, 3, false>(g, num_sms, s);
}

int launch_gather_exact(int etype, int ndn, bool sym, const GArgs &g, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_Q4: return launch_gx_nne<4>(ndn, sym, g, num_sms, s);
    case FEGPU_H8: return launch_gx_nne<8>(ndn, sym, g, num_sms, s);
    case FEGPU_H20: return launch_gx_nne<20>(ndn, sym, g, num_sms, s);
    case FEGPU_T4: return launch_gx_nne<4>(ndn, sym, g, num_sms, s);
    case FEGPU_T10: return launch_gx_nne<10>(ndn, sym, g, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

int launch_exact(int etype, int form, const KArgs &a, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_Q4: return launch_exact_q4(form, a, num_sms, s);
    case FEGPU_H8: return launch_exact_h8(form, a, num_sms, s);
    case FEGPU_H20: return launch_exact_h20(form, a, num_sms, s);
    case FEGPU_T4: return launch_exact_t4(form, a, num_sms, s);
    case FEGPU_T10: return launch_exact_t10(form, a, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

// CTAs of the block kernel resident per SM (shared memory; registers allow
// four of 256 threads)
int exact_ctas_per_sm(int etype, int form, int npts, int te) {
  const size_t smem = exact_layout(nodes_per_elem(etype), manif_dim(etype), npts, te, form).total;
  return static_cast<int>(std::max<size_t>(1, std::min<size_t>(4, (228 * 1024) / (smem + 1024))));
}

// Chunks of four waves of element tiles over the GPU (at least 256
// elements): the block kernel is FP64-bound, and a chunk of fewer tiles than
// CTA slots leaves SMs idle while it runs (one 16 MB chunk of T10 blocks, 163
// tiles on 304 slots: FP64 pipe 79 % busy on the active SMs, 43 % over the
// launch).  The ring of span + 2 chunks then exceeds the L2, which this
// compute-bound path does not need.
void build_exact_plan(fegpu_dofmap *dm, int block_values, int form) {
  fegpu_femm *fm = dm->femm;
  cudaStream_t s = fm->ctx->stream;
  const int64_t E = fm->nelem;
  build_node_lists(dm, nullptr);
  const int te = exact_tile(fm->etype, form, fm->npts);
  const int64_t slots =
      static_cast<int64_t>(fm->ctx->num_sms) * exact_ctas_per_sm(fm->etype, form, fm->npts, te);
  dm->x_chunk = std::max<int64_t>(256, 4 * slots * te);
  dm->x_chunk = std::min<int64_t>(dm->x_chunk, std::max<int64_t>(E, 1));
  std::vector<int32_t> order;
  plan_chunks(dm, dm->x_chunk, dm->x_chunk_nodes, order, dm->x_span, dm->x_ring);
  dm->x_gnodes.alloc(sizeof(int32_t) * std::max<size_t>(order.size(), 1));
  if (!order.empty())
    FEGPU_CUDA(cudaMemcpyAsync(dm->x_gnodes.p, order.data(), sizeof(int32_t) * order.size(),
                               cudaMemcpyHostToDevice, s));
  dm->x_ke.alloc(sizeof(double) * static_cast<size_t>(dm->x_ring) * dm->x_chunk * block_values);
  FEGPU_CUDA(cudaStreamSynchronize(s));
  dm->exact_ready = true;
}

}  // namespace

// elements per tile of the reference-order block kernel: what fits the
// shared-memory budget of one of its CTAs (below), at least one element
int exact_tile(int etype, int form, int npts) {
  const int nne = nodes_per_elem(etype), mdim = manif_dim(etype);
  const size_t one = exact_layout(nne, mdim, npts, 1, form).total;
  const size_t two = exact_layout(nne, mdim, npts, 2, form).total;
  const size_t per = two - one;
  const size_t fixed = one - per;
  // two CTAs per SM, or one for elements whose blocks take more than 24 KB of
  // shared memory each.  T10 and H20 elasticity, whose point sums run on the
  // integer units, take three CTAs per SM instead (more warps to cover the
  // integer chains' latency): 16 T10 elements per tile (T10 60^3: 30.3
  // against 31.4 ms with 26 and two CTAs; 14, 15, 17, 18 and 20 per tile
  // slower), one H20 element (H20 40^3: 31.2 against 40.0 ms with three and
  // one CTA)
  const bool elast = form == F_ELAST_ISO || form == F_ELAST_GEN;
  size_t budget = per > 24 * 1024 ? 220 * 1024 : 110 * 1024;
  if (elast && etype == FEGPU_T10) budget = 68 * 1024;
  if (elast && etype == FEGPU_H20) budget = 72 * 1024;
  int te = static_cast<int>((budget - std::min(budget, fixed)) / std::max<size_t>(per, 1));
  te = std::max(1, std::min(te, 64));
  // FEGPU_EXACT_TILE fixes the elements per tile (tuning; capped by the
  // shared memory of one CTA)
  if (const char *env = std::getenv("FEGPU_EXACT_TILE")) {
    const int v = std::atoi(env);
    if (v > 0) {
      te = v;
      while (te > 1 && exact_layout(nne, mdim, npts, te, form).total > 227 * 1024) --te;
    }
  }
  FEGPU_REQUIRE(exact_layout(nne, mdim, npts, te, form).total <= 227 * 1024,
                "quadrature rule too large for the reference-order element kernel");
  return te;
}

// Element blocks of chunk c on the side stream, the gather of the nodes that
// chunk completes on the context stream (as the mixed path runs).
void run_exact(fegpu_dofmap *dm, int form, KArgs &a, bool symmetric) {
  fegpu_femm *fm = dm->femm;
  fegpu_context *ctx = fm->ctx;
  const int nne = fm->nne, ndn = dm->ndn;
  const int bs = ndn * ndn, nblk = nne * (nne + 1) / 2;
  // the plan depends on the tile (chunks are waves of tiles): rebuilt when
  // another form or rule changes it
  const int te = exact_tile(fm->etype, form, fm->npts);
  if (!dm->exact_ready || dm->x_tile != te) {
    build_exact_plan(dm, nblk * bs, form);
    dm->x_tile = te;
  }
  a.conn = fm->conn_orig.as<int32_t>();
  a.te = te;
  GArgs g;
  std::memset(&g, 0, sizeof(g));
  g.n2e_ptr = dm->n2e_ptr.as<int64_t>();
  g.n2e_elem = dm->n2e_elem.as<int32_t>();
  g.n2e_loc = dm->n2e_loc.as<uint8_t>();
  g.nodes = dm->x_gnodes.as<int32_t>();
  g.nptr = dm->nptr.as<int64_t>();
  g.pos = dm->pos_orig.as<uint16_t>();
  g.ke64 = dm->x_ke.as<double>();
  g.chunk = dm->x_chunk;
  g.ring = dm->x_ring;
  g.dof = dm->dof.as<int32_t>();
  g.rowptr = dm->rowptr.as<int64_t>();
  g.colperm = dm->contiguous ? nullptr : dm->colperm.as<int32_t>();
  g.cpoff = dm->contiguous ? nullptr : dm->cpoff.as<int64_t>();
  g.val = a.val;
  g.maxdeg = dm->maxdeg;
  g.check = a.check;
  g.nnz = dm->nnz;
  const int64_t nch = static_cast<int64_t>(dm->x_chunk_nodes.size()) - 1;
  cudaStream_t s0 = ctx->stream;
  if (!ctx->side) FEGPU_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
  while (static_cast<int>(ctx->ev_blocks.size()) < dm->x_ring) {
    cudaEvent_t e1, e2;
    FEGPU_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
    FEGPU_CUDA(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
    ctx->ev_blocks.push_back(e1);
    ctx->ev_gather.push_back(e2);
  }
  if (ctx->timing) FEGPU_CUDA(cudaEventRecord(ctx->ev0, s0));
  FEGPU_CUDA(cudaEventRecord(ctx->ev_gather[0], s0));  // work before this call
  FEGPU_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_gather[0], 0));
  for (int64_t c = 0; c < nch; ++c) {
    const int slot = static_cast<int>(c % dm->x_ring);
    if (c >= dm->x_ring) {
      const int64_t reader = c - dm->x_ring + dm->x_span;  // last gather reading the slot
      FEGPU_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_gather[reader % dm->x_ring], 0));
    }
    a.e0 = c * dm->x_chunk;
    a.e1 = std::min(fm->nelem, (c + 1) * dm->x_chunk);
    a.ke64 = dm->x_ke.as<double>() + slot * dm->x_chunk * nblk * bs;
    ctx->launches += launch_exact(fm->etype, form, a, ctx->num_sms, ctx->side);
    FEGPU_CUDA(cudaEventRecord(ctx->ev_blocks[slot], ctx->side));
    FEGPU_CUDA(cudaStreamWaitEvent(s0, ctx->ev_blocks[slot], 0));
    g.n0 = dm->x_chunk_nodes[c];
    g.n1 = dm->x_chunk_nodes[c + 1];
    ctx->launches += launch_gather_exact(fm->etype, ndn, symmetric, g, ctx->num_sms, s0);
    FEGPU_CUDA(cudaEventRecord(ctx->ev_gather[slot], s0));
  }
  if (ctx->timing) {
    FEGPU_CUDA(cudaEventRecord(ctx->ev1, s0));
    FEGPU_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    FEGPU_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->kernel_ms += ms;
  }
}

}  // namespace fegpu

// ---- device self-test of the integer-unit addition ----------------------
namespace fegpu {
namespace {

__device__ __forceinline__ uint64_t st_mix(uint64_t z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double st_make(uint64_t sign, uint64_t ex, uint64_t frac) {
  return sf_double((sign << 63) | (ex << 52) | (frac & 0x000fffffffffffffull));
}

// operand pairs of four kinds (uniform bit patterns; exponent differences
// 0..70; near-cancellations; ties to even), sf_add against __dadd_rn
__global__ void k_selftest_soft_add(uint64_t seed, int64_t n, unsigned long long *bad,
                                    unsigned long long *first) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t r1 = st_mix(seed + 4 * static_cast<uint64_t>(i));
    const uint64_t r2 = st_mix(seed + 4 * static_cast<uint64_t>(i) + 1);
    const uint64_t r3 = st_mix(seed + 4 * static_cast<uint64_t>(i) + 2);
    double x, y;
    switch (i & 3) {
      case 0:
        x = sf_double(r1);
        y = sf_double(r2);
        break;
      case 1: {
        const uint64_t ex = 1 + r3 % 2046, d = (r3 >> 20) % 71;
        x = st_make(r1 >> 63, ex, r1);
        y = st_make(r2 >> 63, ex > d ? ex - d : 1, r2);
        break;
      }
      case 2: {
        x = st_make(r1 >> 63, 1 + r3 % 2046, r1);
        const int64_t k = static_cast<int64_t>((r3 >> 20) % 9) - 4;
        y = -sf_double(sf_bits(x) + static_cast<uint64_t>(k));
        break;
      }
      default: {
        const uint64_t ex = 60 + r3 % 1900, d = 1 + (r3 >> 20) % 56;
        x = st_make(r1 >> 63, ex, r1 & ~0xffull);
        y = st_make(r2 >> 63, ex - d,
                    (r2 & 0x000ffffffffff000ull) | (1ull << ((r3 >> 40) % 12)));
        break;
      }
    }
    const double s = sf_add(x, y), h = __dadd_rn(x, y);
    const bool same = sf_bits(s) == sf_bits(h) || (isnan(s) && isnan(h));
    if (!same) {
      atomicAdd(bad, 1ull);
      atomicMin(first, static_cast<unsigned long long>(i));
    }
  }
}

}  // namespace
}  // namespace fegpu

extern "C" int fegpu_selftest_soft_add(fegpu_context *ctx, int64_t n, uint64_t seed,
                                       int64_t *mismatches, int64_t *first) {
  using namespace fegpu;
  try {
    FEGPU_REQUIRE(ctx && mismatches && n >= 0, "null handle or negative count");
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    DevBuf d;
    d.alloc(2 * sizeof(unsigned long long));
    const unsigned long long init[2] = {0ull, ~0ull};
    FEGPU_CUDA(cudaMemcpyAsync(d.p, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    auto *p = d.as<unsigned long long>();
    if (n > 0) {
      const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, 8 * ctx->num_sms));
      k_selftest_soft_add<<<grid, 256, 0, ctx->stream>>>(seed, n, p, p + 1);
      FEGPU_CUDA(cudaGetLastError());
      ctx->launches += 1;
    }
    unsigned long long out[2];
    FEGPU_CUDA(cudaMemcpyAsync(out, d.p, sizeof(out), cudaMemcpyDeviceToHost, ctx->stream));
    FEGPU_CUDA(cudaStreamSynchronize(ctx->stream));
    *mismatches = static_cast<int64_t>(out[0]);
    if (first) *first = out[0] ? static_cast<int64_t>(out[1]) : -1;
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  }
}
