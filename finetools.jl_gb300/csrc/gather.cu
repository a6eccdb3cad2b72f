// Mixed-precision assembly by row gather.
//
// On this GPU an FP64 add or an f32->f64 conversion runs at ~0.5 T/s, so one
// FP64 add per element contribution (230 M for an H20 40^3 block, 1.17 G for
// a T10 60^3 block) costs more than streaming the whole CSR through HBM.  The
// mixed path therefore never adds into the global matrix element by element:
//   1. element phase: the FP32 node-pair blocks of a chunk of elements (in
//      element order) go to a ring buffer that stays L2-resident;
//   2. gather phase: one warp per node accumulates the blocks of its incident
//      elements (in element order: deterministic) into its rows with
//      compensated FP32 sums (two-sum, ~48-bit significand), converts each
//      entry to FP64 with integer operations only, and writes every CSR value
//      of the node's rows exactly once (plain coalesced stores, no RMW).
// A node is gathered right after the chunk holding its last element, so the
// ring needs only (span of a node's elements in chunks) + 1 chunks.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

constexpr int kWarpsPerCta = 8;

// floats of shared memory per warp: hi and lo accumulators of the node's
// NDN rows, rounded up to a multiple of four
__host__ __device__ inline int gather_warp_stride(int ndn, int maxdeg) {
  const int n = 2 * ndn * maxdeg * ndn;
  return (n + 3) / 4 * 4;
}

// Error-free accumulation of v into (h, l): two-sum (Knuth).
__device__ __forceinline__ void two_sum_acc(float &h, float &l, float v) {
  const float s = __fadd_rn(h, v);
  const float bb = __fsub_rn(s, h);
  const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  h = s;
  l = __fadd_rn(l, err);
}

// (h + l) rounded to FP64 using integer arithmetic only (no FP64 pipe).
// h, l is first renormalised so that |l| <= ulp(h)/2; the exact sum is then
// formed as a 64-bit fixed-point integer aligned 37 bits below h's leading
// bit (bits of l further down are truncated: < 2^-60 relative), normalised
// and rounded to 53 bits (nearest, ties to even).
__device__ __forceinline__ double ff_to_double(float h, float l) {
  const float s = __fadd_rn(h, l);
  l = __fsub_rn(l, __fsub_rn(s, h));
  h = s;
  const uint32_t hb = __float_as_uint(h);
  const uint32_t eh = (hb >> 23) & 0xffu;
  if (eh == 0u) {
    // zero (or an FP32-subnormal sum, below 1.2e-38): signed zero
    return __longlong_as_double(static_cast<long long>(static_cast<uint64_t>(hb >> 31) << 63));
  }
  if (eh == 0xffu) {  // inf / nan keep their class
    const uint64_t nanbit = (hb & 0x7fffffu) ? (1ull << 51) : 0ull;
    return __longlong_as_double(static_cast<long long>(
        (static_cast<uint64_t>(hb >> 31) << 63) | (0x7ffull << 52) | nanbit));
  }
  const uint64_t mh = static_cast<uint64_t>((hb & 0x7fffffu) | 0x800000u);
  uint64_t H = mh << 37;
  const uint32_t lb = __float_as_uint(l);
  const uint32_t el = (lb >> 23) & 0xffu;
  if (el != 0u && el != 0xffu) {
    const uint64_t ml = static_cast<uint64_t>((lb & 0x7fffffu) | 0x800000u);
    const int d = static_cast<int>(eh) - static_cast<int>(el);
    uint64_t L = 0;
    if (d <= 37) L = ml << (37 - d);
    else if (d < 37 + 24) L = ml >> (d - 37);
    if ((lb >> 31) == (hb >> 31)) H += L;
    else H -= L;
  }
  const int p = 63 - __clzll(static_cast<long long>(H));  // 59..61
  const int drop = p - 52;
  uint64_t mant = H >> drop;
  const uint64_t rem = H & ((1ull << drop) - 1ull);
  const uint64_t half = 1ull << (drop - 1);
  if (rem > half || (rem == half && (mant & 1ull))) ++mant;
  int p2 = p;
  if (mant >> 53) {
    mant >>= 1;
    ++p2;
  }
  const uint64_t E = static_cast<uint64_t>(p2 + static_cast<int>(eh) + 836);
  const uint64_t bits = (static_cast<uint64_t>(hb >> 31) << 63) | (E << 52) |
                        (mant & ((1ull << 52) - 1ull));
  return __longlong_as_double(static_cast<long long>(bits));
}

template <int NNE, int NDN, bool INLINE_SLOT>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_gather(const GArgs g) {
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int BS = NDN * NDN;
  extern __shared__ __align__(16) float gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cmax = g.maxdeg * NDN;
  // per-warp region padded to a multiple of 4 floats: every warp's region
  // starts on a 16-byte boundary (the zeroing below stores float4)
  const int wstride = gather_warp_stride(NDN, g.maxdeg);
  float *hi = gsm + static_cast<size_t>(warp) * wstride;
  float *lo = hi + NDN * cmax;
  for (int64_t t = g.n0 + static_cast<int64_t>(blockIdx.x) * kWarpsPerCta + warp; t < g.n1;
       t += static_cast<int64_t>(gridDim.x) * kWarpsPerCta) {
    const int32_t A = g.nodes[t];
    const int cols = static_cast<int>(g.nptr[A + 1] - g.nptr[A]) * NDN;
    {
      float4 *z = reinterpret_cast<float4 *>(hi);  // hi and lo are contiguous
      const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int c = lane; c < (2 * NDN * cmax) / 4; c += 32) z[c] = zero;
      for (int c = ((2 * NDN * cmax) / 4) * 4 + lane; c < 2 * NDN * cmax; c += 32) hi[c] = 0.f;
    }
    __syncwarp();
    for (int64_t q = g.n2e_ptr[A]; q < g.n2e_ptr[A + 1]; ++q) {
      const int64_t e = g.n2e_elem[q];
      const int a = g.n2e_loc[q];
      int64_t slot;
      if constexpr (INLINE_SLOT) {
        const int32_t e32 = static_cast<int32_t>(e), ch = static_cast<int32_t>(g.chunk);
        const int32_t ce = e32 / ch;
        slot = static_cast<int64_t>(ce % g.ring) * ch + (e32 - ce * ch);
      } else {
        slot = g.n2e_slot[q];
      }
      const float *kb = g.ke + slot * NBLK * BS;
      const uint16_t *pe = g.pos + (e * NNE + a) * NNE;
      for (int task = lane; task < NNE * NDN; task += 32) {
        const int b = task / NDN, j = task - (task / NDN) * NDN;
        const int col = pe[b] * NDN + j;
        if (a <= b) {
          const float *blk = kb + (a * NNE - a * (a - 1) / 2 + (b - a)) * BS;
#pragma unroll
          for (int i = 0; i < NDN; ++i) two_sum_acc(hi[i * cmax + col], lo[i * cmax + col], blk[i * NDN + j]);
        } else {
          const float *blk = kb + (b * NNE - b * (b - 1) / 2 + (a - b)) * BS;
#pragma unroll
          for (int i = 0; i < NDN; ++i) two_sum_acc(hi[i * cmax + col], lo[i * cmax + col], blk[j * NDN + i]);
        }
      }
      __syncwarp();
    }
#pragma unroll
    for (int i = 0; i < NDN; ++i) {
      const int64_t base = g.rowptr[g.dof[A * NDN + i]];
      for (int c = lane; c < cols; c += 32) {
        const int64_t off = g.colperm ? g.colperm[g.cpoff[A] * NDN + c] : c;
        g.val[base + off] = ff_to_double(hi[i * cmax + c], lo[i * cmax + c]);
      }
    }
    __syncwarp();
  }
}

template <int NNE, int NDN, bool INLINE_SLOT = false>
int launch_t(const GArgs &g, int num_sms, cudaStream_t s) {
  const int64_t n = g.n1 - g.n0;
  if (n <= 0) return 0;
  const size_t smem = sizeof(float) * static_cast<size_t>(gather_warp_stride(NDN, g.maxdeg)) * kWarpsPerCta;
  FEGPU_REQUIRE(smem <= 227 * 1024, "node degree too large for the row gather");
  auto kern = k_gather<NNE, NDN, INLINE_SLOT>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpsPerCta * 32, smem));
  per_sm = std::max(per_sm, 1);
  const int64_t ctas = (n + kWarpsPerCta - 1) / kWarpsPerCta;
  const int grid = static_cast<int>(std::min<int64_t>(ctas, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kWarpsPerCta * 32, smem, s>>>(g);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

__global__ void k_unsort_pos(const uint16_t *pos_sorted, const int32_t *perm, int64_t nelem,
                             int nn2, uint16_t *pos_orig) {
  const int64_t total = nelem * nn2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t es = t / nn2;
    pos_orig[static_cast<int64_t>(perm[es]) * nn2 + (t - es * nn2)] = pos_sorted[t];
  }
}

}  // namespace

int launch_gather(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_H8: return ndn == 1 ? launch_t<8, 1>(g, num_sms, s) : launch_t<8, 3>(g, num_sms, s);
    case FEGPU_H20: return ndn == 1 ? launch_t<20, 1>(g, num_sms, s) : launch_t<20, 3>(g, num_sms, s);
    case FEGPU_T4: return ndn == 1 ? launch_t<4, 1>(g, num_sms, s) : launch_t<4, 3>(g, num_sms, s);
    case FEGPU_T10: return ndn == 1 ? launch_t<10, 1>(g, num_sms, s) : launch_t<10, 3>(g, num_sms, s);
    case FEGPU_Q4: return ndn == 1 ? launch_t<4, 1>(g, num_sms, s) : launch_t<4, 3>(g, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

int launch_gather_inline_slot(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_H8: return ndn == 1 ? launch_t<8, 1, true>(g, num_sms, s) : launch_t<8, 3, true>(g, num_sms, s);
    case FEGPU_H20: return ndn == 1 ? launch_t<20, 1, true>(g, num_sms, s) : launch_t<20, 3, true>(g, num_sms, s);
    case FEGPU_T4: return ndn == 1 ? launch_t<4, 1, true>(g, num_sms, s) : launch_t<4, 3, true>(g, num_sms, s);
    case FEGPU_T10: return ndn == 1 ? launch_t<10, 1, true>(g, num_sms, s) : launch_t<10, 3, true>(g, num_sms, s);
    case FEGPU_Q4: return ndn == 1 ? launch_t<4, 1, true>(g, num_sms, s) : launch_t<4, 3, true>(g, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

// Node -> element lists, chunk plan and element-order slot maps.
void build_gather_plan(fegpu_dofmap *dm, int block_values) {
  fegpu_femm *fm = dm->femm;
  fegpu_context *ctx = fm->ctx;
  cudaStream_t s = ctx->stream;
  const int nne = fm->nne;
  const int64_t N = fm->nnodes, E = fm->nelem;
  const std::vector<int32_t> &c0 = fm->conn_host;
  // chunk: ~24 MB of FP32 blocks, at least 1024 elements
  const int64_t per_elem = static_cast<int64_t>(block_values) * 4;
  dm->chunk = std::max<int64_t>(1024, (24ll << 20) / std::max<int64_t>(per_elem, 1));
  dm->chunk = std::min<int64_t>(dm->chunk, std::max<int64_t>(E, 1));
  const int64_t nch = (E + dm->chunk - 1) / dm->chunk;
  // node -> elements (increasing) with local indices
  std::vector<int64_t> ptr(N + 1, 0);
  for (int64_t i = 0; i < E * nne; ++i) ptr[c0[i] + 1]++;
  for (int64_t n = 0; n < N; ++n) ptr[n + 1] += ptr[n];
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  std::vector<int32_t> elem(static_cast<size_t>(E) * nne);
  std::vector<uint8_t> loc(static_cast<size_t>(E) * nne);
  for (int64_t e = 0; e < E; ++e)
    for (int a = 0; a < nne; ++a) {
      const int64_t q = fill[c0[e * nne + a]]++;
      elem[q] = static_cast<int32_t>(e);
      loc[q] = static_cast<uint8_t>(a);
    }
  std::vector<int32_t> slot(elem.size());
  // a node is gathered after the chunk of its last element
  dm->node_first.assign(N, -1);
  dm->node_last.assign(N, -1);
  for (int64_t n = 0; n < N; ++n)
    if (ptr[n + 1] > ptr[n]) {
      dm->node_first[n] = elem[ptr[n]];
      dm->node_last[n] = elem[ptr[n + 1] - 1];
    }
  std::vector<int64_t> cnt(nch + 1, 0);
  int64_t span = 0;
  for (int64_t n = 0; n < N; ++n) {
    if (ptr[n + 1] == ptr[n]) continue;
    const int64_t cmin = elem[ptr[n]] / dm->chunk, cmaxc = elem[ptr[n + 1] - 1] / dm->chunk;
    span = std::max(span, cmaxc - cmin);
    cnt[cmaxc + 1]++;
  }
  for (int64_t c = 0; c < nch; ++c) cnt[c + 1] += cnt[c];
  dm->chunk_nodes = cnt;
  std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
  std::vector<int32_t> order(cnt[nch]);
  for (int64_t n = 0; n < N; ++n) {
    if (ptr[n + 1] == ptr[n]) continue;
    order[at[elem[ptr[n + 1] - 1] / dm->chunk]++] = static_cast<int32_t>(n);
  }
  dm->ring = static_cast<int>(std::min<int64_t>(span + 1, nch));
  for (size_t q = 0; q < elem.size(); ++q) {
    const int64_t ce = elem[q] / dm->chunk;
    slot[q] = static_cast<int32_t>((ce % dm->ring) * dm->chunk + (elem[q] - ce * dm->chunk));
  }
  dm->n2e_slot.alloc(sizeof(int32_t) * std::max<size_t>(slot.size(), 1));
  if (!slot.empty())
    FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_slot.p, slot.data(), sizeof(int32_t) * slot.size(),
                               cudaMemcpyHostToDevice, s));
  dm->n2e_ptr.alloc(sizeof(int64_t) * (N + 1));
  dm->n2e_elem.alloc(sizeof(int32_t) * elem.size());
  dm->n2e_loc.alloc(loc.size());
  dm->gnodes.alloc(sizeof(int32_t) * std::max<size_t>(order.size(), 1));
  FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_ptr.p, ptr.data(), sizeof(int64_t) * (N + 1),
                             cudaMemcpyHostToDevice, s));
  FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_elem.p, elem.data(), sizeof(int32_t) * elem.size(),
                             cudaMemcpyHostToDevice, s));
  FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_loc.p, loc.data(), loc.size(), cudaMemcpyHostToDevice, s));
  if (!order.empty())
    FEGPU_CUDA(cudaMemcpyAsync(dm->gnodes.p, order.data(), sizeof(int32_t) * order.size(),
                               cudaMemcpyHostToDevice, s));
  dm->ke.alloc(sizeof(float) * static_cast<size_t>(dm->ring) * dm->chunk * block_values);
  const int64_t np = E * nne * nne;
  dm->pos_orig.alloc(sizeof(uint16_t) * std::max<int64_t>(np, 1));
  if (np > 0) {
    const int grid = static_cast<int>(std::min<int64_t>((np + 255) / 256, 1 << 20));
    k_unsort_pos<<<grid, 256, 0, s>>>(dm->pos.as<uint16_t>(), fm->perm.as<int32_t>(), E, nne * nne,
                                      dm->pos_orig.as<uint16_t>());
    FEGPU_CUDA(cudaGetLastError());
    ctx->launches++;
  }
  FEGPU_CUDA(cudaStreamSynchronize(s));
  dm->gather_ready = true;
}

}  // namespace fegpu
