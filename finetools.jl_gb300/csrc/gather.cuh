// Row gather of the mixed-precision path: per-node accumulation of element
// blocks with compensated FP32 sums and integer-only rounding to FP64.
// Shared by the single-matrix gather kernel (gather.cu) and the batch kernel
// (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fegpu_internal.h"

namespace fegpu {

constexpr int kGatherWarps = 8;

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
// and rounded to 53 bits (nearest, ties to even).  General case; the row
// gather uses ff_to_double below, which calls this one for the rare inputs
// outside its fast path.
static __device__ __noinline__ double ff_to_double_exact(float h, float l) {
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


// (h + l) as an FP64 value, integer arithmetic only, for the common case of
// a normal h and |l| <= ulp(h)/2 (after renormalisation): h's 24-bit
// mantissa is placed in the 53-bit mantissa of the result and l is added at
// its position, 2^(29 - d) units of the result's last place with d the
// exponent difference (d >= 24); bits of l below the result's last place are
// truncated (faithful: error < 1 ulp of FP64).  Other inputs (zero,
// subnormal, inf/nan, |l| not small against h) take ff_to_double_exact.
__device__ __forceinline__ double ff_to_double(float h, float l) {
  const float s = __fadd_rn(h, l);
  l = __fsub_rn(l, __fsub_rn(s, h));
  h = s;
  const uint32_t hb = __float_as_uint(h), lb = __float_as_uint(l);
  const uint32_t eh = (hb >> 23) & 0xffu, el = (lb >> 23) & 0xffu;
  const int d = static_cast<int>(eh) - static_cast<int>(el);
  if (eh == 0u || eh == 0xffu || (el != 0u && d < 24)) return ff_to_double_exact(h, l);
  uint64_t M = static_cast<uint64_t>((hb & 0x7fffffu) | 0x800000u) << 29;
  if (el != 0u && d < 61) {
    const uint32_t ml = (lb & 0x7fffffu) | 0x800000u;
    const uint32_t c = d <= 29 ? (ml << (29 - d)) : (ml >> (d - 29));
    M = ((lb ^ hb) >> 31) ? M - c : M + c;
  }
  uint64_t E = static_cast<uint64_t>(eh) + 896u;
  if (M < (1ull << 52)) {  // h a power of two, l of the other sign
    M <<= 1;
    E -= 1u;
  }
  return __longlong_as_double(static_cast<long long>(
      (static_cast<uint64_t>(hb >> 31) << 63) | (E << 52) | (M & ((1ull << 52) - 1ull))));
}

// One warp gathers the rows of node A: accumulators hi/lo (NDN x cmax floats
// each, in the warp's shared region), blocks of the incident elements in
// element order, then one FP64 store per CSR value of the node's rows.
// L2ONLY reads the blocks with ld.global.cg (no L1 allocation): required when
// the blocks were written earlier in the same launch by other CTAs.
template <int NNE, int NDN, bool INLINE_SLOT, bool L2ONLY = false>
__device__ __forceinline__ void gather_node(const GArgs &g, int32_t A, float *hi, float *lo,
                                            int lane) {
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int BS = NDN * NDN;
  constexpr int NTASK = NNE * NDN;  // (b, j): node of the element, column component
  constexpr int NSLOT = (NTASK + 31) / 32;
  const int cmax = g.maxdeg * NDN;
  const int cols = static_cast<int>(g.nptr[A + 1] - g.nptr[A]) * NDN;
  {
    float4 *z = reinterpret_cast<float4 *>(hi);  // hi and lo are contiguous
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c = lane; c < (2 * NDN * cmax) / 4; c += 32) z[c] = zero;
    for (int c = ((2 * NDN * cmax) / 4) * 4 + lane; c < 2 * NDN * cmax; c += 32) hi[c] = 0.f;
  }
  // the lane's (b, j) tasks, fixed for all incident elements
  int tb[NSLOT], tj[NSLOT], trow[NSLOT];
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const int task = min(lane + 32 * s, NTASK - 1);
    tb[s] = task / NDN;
    tj[s] = task - tb[s] * NDN;
    trow[s] = tb[s] * NNE - tb[s] * (tb[s] - 1) / 2 - tb[s];  // pair(b, x) = trow + x, x >= b
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
    const int rowa = a * NNE - a * (a - 1) / 2 - a;
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      if (lane + 32 * s >= NTASK) break;
      const int b = tb[s], j = tj[s];
      const bool up = a <= b;  // block (a, b) stored; else (b, a), transposed
      const float *blk = kb + (up ? rowa + b : trow[s] + a) * BS + (up ? j : j * NDN);
      const int step = up ? NDN : 1;
      const int col = pe[b] * NDN + j;
      float v[NDN];
#pragma unroll
      for (int i = 0; i < NDN; ++i) v[i] = L2ONLY ? __ldcg(blk + i * step) : blk[i * step];
#pragma unroll
      for (int i = 0; i < NDN; ++i) two_sum_acc(hi[i * cmax + col], lo[i * cmax + col], v[i]);
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

}  // namespace fegpu
