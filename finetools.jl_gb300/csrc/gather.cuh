// Row gather of the mixed-precision path: per-node accumulation of element
// blocks with compensated FP32 sums, rounded once to FP64 on the integer and
// FP32 pipes.
// Shared by the single-matrix gather kernel (gather.cu) and the batch kernel
// (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fegpu_internal.h"
#include "ffconv.h"

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

// a - b rounded once, on a register pair (fma(b, -1, a) is exact up to the
// one rounding, like __fsub_rn)
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
// two_sum_acc on two independent accumulators at once (paired FP32
// instructions; the same operations per component)
__device__ __forceinline__ void two_sum_acc2(float2 &h, float2 &l, float2 v) {
  const float2 s = __fadd2_rn(h, v);
  const float2 bb = fsub2(s, h);
  const float2 err = __fadd2_rn(fsub2(h, fsub2(s, bb)), fsub2(v, bb));
  h = s;
  l = __fadd2_rn(l, err);
}

// The accumulators of column c of a node's rows: NDN = 3 keeps rows 0 and 1
// as one float4 (h0, h1, l0, l1) in a01[c] and row 2 as (h2, l2) in a2[c];
// NDN = 1 keeps (h, l) in a2[c].  Same size as NDN (hi, lo) float pairs.
template <int NDN> struct GatherAcc {
  float4 *a01;
  float2 *a2;
  __device__ __forceinline__ GatherAcc(float *base, int cmax)
      : a01(reinterpret_cast<float4 *>(base)),
        a2(reinterpret_cast<float2 *>(base + (NDN == 3 ? 4 * cmax : 0))) {}
  __device__ __forceinline__ void add(int c, const float (&v)[NDN]) const {
    if constexpr (NDN == 3) {
      float4 a = a01[c];
      float2 h = make_float2(a.x, a.y), l = make_float2(a.z, a.w);
      two_sum_acc2(h, l, make_float2(v[0], v[1]));
      a01[c] = make_float4(h.x, h.y, l.x, l.y);
    }
    float2 b = a2[c];
    two_sum_acc(b.x, b.y, v[NDN - 1]);
    a2[c] = b;
  }
  // (h, l) of row i at column c
  __device__ __forceinline__ void get(int c, float (&h)[NDN], float (&l)[NDN]) const {
    if constexpr (NDN == 3) {
      const float4 a = a01[c];
      h[0] = a.x;
      h[1] = a.y;
      l[0] = a.z;
      l[1] = a.w;
    }
    const float2 b = a2[c];
    h[NDN - 1] = b.x;
    l[NDN - 1] = b.y;
  }
};

// One warp gathers the rows of node A: accumulators (GatherAcc, 2 NDN cmax
// floats in the warp's shared region), blocks of the incident elements in
// element order, then one FP64 store per CSR value of the node's rows.
// L2ONLY reads the blocks with ld.global.cg (no L1 allocation): required when
// the blocks were written earlier in the same launch by other CTAs.  PIPE
// loads element k + 1's block entries before accumulating element k (more
// registers: the persistent batch kernel, capped at 128, keeps the plain loop).
template <int NNE, int NDN, bool INLINE_SLOT, bool L2ONLY = false, bool PIPE = !L2ONLY>
__device__ __forceinline__ void gather_node(const GArgs &g, int32_t A, float *accbase, int lane) {
  static_assert(NDN == 1 || NDN == 3, "the mixed path gathers 1 or 3 DOFs per node");
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int BS = NDN * NDN;
  constexpr int NTASK = NNE * NDN;  // (b, j): node of the element, column component
  constexpr int NSLOT = (NTASK + 31) / 32;
  const int cmax = g.maxdeg * NDN;
  const int cols = static_cast<int>(g.nptr[A + 1] - g.nptr[A]) * NDN;
  const GatherAcc<NDN> acc(accbase, cmax);
  // zero the node's own columns only (the others are not touched)
  for (int c = lane; c < cols; c += 32) {
    if constexpr (NDN == 3) acc.a01[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    acc.a2[c] = make_float2(0.f, 0.f);
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
  if constexpr (PIPE) {
  __syncwarp();
  // incident elements in element order, 32 at a time: lane k holds the k-th
  // element, its local node index and its ring slot; the block entries and
  // columns of element k + 1 are loaded before element k is accumulated, so
  // the L2 round trips of consecutive elements overlap
  const int64_t qa = g.n2e_ptr[A], qz = g.n2e_ptr[A + 1];
  for (int64_t qb = qa; qb < qz; qb += 32) {
    const int cnt = static_cast<int>(min(static_cast<int64_t>(32), qz - qb));
    int32_t my_e = 0, my_slot = 0;
    int my_a = 0;
    if (lane < cnt) {
      my_e = g.n2e_elem[qb + lane];
      my_a = g.n2e_loc[qb + lane];
      if constexpr (INLINE_SLOT) {
        const int32_t ch = static_cast<int32_t>(g.chunk);
        const int32_t ce = my_e / ch;
        my_slot = (ce % g.ring) * ch + (my_e - ce * ch);
      } else {
        my_slot = g.n2e_slot[qb + lane];
      }
    }
    float vc[NSLOT][NDN], vn[NSLOT][NDN];
    int cc[NSLOT], cn[NSLOT];
    auto fetch = [&](int k, float (&v)[NSLOT][NDN], int (&col)[NSLOT]) {
      const int32_t e = __shfl_sync(0xffffffffu, my_e, k);
      const int a = __shfl_sync(0xffffffffu, my_a, k);
      const int32_t slot = __shfl_sync(0xffffffffu, my_slot, k);
      const float *kb = g.ke + static_cast<int64_t>(slot) * NBLK * BS;
      const uint16_t *pe = g.pos + (static_cast<int64_t>(e) * NNE + a) * NNE;
      const int rowa = a * NNE - a * (a - 1) / 2 - a;
#pragma unroll
      for (int s2 = 0; s2 < NSLOT; ++s2) {
        col[s2] = 0;
#pragma unroll
        for (int i = 0; i < NDN; ++i) v[s2][i] = 0.f;
        if (lane + 32 * s2 < NTASK) {
          const int b = tb[s2], j = tj[s2];
          const bool up = a <= b;  // block (a, b) stored; else (b, a), transposed
          const float *blk = kb + (up ? rowa + b : trow[s2] + a) * BS + (up ? j : j * NDN);
          const int step = up ? NDN : 1;
          col[s2] = pe[b] * NDN + j;
#pragma unroll
          for (int i = 0; i < NDN; ++i) v[s2][i] = L2ONLY ? __ldcg(blk + i * step) : blk[i * step];
        }
      }
    };
    fetch(0, vc, cc);
    for (int k = 0; k < cnt; ++k) {
      if (k + 1 < cnt) fetch(k + 1, vn, cn);
#pragma unroll
      for (int s2 = 0; s2 < NSLOT; ++s2) {
        if (lane + 32 * s2 >= NTASK) break;
        acc.add(cc[s2], vc[s2]);
      }
      __syncwarp();
#pragma unroll
      for (int s2 = 0; s2 < NSLOT; ++s2) {
        cc[s2] = cn[s2];
#pragma unroll
        for (int i = 0; i < NDN; ++i) vc[s2][i] = vn[s2][i];
      }
    }
  }
  } else {
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
      acc.add(col, v);
    }
    __syncwarp();
  }
  }
  int64_t base[NDN];
#pragma unroll
  for (int i = 0; i < NDN; ++i) base[i] = g.rowptr[g.dof[A * NDN + i]];
  for (int c = lane; c < cols; c += 32) {
    const int64_t off = g.colperm ? g.colperm[g.cpoff[A] * NDN + c] : c;
    float h[NDN], l[NDN];
    acc.get(c, h, l);
#pragma unroll
    for (int i = 0; i < NDN; ++i)
      if (dcheck(g.check, CK_GATHER, base[i] + off, g.nnz))  // debug builds
        g.val[base[i] + off] = ff_to_double(h[i], l[i]);
  }
  __syncwarp();
}

}  // namespace fegpu
