// Tensor-core element blocks for isotropic elasticity (the mixed path's
// element phase on the 5th-generation tensor cores, tcgen05 kind::tf32).
//
// Per element the Gram sums M^{mn}_ab = sum_q g_am(q) (w_q g_bn(q)) are one
// matrix product D = A B^T with A[(a,m), q] = g_am(q) and B[(b,n), q] =
// w_q g_bn(q) (K = the quadrature points, padded to a multiple of 8).  The
// FP32 operands are split into TF32 pairs (x = hi + lo, both TF32) and the
// product is formed as A_hi B_hi + A_lo B_hi + A_hi B_lo, accumulated in FP32
// in tensor memory: about FP32 accuracy at tensor-core speed.
//
// Rows and columns: node a of an element has rows 3*(a mod 10) + m of the
// element's 32-row slot a / 10 (two slots for H20, one for the other solids),
// so the three rows of a node sit in one warp and the elements of a 128-row
// group are the quarters of tensor memory the four warps can read.  A group
// holds 128 / (32 * slots) elements; one MMA chain computes their D's at once
// (the off-diagonal element pairs of the product are computed and ignored).
//
// Per group of elements:
//   geometry (phases A, B, B' of the FP32 tile, mixed_fast.cuh);
//   operands: one thread per (element, node, 4 points) writes the 3 x 4
//     values of A and B, split hi / lo, as float4's into the K-major
//     no-swizzle layout of the MMA (8-row x 16-byte core matrices, K-adjacent
//     cores 128 B apart, 8-row groups Kpad * 32 B apart);
//   one thread issues the 3 * Kpad / 8 MMAs (M = 128, N = 128, K = 8) and
//     commits them to an mbarrier; every thread waits for it (bounded);
//   epilogue: each thread loads its row of D from tensor memory (tcgen05.ld
//     32x32b), exchanges the node's three rows by warp shuffles for the form
//     map K[(a,i),(b,j)] = lam D[(a,i),(b,j)] + mu D[(a,j),(b,i)]
//     + delta_ij mu sum_m D[(a,m),(b,m)], stores the blocks b >= a to a
//     staging area, the diagonal block is made exactly symmetric, and the
//     group's blocks leave with coalesced float4 stores (the same ring layout
//     as the FP32 tile).
#pragma once

#include "mixed_fast.cuh"

namespace fegpu {

constexpr int kTcThreads = 128;  // four warps: the four lane quarters of tensor memory
constexpr int kTcColumns = 128;  // tensor-memory columns per CTA (N = 128, FP32)

template <int NNE> struct TcShape {
  static_assert(NNE <= 20, "at most two 32-row slots per element");
  static constexpr int S = (NNE + 9) / 10;  // 32-row slots per element
  static constexpr int EPG = 4 / S;         // elements per 128-row group
};

__host__ __device__ constexpr int tc_kpad(int npts) { return (npts + 7) / 8 * 8; }

struct TcLayout {
  size_t op_bytes, ops, conn, fx, jinv, det, w, lame, stage, bar, total;
};

// ops: A_hi, A_lo, B_hi, B_lo (each 128 rows x Kpad FP32, core-matrix order)
__host__ __device__ inline TcLayout tc_layout(int nne, int npts) {
  const int S = (nne + 9) / 10, epg = 4 / S;
  TcLayout L;
  size_t o = 0;
  L.op_bytes = static_cast<size_t>(128) * tc_kpad(npts) * 4;
  L.ops = o;
  o += 4 * L.op_bytes;
  L.conn = o;
  o += sizeof(int32_t) * epg * nne;
  o = align_up(o, 16);
  L.fx = o;
  o += sizeof(float4) * epg * nne;
  L.jinv = o;
  o += sizeof(float) * epg * npts * 9;
  L.det = o;
  o += sizeof(float) * epg * npts;
  L.w = o;
  o += sizeof(float) * epg * npts;
  L.lame = o;
  o += sizeof(float) * epg * 2;
  o = align_up(o, 16);
  L.stage = o;
  o += sizeof(float) * epg * (nne * (nne + 1) / 2) * 9;
  o = align_up(o, 16);
  L.bar = o;
  o += 16;  // mbarrier (8 B), tensor-memory address (4 B)
  L.total = align_up(o, 128);
  return L;
}

__device__ __forceinline__ uint32_t tc_smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start, LBO (K-adjacent core
// matrices), SBO (8-row groups), the fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) |
         (static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16) |
         (static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) |
                              ((128u >> 4) << 24);

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc));
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Bounded wait for the MMA chain's commit (phase `parity` of the mbarrier):
// true when it completed, false after about two seconds of %globaltimer.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
    if (done) return true;
    if ((it & 63u) == 63u) {
      uint64_t t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > 2000000000ull || it > (1u << 28)) return false;
    }
  }
}

template <int ET>
__global__ void __launch_bounds__(kTcThreads) k_blocks_tc(const KArgs a) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  static_assert(MDIM == 3, "solid elements");
  constexpr int S = TcShape<NNE>::S, EPG = TcShape<NNE>::EPG;
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int npts = a.npts;
  const int kpad = tc_kpad(npts), kg = kpad / 4;
  const TcLayout L = tc_layout(NNE, npts);
  float *opA_hi = reinterpret_cast<float *>(smem + L.ops);
  float *opA_lo = reinterpret_cast<float *>(smem + L.ops + L.op_bytes);
  float *opB_hi = reinterpret_cast<float *>(smem + L.ops + 2 * L.op_bytes);
  float *opB_lo = reinterpret_cast<float *>(smem + L.ops + 3 * L.op_bytes);
  int32_t *sConn = reinterpret_cast<int32_t *>(smem + L.conn);
  float4 *fX = reinterpret_cast<float4 *>(smem + L.fx);
  float *sJinv = reinterpret_cast<float *>(smem + L.jinv);
  float *sDet = reinterpret_cast<float *>(smem + L.det);
  float *sW = reinterpret_cast<float *>(smem + L.w);
  float *sLame = reinterpret_cast<float *>(smem + L.lame);
  float *sStage = reinterpret_cast<float *>(smem + L.stage);
  uint64_t *sBar = reinterpret_cast<uint64_t *>(smem + L.bar);
  uint32_t *sTmem = reinterpret_cast<uint32_t *>(smem + L.bar + 8);
  const float *fdN = a.tab32 + npts * NNE;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbo = static_cast<uint32_t>(kpad) * 32u;  // bytes per 8-row group

  // operand padding (rows of unused lanes, points >= npts) stays zero: the
  // operand writes below never touch it
  for (size_t i = tid; i < 4 * L.op_bytes / 16; i += kTcThreads)
    reinterpret_cast<float4 *>(smem + L.ops)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid == 0)
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(sBar)));
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_smem_u32(sTmem)),
                 "r"(kTcColumns));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *sTmem;
  const uint32_t bar = tc_smem_u32(sBar);

  const int64_t nel = a.e1 - a.e0;
  const int64_t ngroups = (nel + EPG - 1) / EPG;
  uint32_t parity = 0;
  bool failed = false;
  for (int64_t grp = blockIdx.x; grp < ngroups && !failed; grp += gridDim.x) {
    const int64_t eb = a.e0 + grp * EPG;
    const int ne = static_cast<int>(min(static_cast<int64_t>(EPG), a.e1 - eb));
    // geometry of the group (begins with a barrier: the previous group's
    // epilogue is done with shared and tensor memory)
    asm volatile("tcgen05.fence::before_thread_sync;");
    fast_geometry<ET, F_ELAST_ISO>(a, eb, ne, sConn, fX, sJinv, sDet, sW, sLame);
    // operands: task = (element, 4-point group, node), node fastest (the 8
    // rows a float4 wavefront writes fall in distinct bank groups)
    for (int t = tid; t < ne * kg * NNE; t += kTcThreads) {
      const int k = t % NNE;
      const int j = (t / NNE) % kg;
      const int e = t / (NNE * kg);
      float gA[3][4], gB[3][4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = 4 * j + u;
        float g[3] = {0.f, 0.f, 0.f}, w = 0.f;
        if (q < npts) {
          const float *inv = sJinv + (e * npts + q) * 9;
          const float *d = fdN + (q * NNE + k) * 3;
#pragma unroll
          for (int c = 0; c < 3; ++c) g[c] = fmaf(d[0], inv[c], fmaf(d[1], inv[3 + c], d[2] * inv[6 + c]));
          w = sW[e * npts + q];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          gA[c][u] = g[c];
          gB[c][u] = w * g[c];
        }
      }
      const int rbase = e * S * 32 + (k / 10) * 32 + (k % 10) * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int r = rbase + c;
        const size_t off = ((r >> 3) * static_cast<size_t>(sbo) + j * 128 + (r & 7) * 16) / 4;
        float ah[4], al[4], bh[4], bl[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          ah[u] = tf32_rna(gA[c][u]);
          al[u] = tf32_rna(gA[c][u] - ah[u]);
          bh[u] = tf32_rna(gB[c][u]);
          bl[u] = tf32_rna(gB[c][u] - bh[u]);
        }
        *reinterpret_cast<float4 *>(opA_hi + off) = make_float4(ah[0], ah[1], ah[2], ah[3]);
        *reinterpret_cast<float4 *>(opA_lo + off) = make_float4(al[0], al[1], al[2], al[3]);
        *reinterpret_cast<float4 *>(opB_hi + off) = make_float4(bh[0], bh[1], bh[2], bh[3]);
        *reinterpret_cast<float4 *>(opB_lo + off) = make_float4(bl[0], bl[1], bl[2], bl[3]);
      }
    }
    // the operands become visible to the tensor core; one thread issues
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0) {
      const uint32_t ahi = tc_smem_u32(opA_hi), alo = tc_smem_u32(opA_lo);
      const uint32_t bhi = tc_smem_u32(opB_hi), blo = tc_smem_u32(opB_lo);
      const uint32_t pa[3] = {ahi, alo, ahi}, pb[3] = {bhi, bhi, blo};
      uint32_t acc = 0;
      for (int p = 0; p < 3; ++p)
        for (int s = 0; s < kpad / 8; ++s) {
          tc_mma(tmem, tc_desc(pa[p] + s * 256, 128, sbo), tc_desc(pb[p] + s * 256, 128, sbo), acc);
          acc = 1;
        }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
    }
    const bool ok = tc_wait(bar, parity);
    parity ^= 1u;
    if (__syncthreads_or(!ok)) {
      failed = true;
      if (tid == 0 && a.status) atomicExch(a.status, 3);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    // epilogue: row (a, i) of element e of the group
    {
      const int e = warp / S;
      const int na = (warp % S) * 10 + lane / 3;
      const int i = lane % 3;
      const bool valid = e < ne && lane < 30 && na < NNE;
      float R[S * 32];
#pragma unroll
      for (int h = 0; h < S; ++h)
        tc_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + e * S * 32 + h * 32, R + h * 32);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      const float lam = valid ? sLame[2 * e] : 0.f, mu = valid ? sLame[2 * e + 1] : 0.f;
      const int base = lane - i;
      const int src1 = min(base + (i + 1) % 3, 31), src2 = min(base + (i + 2) % 3, 31);
      const int s0 = min(base, 31), s1 = min(base + 1, 31), s2 = min(base + 2, 31);
      float *kb = sStage + e * NBLK * 9;
#pragma unroll
      for (int b = 0; b < NNE; ++b) {
        const int cb = (b / 10) * 32 + (b % 10) * 3;
        const float x0 = R[cb], x1 = R[cb + 1], x2 = R[cb + 2];
        const float d = i == 0 ? x0 : (i == 1 ? x1 : x2);         // D[(a,i),(b,i)]
        const float p1 = i == 0 ? x2 : (i == 1 ? x0 : x1);        // x[(i+2)%3]
        const float p2 = i == 0 ? x1 : (i == 1 ? x2 : x0);        // x[(i+1)%3]
        const float r1 = __shfl_sync(0xffffffffu, p1, src1);      // D[(a,(i+1)%3),(b,i)]
        const float r2 = __shfl_sync(0xffffffffu, p2, src2);      // D[(a,(i+2)%3),(b,i)]
        const float d0 = __shfl_sync(0xffffffffu, d, s0);
        const float d1 = __shfl_sync(0xffffffffu, d, s1);
        const float d2 = __shfl_sync(0xffffffffu, d, s2);
        const float mtr = mu * (d0 + d1 + d2);
        // y_j = D[(a,j),(b,i)]
        const float y0 = i == 0 ? d : (i == 1 ? r2 : r1);
        const float y1 = i == 1 ? d : (i == 2 ? r2 : r1);
        const float y2 = i == 2 ? d : (i == 0 ? r2 : r1);
        if (valid && b >= na) {
          float *out = kb + (na * NNE - na * (na - 1) / 2 + (b - na)) * 9 + i * 3;
          out[0] = fmaf(lam, x0, mu * y0) + (i == 0 ? mtr : 0.f);
          out[1] = fmaf(lam, x1, mu * y1) + (i == 1 ? mtr : 0.f);
          out[2] = fmaf(lam, x2, mu * y2) + (i == 2 ? mtr : 0.f);
        }
      }
      __syncwarp();
      // the diagonal block (a, a): lower entries from the upper ones
      if (valid) {
        float *dblk = kb + (na * NNE - na * (na - 1) / 2) * 9;
        for (int jj = 0; jj < i; ++jj) dblk[i * 3 + jj] = dblk[jj * 3 + i];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    {
      const int64_t nfl = static_cast<int64_t>(ne) * NBLK * 9;
      float *dst = a.ke + static_cast<int64_t>(eb - a.e0) * NBLK * 9;
      if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0 && (nfl & 3) == 0) {
        const float4 *s4 = reinterpret_cast<const float4 *>(sStage);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
        for (int64_t t = tid; t < nfl / 4; t += kTcThreads) d4[t] = s4[t];
      } else {
        for (int64_t t = tid; t < nfl; t += kTcThreads) dst[t] = sStage[t];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTcColumns));
  }
}

// Tensor-core element blocks are opt-in (FEGPU_MIXED_TC=1): on GB300 the
// FP32-pipe tile is faster for these small per-element products (H20 40^3:
// 1.8 ms per mixed assembly against 3.3 ms; the staging of split operands and
// the tensor-memory epilogue execute more instructions per element than the
// register-tiled Gram sums they replace).  They need a status word (both
// mixed entry points pass one) and at most 32 quadrature points.
inline bool tc_enabled(const KArgs &a) {
  if (!a.status || a.npts > 32) return false;
  const char *env = std::getenv("FEGPU_MIXED_TC");
  return env && env[0] == '1';
}

template <int ET>
int launch_blocks_tc(const KArgs &a, int num_sms, cudaStream_t s) {
  constexpr int NNE = ElemT<ET>::NNE;
  const TcLayout L = tc_layout(NNE, a.npts);
  auto kern = k_blocks_tc<ET>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(L.total)));
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  // resident CTAs per SM: shared memory (227 KB, 1 KB reserved per CTA) and
  // tensor memory (kTcColumns per CTA of 512)
  const int per_sm = std::max(
      1, std::min(static_cast<int>((227 * 1024) / (L.total + 1024)), 512 / kTcColumns));
  const int64_t nel = a.e1 - a.e0;
  if (nel <= 0) return 0;
  const int64_t ngroups = (nel + TcShape<NNE>::EPG - 1) / TcShape<NNE>::EPG;
  const int grid = static_cast<int>(std::min<int64_t>(ngroups, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kTcThreads, L.total, s>>>(a);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace fegpu
