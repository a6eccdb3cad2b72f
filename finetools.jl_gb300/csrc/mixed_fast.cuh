// Register-tiled FP32 element blocks: the mixed path's element phase for the
// isotropic forms (scalar diffusion, isotropic elasticity) and the dot form.
//
// Same results as the tile of mixed.cuh (same FP32 arithmetic per block entry:
// sums over the points in point order), organised for the FMA pipe:
//   A. connectivity, FP32 coordinates relative to the element's first node
//      (float4), Lame pair of the element; T10: each mid-edge node tested
//      against its edge midpoint (FP64);
//   B. one thread per (element, point): J = X' dN, det J and J^-1 in FP32;
//      a straight-sided T10 instead takes its constant corner Jacobian, J^-1
//      and det J formed once in FP64 by the point-0 thread;
//   B'. one thread per (element, point): distortion test over the element's
//      points, FP64 J, det J, J^-1 for flagged elements (distorted, or curved
//      T10), point weight w (det J times the rule weight, the other dimension
//      and a scalar coefficient);
//   C. one thread per (element, point, node): g = dN J^-1, stored with w as
//      one float4 (g_x, g_y, g_z, w) at a padded slot (b + b/8, which keeps
//      the four b's of a group in distinct shared-memory banks);
//   D. one thread per (element, tile of TA x TB node pairs): the Gram sums
//      M^{mn}_ab = sum_q (w g_am) g_bn in registers (TA loads of g_a, TB of
//      g_b per point), then the form map and the FP32 block stores (pairs
//      with b >= a only).
#pragma once

#include "mixed.cuh"

namespace fegpu {

// node pairs per tile: 2 a's x 2 b's, or 2 x 4 for H20 in the persistent
// batch kernel (WIDE): there the CTA count is fixed at two per SM and the
// wider tile's register reuse pays (256-mesh batch 90 ms against 95 ms),
// while the single-call kernel runs faster with more, narrower CTAs (H20
// 40^3: 1.69 ms against 1.78 ms per mixed assembly)
template <int NNE, bool WIDE = true> struct FastTiles {
  static constexpr int TA = 2;
  static constexpr int TB = (WIDE && NNE >= 20) ? 4 : 2;
  static constexpr int NA = (NNE + TA - 1) / TA;
  static constexpr int NB = (NNE + TB - 1) / TB;
  // the first tile of row A holding a pair with b >= a:
  // TB B + TB - 1 >= TA A  <=>  B >= floor(TA A / TB)
  __host__ __device__ static constexpr int bmin(int A) { return (TA * A) / TB; }
  // tiles (A, B) holding at least one pair with b >= a, B fastest
  static constexpr int count() {
    int n = 0;
    for (int A = 0; A < NA; ++A)
      for (int B = 0; B < NB; ++B)
        if (TB * B + TB - 1 >= TA * A) ++n;
    return n;
  }
  static constexpr int NT = count();
};

__host__ __device__ constexpr int fast_slot(int b) { return b + b / 8; }
__host__ __device__ constexpr int fast_stride(int nne) { return fast_slot(nne - 1) + 1; }

struct FastLayout {
  size_t conn, fx, jinv, det, w, lame, g, stage, total;
};

// stage: the tile's blocks before the coalesced copy to the ring; it overlays
// the gradients (dead by then) and extends past them when larger.
__host__ __device__ inline FastLayout fast_layout(int nne, int npts, int te, int ndn = 3) {
  FastLayout L;
  size_t o = 0;
  L.conn = o;
  o += sizeof(int32_t) * te * nne;
  o = align_up(o, 16);
  L.fx = o;
  o += sizeof(float4) * te * nne;
  L.jinv = o;
  o += sizeof(float) * te * npts * 9;
  L.det = o;
  o += sizeof(float) * te * npts;
  L.w = o;
  o += sizeof(float) * te * npts;
  L.lame = o;
  o += sizeof(float) * te * 2;
  o = align_up(o, 16);
  L.g = o;
  L.stage = o;
  const size_t gbytes = sizeof(float4) * te * npts * fast_stride(nne);
  const size_t sbytes = sizeof(float) * te * (nne * (nne + 1) / 2) * ndn * ndn;
  o += gbytes > sbytes ? gbytes : sbytes;
  L.total = align_up(o, 16);
  return L;
}

// elements per tile: enough (element, tile) tasks for 256 threads
__host__ __device__ constexpr int fast_tiles_for(int nne, bool wide = true) {
  return nne >= 20 ? (wide ? FastTiles<20, true>::NT : FastTiles<20, false>::NT)
                   : (nne >= 10 ? FastTiles<10>::NT : (nne >= 8 ? FastTiles<8>::NT : FastTiles<4>::NT));
}
// threads of a CTA of the single-call element-block kernel: 128 (eight CTAs
// per SM at 64 registers), so that a barrier between the tile's phases holds
// four warps, not eight; the persistent batch kernel keeps kMixedThreads
constexpr int kFastThreads = 128;

// the largest tile: one (element, node-pair tile) task per thread
inline int max_fast_tile(int etype, bool wide = true) {
  const int nt = fast_tiles_for(nodes_per_elem(etype), wide);
  return std::max(1, (wide ? kMixedThreads : kFastThreads) / nt);
}
inline int default_fast_tile(int etype, bool wide = true) { return max_fast_tile(etype, wide); }

// Phases A, B and B' of the tile (shared with the tensor-core tile of
// mixed_tc.cuh): connectivity and Lame pairs, FP32 coordinates relative to the
// element's first node, J / det J / J^-1 per (element, point), the FP64
// geometry of distorted elements and the point weights.  Starts and ends with
// a CTA barrier.
template <int ET, int FORM>
__device__ __forceinline__ void fast_geometry(const KArgs &a, int64_t eb, int ne, int32_t *sConn,
                                              float4 *fX, float *sJinv, float *sDet, float *sW,
                                              float *sLame) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr bool GRAD = FORM != F_DOT;
  const int npts = a.npts;
  const float *fN = a.tab32;
  const float *fdN = a.tab32 + npts * NNE;
  const float *fw = fdN + npts * NNE * MDIM;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double *tabdN = a.tab + npts * NNE;
  const float tol = static_cast<float>(a.distort_tol);
  const float odim = static_cast<float>(a.otherdim);
  __syncthreads();  // the previous tile is done with shared memory
  for (int i = tid; i < ne * NNE; i += nth) {
    const int32_t c = a.conn[eb * NNE + i];
    sConn[i] = dcheck(a.check, CK_CONN, c, a.nnodes) ? c : 0;  // debug builds
  }
  if constexpr (FORM == F_ELAST_ISO) {
    for (int e = tid; e < ne; e += nth) {
      if (a.coef_kind == FEGPU_COEF_ISO_LAME) {
        sLame[2 * e] = float(a.coef[2 * (eb + e)]);
        sLame[2 * e + 1] = float(a.coef[2 * (eb + e) + 1]);
      } else {
        sLame[2 * e] = float(a.cconst[0]);
        sLame[2 * e + 1] = float(a.cconst[1]);
      }
    }
  }
  __syncthreads();
  // A. FP32 coordinates relative to the first node.  T10 (affine policy): the
  // w slot of a mid-edge node holds 1 when the node is off its edge's
  // midpoint by more than 2^-30 of the edge (FP64 test), else 0
  constexpr bool T10 = (NNE == 10 && MDIM == 3);
  for (int i = tid; i < ne * NNE; i += nth) {
    const int e = i / NNE, k = i - e * NNE;
    const double *p = a.xyz + 4 * static_cast<int64_t>(sConn[i]);
    const double *p0 = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE]);
    float curved = 0.f;
    if constexpr (T10) {
      if (a.t10_affine && k >= 4) {
        // edges of the mid-edge nodes 4..9: (0,1) (1,2) (2,0) (3,0) (3,1) (3,2)
        const int ea = k < 7 ? k - 4 : 3;
        const int eb = k < 7 ? (k == 6 ? 0 : k - 3) : k - 7;
        const double *pa = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE + ea]);
        const double *pb = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE + eb]);
        double dev = 0.0, len = 0.0;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
          dev = fmax(dev, fabs(p[s] - 0.5 * (pa[s] + pb[s])));
          len = fmax(len, fabs(pb[s] - pa[s]));
        }
        curved = dev > 0x1p-30 * len ? 1.f : 0.f;
      }
    }
    fX[i] = make_float4(float(p[0] - p0[0]), float(p[1] - p0[1]), float(p[2] - p0[2]), curved);
  }
  __syncthreads();
  // B. J, det J, J^-1 per (element, point)
  for (int i = tid; i < ne * npts; i += nth) {
    const int e = i / npts, q = i - e * npts;
    const float4 *X = fX + e * NNE;
    const float *d = fdN + q * NNE * MDIM;
    float J[3][MDIM];
    if constexpr (T10 && GRAD) {
      bool affine = a.t10_affine != 0;
#pragma unroll
      for (int k = 4; k < 10; ++k) affine = affine && X[k].w == 0.f;
      if (affine) {
        // straight-sided T10: x = X0 + r (X1 - X0) + s (X2 - X0) + t (X3 - X0),
        // J constant; formed once per element in FP64 from the corners (the
        // point-0 thread) and rounded to FP32 for every point
        if (q == 0) {
          const int32_t *ce = sConn + e * NNE;
          const double *p0 = a.xyz + 4 * static_cast<int64_t>(ce[0]);
          double Jd[3][3], invd[9], detd;
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const double *pm = a.xyz + 4 * static_cast<int64_t>(ce[m + 1]);
#pragma unroll
            for (int s = 0; s < 3; ++s) Jd[s][m] = pm[s] - p0[s];
          }
          inverse3_fp64(Jd, invd, detd);
          for (int qq = 0; qq < npts; ++qq) {
#pragma unroll
            for (int r = 0; r < 9; ++r) sJinv[(i + qq) * 9 + r] = float(invd[r]);
            sDet[i + qq] = float(detd);
          }
        }
        continue;
      }
    }
#pragma unroll
    for (int s = 0; s < 3; ++s)
#pragma unroll
      for (int m = 0; m < MDIM; ++m) J[s][m] = 0.f;
#pragma unroll 4
    for (int k = 0; k < NNE; ++k) {
      const float4 x = X[k];
#pragma unroll
      for (int m = 0; m < MDIM; ++m) {
        const float dk = d[k * MDIM + m];
        J[0][m] = fmaf(x.x, dk, J[0][m]);
        J[1][m] = fmaf(x.y, dk, J[1][m]);
        J[2][m] = fmaf(x.z, dk, J[2][m]);
      }
    }
    float *inv = sJinv + i * 9;
    float det;
    if constexpr (!GRAD) {
      if constexpr (MDIM == 3) {
        det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
              J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
              J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      } else if (a.sdim == 2) {
        det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
      } else {
        const float c1 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
        const float c2 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
        const float c3 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
        det = sqrtf(c1 * c1 + c2 * c2 + c3 * c3);
      }
    } else if constexpr (MDIM == 3) {
      const float c0 = J[1][1] * J[2][2] - J[2][1] * J[1][2];
      const float c1 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
      const float c2 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      det = J[0][0] * c0 - J[0][1] * c1 + J[0][2] * c2;
      const float id = 1.f / det;
      inv[0] = c0 * id;
      inv[1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
      inv[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      inv[3] = -c1 * id;
      inv[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      inv[5] = -(J[0][0] * J[1][2] - J[1][0] * J[0][2]) * id;
      inv[6] = (J[1][0] * J[2][1] - J[2][0] * J[1][1]) * id;
      inv[7] = -(J[0][0] * J[2][1] - J[2][0] * J[0][1]) * id;
      inv[8] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) * id;
    } else {
      det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
      const float id = 1.f / det;
      inv[0] = J[1][1] * id;
      inv[1] = -J[0][1] * id;
      inv[3] = -J[1][0] * id;
      inv[4] = J[0][0] * id;
    }
    sDet[i] = det;
  }
  __syncthreads();
  // B'. distorted elements: FP64 geometry; then the point weight
  for (int i = tid; i < ne * npts; i += nth) {
    const int e = i / npts, q = i - e * npts;
    float det = sDet[i];
    if constexpr (GRAD) {
      float dmin = 3.0e38f, dmax = 0.f;
      for (int r = 0; r < npts; ++r) {
        const float v = fabsf(sDet[e * npts + r]);
        dmin = fminf(dmin, v);
        dmax = fmaxf(dmax, v);
      }
      bool curved = false;
      if constexpr (T10) {
        if (a.t10_affine) {
#pragma unroll
          for (int k = 4; k < 10; ++k) curved = curved || fX[e * NNE + k].w != 0.f;
        }
      }
      if (curved || !(dmin > tol * dmax)) {
        double inv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, dd;
        jacobian_fp64<NNE, MDIM>(a.xyz, sConn + e * NNE, tabdN + q * NNE * MDIM, a.sdim, inv, dd);
#pragma unroll
        for (int r = 0; r < 9; ++r) sJinv[i * 9 + r] = float(inv[r]);
        det = float(dd);
      }
    }
    float w = det * fw[q];
    if (MDIM == 2 && (GRAD || a.measure_m == 3)) {
      if (a.axisym) {  // 2 pi r, r from the element's first node and the relative coordinates
        float r = 0.f;
        for (int k = 0; k < NNE; ++k) r = fmaf(fN[q * NNE + k], fX[e * NNE + k].x, r);
        r += float(a.xyz[4 * static_cast<int64_t>(sConn[e * NNE])]);
        w *= 2.f * 3.14159265f * r;
      } else {
        w *= odim;
      }
    }
    if constexpr (FORM == F_DIFF_ISO || FORM == F_DOT) {
      float c = 1.f;
      if (a.coef_kind == FEGPU_COEF_CONST) c = float(a.cconst[0]);
      else if (a.coef_kind == FEGPU_COEF_PER_ELEMENT) c = float(a.coef[eb + e]);
      else if (a.coef_kind == FEGPU_COEF_PER_QP) c = float(a.coef[(eb + e) * npts + q]);
      w *= c;
    }
    sW[i] = w;
  }
  __syncthreads();
}

template <int ET, int FORM, int NDN, bool WIDE = true>
__device__ __forceinline__ void mixed_tile_fast(const KArgs &a, int64_t eb, int ne,
                                                unsigned char *smem, float *ke, int64_t e0) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int BS = NDN * NDN;
  constexpr bool GRAD = FORM != F_DOT;
  constexpr int SLOTS = fast_stride(NNE);
  using T = FastTiles<NNE, WIDE>;
  constexpr int TA = T::TA, TB = T::TB, NT = T::NT;
  static_assert(FORM == F_DIFF_ISO || FORM == F_ELAST_ISO || FORM == F_DOT, "isotropic forms");
  const int npts = a.npts, te = a.te;
  const FastLayout L = fast_layout(NNE, npts, te, NDN);
  const float *fN = a.tab32;
  const float *fdN = a.tab32 + npts * NNE;
  int32_t *sConn = reinterpret_cast<int32_t *>(smem + L.conn);
  float4 *fX = reinterpret_cast<float4 *>(smem + L.fx);
  float *sJinv = reinterpret_cast<float *>(smem + L.jinv);
  float *sDet = reinterpret_cast<float *>(smem + L.det);
  float *sW = reinterpret_cast<float *>(smem + L.w);
  float *sLame = reinterpret_cast<float *>(smem + L.lame);
  float4 *sG = reinterpret_cast<float4 *>(smem + L.g);
  const int tid = threadIdx.x, nth = blockDim.x;

  fast_geometry<ET, FORM>(a, eb, ne, sConn, fX, sJinv, sDet, sW, sLame);
  // C. (g, w) per (element, point, node): thread t handles node t % NNE of
  // the (element, point) rows t / NNE, t / NNE + R, ... (R = threads / NNE)
  if constexpr (GRAD) {
    const int R = nth / NNE;
    const int k = tid % NNE, r0 = tid / NNE;
    if (r0 < R) {
      int q = r0 % npts;
      const int qstep = R % npts;
      for (int eq = r0; eq < ne * npts; eq += R) {
        const float *inv = sJinv + eq * 9;
        const float *d = fdN + (q * NNE + k) * MDIM;
        float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < MDIM; ++c) {
          float v = 0.f;
#pragma unroll
          for (int m = 0; m < MDIM; ++m) v = fmaf(d[m], inv[m * 3 + c], v);
          g[c] = v;
        }
        sG[eq * SLOTS + fast_slot(k)] = make_float4(g[0], g[1], g[2], sW[eq]);
        q += qstep;
        if (q >= npts) q -= npts;
      }
    }
    __syncthreads();
  }
  // D. Gram sums per (element, tile of node pairs), form map, block stores.
  // One task per thread (te * NT <= threads): the staging barrier below is
  // reached by every thread.
  {
    const int i = tid;
    const bool active = i < ne * NT;
    const int e = active ? i / NT : 0;
    // task t -> tile (A, B), row after row with B fastest: a loop over the
    // rows (row A holds the tiles B >= bmin(A)) for the long tile lists
    // (H20: 55 tiles), an unrolled search for the short ones
    int t = active ? i - e * NT : 0, A = 0, B = 0;
    if constexpr (NT > 16) {
      for (; A < T::NA - 1; ++A) {
        const int len = T::NB - T::bmin(A);
        if (t < len) break;
        t -= len;
      }
      B = T::bmin(A) + t;
    } else {
      int n = 0;
      bool found = false;
#pragma unroll
      for (int AA = 0; AA < T::NA; ++AA)
#pragma unroll
        for (int BB = 0; BB < T::NB; ++BB)
          if (BB >= T::bmin(AA)) {
            if (!found && n == t) {
              A = AA;
              B = BB;
              found = true;
            }
            ++n;
          }
    }
    int ia[TA], ib[TB];
#pragma unroll
    for (int u = 0; u < TA; ++u) ia[u] = min(TA * A + u, NNE - 1);
#pragma unroll
    for (int v = 0; v < TB; ++v) ib[v] = min(TB * B + v, NNE - 1);
    constexpr int NM = (FORM == F_ELAST_ISO) ? 9 : 1;
    float M[TA][TB][NM];
#pragma unroll
    for (int u = 0; u < TA; ++u)
#pragma unroll
      for (int v = 0; v < TB; ++v)
#pragma unroll
        for (int r = 0; r < NM; ++r) M[u][v][r] = 0.f;
    if constexpr (GRAD) {
      const float4 *G = sG + static_cast<size_t>(e) * npts * SLOTS;
      for (int q = 0; q < (active ? npts : 0); ++q) {
        const float4 *Gq = G + q * SLOTS;
        float wa[TA][3];
#pragma unroll
        for (int u = 0; u < TA; ++u) {
          const float4 x = Gq[fast_slot(ia[u])];
          wa[u][0] = x.w * x.x;
          wa[u][1] = x.w * x.y;
          wa[u][2] = x.w * x.z;
        }
#pragma unroll
        for (int v = 0; v < TB; ++v) {
          const float4 y = Gq[fast_slot(ib[v])];
#pragma unroll
          for (int u = 0; u < TA; ++u) {
            if constexpr (FORM == F_ELAST_ISO) {
              M[u][v][0] = fmaf(wa[u][0], y.x, M[u][v][0]);
              M[u][v][1] = fmaf(wa[u][0], y.y, M[u][v][1]);
              M[u][v][2] = fmaf(wa[u][0], y.z, M[u][v][2]);
              M[u][v][3] = fmaf(wa[u][1], y.x, M[u][v][3]);
              M[u][v][4] = fmaf(wa[u][1], y.y, M[u][v][4]);
              M[u][v][5] = fmaf(wa[u][1], y.z, M[u][v][5]);
              M[u][v][6] = fmaf(wa[u][2], y.x, M[u][v][6]);
              M[u][v][7] = fmaf(wa[u][2], y.y, M[u][v][7]);
              M[u][v][8] = fmaf(wa[u][2], y.z, M[u][v][8]);
            } else {
              M[u][v][0] = fmaf(wa[u][0], y.x, fmaf(wa[u][1], y.y, fmaf(wa[u][2], y.z, M[u][v][0])));
            }
          }
        }
      }
    } else {
      // dot: s_ab = sum_q w N_a N_b (src/FEMMBaseModule.jl:1357-1361)
      for (int q = 0; q < (active ? npts : 0); ++q) {
        const float w = sW[e * npts + q];
        float wn[TA];
#pragma unroll
        for (int u = 0; u < TA; ++u) wn[u] = w * fN[q * NNE + ia[u]];
#pragma unroll
        for (int v = 0; v < TB; ++v) {
          const float nb = fN[q * NNE + ib[v]];
#pragma unroll
          for (int u = 0; u < TA; ++u) M[u][v][0] = fmaf(wn[u], nb, M[u][v][0]);
        }
      }
    }
    float lam = 0.f, mu = 0.f;
    if constexpr (FORM == F_ELAST_ISO) {
      lam = sLame[2 * e];
      mu = sLame[2 * e + 1];
    }
    // blocks go to a staging copy of the tile's ring segment in shared memory
    // (over the gradients, once every thread is done with them), then out
    // with coalesced stores
    __syncthreads();
    float *kb = reinterpret_cast<float *>(smem + L.stage) + static_cast<int64_t>(e) * NBLK * BS;
#pragma unroll
    for (int u = 0; u < TA; ++u) {
      const int pa = TA * A + u;
#pragma unroll
      for (int v = 0; v < TB; ++v) {
        const int pb = TB * B + v;
        if (!active || pa >= NNE || pb >= NNE || pb < pa) continue;
        float *out = kb + (pa * NNE - pa * (pa - 1) / 2 + (pb - pa)) * BS;
        if constexpr (FORM == F_DIFF_ISO) {
          out[0] = M[u][v][0];
        } else if constexpr (FORM == F_DOT) {
          const double *cm = (pb == pa) ? a.cdiag : a.cab;
#pragma unroll
          for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
            for (int jj = 0; jj < NDN; ++jj) out[ii * NDN + jj] = M[u][v][0] * float(cm[ii * NDN + jj]);
        } else {
          const float *m = M[u][v];
          const float mtr = mu * (m[0] + m[4] + m[8]);
          float V[3][3];
#pragma unroll
          for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj)
              V[ii][jj] = fmaf(lam, m[ii * 3 + jj], mu * m[jj * 3 + ii]) + (ii == jj ? mtr : 0.f);
          if (pb == pa) {
#pragma unroll
            for (int ii = 0; ii < 3; ++ii)
#pragma unroll
              for (int jj = 0; jj < ii; ++jj) V[ii][jj] = V[jj][ii];
          }
#pragma unroll
          for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) out[ii * 3 + jj] = V[ii][jj];
        }
      }
    }
  }
  __syncthreads();
  {
    const int64_t nfl = static_cast<int64_t>(ne) * NBLK * BS;
    const float *src = reinterpret_cast<const float *>(smem + L.stage);
    float *dst = ke + static_cast<int64_t>(eb - e0) * NBLK * BS;
    if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0 && (nfl & 3) == 0) {
      const float4 *s4 = reinterpret_cast<const float4 *>(src);
      float4 *d4 = reinterpret_cast<float4 *>(dst);
      for (int64_t i = tid; i < nfl / 4; i += nth) d4[i] = s4[i];
    } else {
      for (int64_t i = tid; i < nfl; i += nth) dst[i] = src[i];
    }
  }
}

// ---- the element-block kernel of the single-matrix mixed path ---------------

template <int FORM> constexpr bool kFastForm =
    FORM == F_DIFF_ISO || FORM == F_ELAST_ISO || FORM == F_DOT;

// Elements per tile of the general-coefficient tile (mixed.cuh): enough Gram
// tasks for the CTA, within a shared-memory budget that leaves two CTAs per SM.
inline int default_general_tile(int etype, int npts) {
  const int nne = nodes_per_elem(etype), mdim = manif_dim(etype);
  const size_t budget = 72 * 1024;
  const MixedLayout one = mixed_layout(nne, mdim, npts, 1);
  const MixedLayout two = mixed_layout(nne, mdim, npts, 2);
  const size_t per = two.total - one.total;
  const size_t fixed = one.total - per;
  const int fit = static_cast<int>((budget - std::min(budget, fixed)) / per);
  const int want = (kMixedThreads + mixed_groups(nne) - 1) / mixed_groups(nne);
  return std::max(1, std::min(fit, want));
}

// shared memory of one tile of te elements of a form
inline size_t tile_smem_bytes(int etype, int form, int npts, int te) {
  const int nne = nodes_per_elem(etype);
  if (form == F_DIFF_ISO || form == F_ELAST_ISO || form == F_DOT)
    return fast_layout(nne, npts, te, 3).total;  // the largest block size (ndn 3)
  return mixed_layout(nne, manif_dim(etype), npts, te).total;
}

// elements per tile; rules with many points (Gauss orders above 3) get fewer
// elements so that a tile's tables stay within a CTA's shared memory
inline int default_tile(int etype, int form, int npts, bool wide = true) {
  int te = (form == F_DIFF_ISO || form == F_ELAST_ISO || form == F_DOT)
               ? default_fast_tile(etype, wide)
               : default_general_tile(etype, npts);
  while (te > 1 && tile_smem_bytes(etype, form, npts, te) > 200 * 1024) --te;
  return te;
}

// the register-tiled forms, held to 64 registers: eight CTAs per SM
template <int ET, int FORM, int NDN>
__global__ void __launch_bounds__(kFastThreads, 8) k_blocks_mixed(const KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t nel = a.e1 - a.e0;
  const int64_t ntiles = (nel + a.te - 1) / a.te;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t eb = a.e0 + tile * a.te;
    const int ne = static_cast<int>(min(static_cast<int64_t>(a.te), a.e1 - eb));
    mixed_tile_fast<ET, FORM, NDN, false>(a, eb, ne, smem, a.ke, a.e0);
  }
}

// general conductivity / general D (the tile of mixed.cuh)
template <int ET, int FORM, int NDN>
__global__ void __launch_bounds__(kMixedThreads) k_blocks_mixed_general(const KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t nel = a.e1 - a.e0;
  const int64_t ntiles = (nel + a.te - 1) / a.te;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t eb = a.e0 + tile * a.te;
    const int ne = static_cast<int>(min(static_cast<int64_t>(a.te), a.e1 - eb));
    mixed_tile<ET, FORM, NDN>(a, eb, ne, smem, a.ke, a.e0);
  }
}

template <int ET, int FORM, int NDN>
int launch_blocks_mixed_t(const KArgs &a, int num_sms, cudaStream_t s) {
  if constexpr (kFastForm<FORM>)
    FEGPU_REQUIRE(a.te >= 1 && a.te <= max_fast_tile(ET, false),
                  "mixed: elements per tile out of range");
  const size_t smem = tile_smem_bytes(ET, FORM, a.npts, a.te);
  void (*kern)(const KArgs);
  if constexpr (kFastForm<FORM>) kern = k_blocks_mixed<ET, FORM, NDN>;
  else kern = k_blocks_mixed_general<ET, FORM, NDN>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  const int threads = kFastForm<FORM> ? kFastThreads : kMixedThreads;
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  per_sm = std::max(per_sm, 1);
  const int64_t nel = a.e1 - a.e0;
  if (nel <= 0) return 0;
  const int64_t ntiles = (nel + a.te - 1) / a.te;
  const int grid = static_cast<int>(std::min<int64_t>(ntiles, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, threads, smem, s>>>(a);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace fegpu
