// FP32 element-block kernel of the mixed-precision path.
//
// For a range of elements (one chunk, element order) it writes the upper
// node-pair blocks of every element matrix, in FP32, to the block ring read
// by the row gather (gather.cu).  Per tile of TE elements:
//   A. connectivity; coordinates relative to the element's first node, in
//      FP32 (the basis gradients sum to zero, so J is unchanged);
//   B. one thread per (element, point): J = X' dN (locjac!), det J and J^-1
//      in FP32; an element whose det_min / det_max over its points is below
//      the distortion threshold gets its J, det J and J^-1 recomputed in FP64
//      from the absolute coordinates (the only FP64 arithmetic of the path);
//   C. one thread per (element, point, node): g = dN J^-1 and the weighted
//      gradient w g (w = det J * weight, times the scalar conductivity or
//      kappa for diffusion), stored as float4 so a point costs one 16-byte
//      shared load per node;
//   D. one thread per (element, node a, group of up to four nodes b >= a):
//      the Gram sums M^{mn}_{ab} = sum_q (w g_am)(g_bn) for four blocks at
//      once (w g_a is loaded once and broadcast across the warp), the
//      coefficient map of the form (isotropic Lame, general D, kappa), and
//      the FP32 block store.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "elements.cuh"

namespace fegpu {

constexpr int kMixedThreads = 256;

struct MixedLayout {
  size_t conn, fx, jac, jinv, jw, det, lame, g, wg, total;
};

__host__ __device__ inline MixedLayout mixed_layout(int nne, int mdim, int npts, int te) {
  MixedLayout L;
  size_t o = 0;
  L.conn = o;
  o += sizeof(int32_t) * te * nne;
  o = align_up(o, 16);
  L.fx = o;
  o += sizeof(float) * te * nne * 3;
  o = align_up(o, 16);
  L.jac = o;
  o += sizeof(float) * te * npts * 9;
  L.jinv = o;
  o += sizeof(float) * te * npts * 9;
  L.lame = o;
  o += sizeof(float) * te * 2;
  L.jw = o;
  o += sizeof(float) * te * npts;
  L.det = o;
  o += sizeof(float) * te * npts;
  o = align_up(o, 16);
  L.g = o;
  o += sizeof(float4) * te * npts * nne;
  L.wg = o;
  o += sizeof(float4) * te * npts * nne;
  L.total = align_up(o, 16);
  return L;
}

// number of (a, group of <= 4 nodes b >= a) tasks of one element
__host__ __device__ constexpr int mixed_groups(int nne) {
  int n = 0;
  for (int a = 0; a < nne; ++a) n += (nne - a + 3) / 4;
  return n;
}

// det J and J^-1 (row-major, flat) of a 3 x 3 Jacobian by cofactors, in FP64
__device__ __forceinline__ void inverse3_fp64(const double (&J)[3][3], double *inv, double &det) {
  double m[3][3];
  det = det_inverse3<double, false, true>(J, m);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) inv[r * 3 + c] = m[r][c];
}

// FP64 Jacobian, determinant and inverse of one point (distorted elements).
template <int NNE, int MDIM>
__device__ void jacobian_fp64(const double *xyz, const int32_t *conn, const double *dN, int sdim,
                              double *inv, double &det) {
  double J[3][MDIM];
#pragma unroll
  for (int s = 0; s < 3; ++s)
#pragma unroll
    for (int m = 0; m < MDIM; ++m) J[s][m] = 0.0;
  for (int k = 0; k < NNE; ++k) {
    const double *p = xyz + 4 * static_cast<int64_t>(conn[k]);
#pragma unroll
    for (int m = 0; m < MDIM; ++m) {
      const double d = dN[k * MDIM + m];
#pragma unroll
      for (int s = 0; s < 3; ++s) J[s][m] = fma(p[s], d, J[s][m]);
    }
  }
  if constexpr (MDIM == 3) {
    inverse3_fp64(J, inv, det);
  } else {
    det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const double id = 1.0 / det;
    inv[0] = J[1][1] * id;
    inv[1] = -J[0][1] * id;
    inv[3] = -J[1][0] * id;
    inv[4] = J[0][0] * id;
    (void)sdim;
  }
}

// One tile: elements [eb, eb + ne) of the launch range starting at a.e0.
// Blocks of element e go to ke + (e - e0) * nblk * ndn^2.
template <int ET, int FORM, int NDN>
__device__ __forceinline__ void mixed_tile(const KArgs &a, int64_t eb, int ne,
                                           unsigned char *smem, float *ke, int64_t e0) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int NGRP = mixed_groups(NNE);
  constexpr int BS = NDN * NDN;
  constexpr bool GRAD = FORM != F_DOT;
  const int npts = a.npts, te = a.te;
  const MixedLayout L = mixed_layout(NNE, MDIM, npts, te);
  // FP32 tables live in global memory (read through L1): N[q][k], dN[q][k][m], w[q]
  const float *fN = a.tab32;
  const float *fdN = a.tab32 + npts * NNE;
  const float *fw = fdN + npts * NNE * MDIM;
  float *sJ = reinterpret_cast<float *>(smem + L.jac);
  float *sLame = reinterpret_cast<float *>(smem + L.lame);
  int32_t *sConn = reinterpret_cast<int32_t *>(smem + L.conn);
  float *fX = reinterpret_cast<float *>(smem + L.fx);
  float *sJinv = reinterpret_cast<float *>(smem + L.jinv);
  float *sJw = reinterpret_cast<float *>(smem + L.jw);
  float *sDet = reinterpret_cast<float *>(smem + L.det);
  float4 *sG = reinterpret_cast<float4 *>(smem + L.g);
  float4 *sWG = reinterpret_cast<float4 *>(smem + L.wg);
  const int tid = threadIdx.x, nth = blockDim.x;
  const double *tabdN = a.tab + npts * NNE;
  const float tol = static_cast<float>(a.distort_tol);
  const float odim = static_cast<float>(a.otherdim);
  {
    __syncthreads();
    for (int i = tid; i < ne * NNE; i += nth) {
      const int32_t c = a.conn[eb * NNE + i];
      sConn[i] = dcheck(a.check, CK_CONN, c, a.nnodes) ? c : 0;  // debug builds
    }
    __syncthreads();
    // A. FP32 coordinates relative to the first node
    for (int i = tid; i < ne * NNE; i += nth) {
      const int e = i / NNE;
      const double *p = a.xyz + 4 * static_cast<int64_t>(sConn[i]);
      const double *p0 = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE]);
#pragma unroll
      for (int s = 0; s < 3; ++s) fX[3 * i + s] = float(p[s] - p0[s]);
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
    // B1. rows of J = X' dN per (element, point, space direction)
    for (int i = tid; i < ne * npts * 3; i += nth) {
      const int eq = i / 3, s = i - eq * 3;
      const int e = eq / npts, q = eq - e * npts;
      const float *X = fX + e * NNE * 3 + s;
      const float *d = fdN + q * NNE * MDIM;
      float r[MDIM];
#pragma unroll
      for (int m = 0; m < MDIM; ++m) r[m] = 0.f;
#pragma unroll
      for (int k = 0; k < NNE; ++k)
#pragma unroll
        for (int m = 0; m < MDIM; ++m) r[m] = fmaf(X[3 * k], d[k * MDIM + m], r[m]);
#pragma unroll
      for (int m = 0; m < MDIM; ++m) sJ[eq * 9 + s * 3 + m] = r[m];
    }
    __syncthreads();
    // B2. det J and J^-1 per (element, point) in FP32
    for (int i = tid; i < ne * npts; i += nth) {
      float J[3][MDIM];
#pragma unroll
      for (int s = 0; s < 3; ++s)
#pragma unroll
        for (int m = 0; m < MDIM; ++m) J[s][m] = sJ[i * 9 + s * 3 + m];
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
    // B'. distorted elements: FP64 Jacobian; then the point weight
    for (int i = tid; i < ne * npts; i += nth) {
      const int e = i / npts, q = i - e * npts;
      float dmin = 3.0e38f, dmax = 0.f;
      for (int r = 0; r < npts; ++r) {
        const float v = fabsf(sDet[e * npts + r]);
        dmin = fminf(dmin, v);
        dmax = fmaxf(dmax, v);
      }
      float det = sDet[i];
      // T10 under the affine policy: FP64 geometry for every element here
      // (this tile does not test for straight sides)
      if (GRAD && (!(dmin > tol * dmax) || (NNE == 10 && a.t10_affine))) {
        double inv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, dd;
        jacobian_fp64<NNE, MDIM>(a.xyz, sConn + e * NNE, tabdN + q * NNE * MDIM, a.sdim, inv, dd);
#pragma unroll
        for (int r = 0; r < 9; ++r) sJinv[i * 9 + r] = float(inv[r]);
        det = float(dd);
      }
      float w = det * fw[q];
      if (MDIM == 2 && (GRAD || a.measure_m == 3)) {
        if (a.axisym) {  // 2 pi r from the first node and the relative coordinates
          float r = 0.f;
          for (int k = 0; k < NNE; ++k) r = fmaf(fN[q * NNE + k], fX[3 * (e * NNE + k)], r);
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
      sJw[i] = w;
    }
    __syncthreads();
    // C. gradients and weighted gradients per (element, point, node)
    for (int i = tid; i < (GRAD ? ne * npts * NNE : 0); i += nth) {
      const int eq = i / NNE, k = i - eq * NNE;
      const int q = eq - (eq / npts) * npts;
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
      const float w = sJw[eq];
      float4 wg = make_float4(w * g[0], w * g[1], w * g[2], 0.f);
      if constexpr (FORM == F_DIFF_GEN) {
        const int e = eq / npts;
        const double *kap =
            a.coef_kind == FEGPU_COEF_PER_ELEMENT ? a.coef + (eb + e) * MDIM * MDIM
            : a.coef_kind == FEGPU_COEF_PER_QP    ? a.coef + ((eb + e) * npts + q) * MDIM * MDIM
                                                  : a.cconst;
        float kg[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int m = 0; m < MDIM; ++m)
#pragma unroll
          for (int p = 0; p < MDIM; ++p) kg[m] = fmaf(float(kap[m * MDIM + p]), g[p], kg[m]);
        wg = make_float4(w * kg[0], w * kg[1], w * kg[2], 0.f);
      }
      sG[i] = make_float4(g[0], g[1], g[2], 0.f);
      sWG[i] = wg;
    }
    __syncthreads();
    // D. Gram sums for (a, up to four b >= a), coefficient map, block store
    for (int i = tid; i < ne * NGRP; i += nth) {
      const int e = i / NGRP;
      int r = i - e * NGRP, pa = 0;
      while (r >= (NNE - pa + 3) / 4) {
        r -= (NNE - pa + 3) / 4;
        ++pa;
      }
      const int b0 = pa + 4 * r;
      const int nb = min(4, NNE - b0);
      float M[4][3][3];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) M[u][m][n] = 0.f;
      const float4 *wa = sWG + (e * npts) * NNE + pa;
      const float4 *gb = sG + (e * npts) * NNE + b0;
      if constexpr (!GRAD) {
        // dot: s_ab = sum_q N_a N_b (Jac w c)_q  (src/FEMMBaseModule.jl:1357-1361)
        for (int q = 0; q < npts; ++q) {
          const float wna = sJw[e * npts + q] * fN[q * NNE + pa];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (u < nb) M[u][0][0] = fmaf(wna, fN[q * NNE + b0 + u], M[u][0][0]);
        }
      }
      for (int q = 0; q < (GRAD ? npts : 0); ++q) {
        const float4 x = wa[q * NNE];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (u < nb) {
            const float4 y = gb[q * NNE + u];
            if constexpr (FORM == F_DIFF_ISO || FORM == F_DIFF_GEN) {
              M[u][0][0] = fmaf(x.x, y.x, fmaf(x.y, y.y, fmaf(x.z, y.z, M[u][0][0])));
            } else {
              const float xs[3] = {x.x, x.y, x.z}, ys[3] = {y.x, y.y, y.z};
#pragma unroll
              for (int m = 0; m < 3; ++m)
#pragma unroll
                for (int n = 0; n < 3; ++n) M[u][m][n] = fmaf(xs[m], ys[n], M[u][m][n]);
            }
          }
        }
      }
      const int64_t es = eb + e;
      float lam = 0.f, mu = 0.f;
      if constexpr (FORM == F_ELAST_ISO) {
        lam = sLame[2 * e];
        mu = sLame[2 * e + 1];
      }
      const double *D = (FORM == F_ELAST_GEN && a.coef_kind == FEGPU_COEF_PER_ELEMENT)
                             ? a.coef + es * 36 : a.cconst;
      float *kb = ke + static_cast<int64_t>(eb + e - e0) * NBLK * BS;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (u >= nb) break;
        const int pb = b0 + u;
        float *out = kb + (pa * NNE - pa * (pa - 1) / 2 + (pb - pa)) * BS;
        if constexpr (FORM == F_DIFF_ISO || FORM == F_DIFF_GEN) {
          out[0] = M[u][0][0];
        } else if constexpr (FORM == F_DOT) {
          // block = s * c (c: the symmetric-assembler arrangement set by the host)
          const double *cm = (pb == pa) ? a.cdiag : a.cab;
#pragma unroll
          for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
            for (int jj = 0; jj < NDN; ++jj) out[ii * NDN + jj] = M[u][0][0] * float(cm[ii * NDN + jj]);
        } else {
          float V[3][3];
          if constexpr (FORM == F_ELAST_ISO) {
            const float mtr = mu * (M[u][0][0] + M[u][1][1] + M[u][2][2]);
#pragma unroll
            for (int ii = 0; ii < 3; ++ii)
#pragma unroll
              for (int jj = 0; jj < 3; ++jj)
                V[ii][jj] = fmaf(lam, M[u][ii][jj], mu * M[u][jj][ii]) + (ii == jj ? mtr : 0.f);
          } else {
#pragma unroll
            for (int ii = 0; ii < 3; ++ii)
#pragma unroll
              for (int jj = 0; jj < 3; ++jj) {
                float v = 0.f;
#pragma unroll
                for (int m = 0; m < 3; ++m)
#pragma unroll
                  for (int n = 0; n < 3; ++n)
                    v = fmaf(float(D[voigt_sel(ii, m) * 6 + voigt_sel(jj, n)]), M[u][m][n], v);
                V[ii][jj] = v;
              }
          }
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
}

}  // namespace fegpu
