// Element-form kernels: one launch per colour, each CTA loops over tiles of TE
// elements of that colour.
//
// Per tile:
//   1. connectivity and node coordinates of the TE elements -> shared memory;
//   2. one thread per (element, quadrature point): locjac! + Jacobian +
//      gradN! (src/MatrixUtilityModule.jl:60-68, src/FESetModule.jl:479-544)
//      -> gradients g and weighted gradients w*g in shared memory;
//   3. one thread per (element, node pair a <= b): the node-pair block of the
//      element matrix.  All forms are written through the Gram matrix of the
//      gradients,  M^{mn}_{ab} = sum_q (detJ w)_q g_am(q) g_bn(q),  and a
//      per-form map:
//        diffusion      Ke_ab        = sum_mn kappa_mn M^{mn}_ab
//        elasticity     Ke_(ai)(bj)  = sum_mn D[s(i,m)][s(j,n)] M^{mn}_ab
//                       (s: Voigt position of B's nonzeros, blmat!,
//                        src/DeforModelRedModule.jl:447-472)
//        dot            Ke_(ai)(bj)  = (sum_q Jw N_a N_b) c_ij
//      which equals B'DB, grad N kappa grad N' and N N' c of the reference
//      (add_btdb_ut_only!, add_gkgt_ut_only!, add_mggt_ut_only!) summed over
//      the quadrature points, with B's structural zeros skipped;
//   4. the block and its mirror are added into the CSR values.  Elements of
//      one colour share no node, so the read-modify-write needs no atomics
//      and every entry is summed in a fixed (colour) order: the result is
//      bitwise reproducible and exactly symmetric.
// The upper triangle by local DOF index is computed and mirrored, as
// complete_lt! (src/MatrixUtilityModule.jl:164-173) and the symmetric
// assembler do.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "fegpu_internal.h"

namespace fegpu {

constexpr int kFormThreads = 256;

template <int ET> struct ElemT;
template <> struct ElemT<FEGPU_Q4> { static constexpr int NNE = 4, MDIM = 2; };
template <> struct ElemT<FEGPU_H8> { static constexpr int NNE = 8, MDIM = 3; };
template <> struct ElemT<FEGPU_H20> { static constexpr int NNE = 20, MDIM = 3; };
template <> struct ElemT<FEGPU_T4> { static constexpr int NNE = 4, MDIM = 3; };
template <> struct ElemT<FEGPU_T10> { static constexpr int NNE = 10, MDIM = 3; };

struct SmemLayout {
  size_t tab, X, G, WG, Jw, det, aff, conn, pairs, total;
};

__host__ __device__ inline size_t align_up(size_t o, size_t a) { return (o + a - 1) / a * a; }

__host__ __device__ inline SmemLayout smem_layout(int nne, int mdim, int npts, int te,
                                                  int tsize, bool grad) {
  SmemLayout L;
  size_t o = 0;
  L.tab = o;
  o += sizeof(double) * (npts * nne + npts * nne * mdim + npts);
  o = align_up(o, 16);
  L.X = o;
  o += sizeof(double) * te * nne * 3;
  o = align_up(o, 16);
  L.G = o;
  if (grad) o += static_cast<size_t>(tsize) * te * npts * nne * mdim;
  o = align_up(o, 16);
  L.WG = o;
  if (grad) o += static_cast<size_t>(tsize) * te * npts * nne * mdim;
  o = align_up(o, 16);
  L.Jw = o;
  o += static_cast<size_t>(tsize) * te * npts;
  o = align_up(o, 16);
  L.det = o;
  o += sizeof(float) * te * npts;
  o = align_up(o, 16);
  // T10 gradient forms: per node, 1 when a mid-edge node is off its edge's
  // midpoint
  L.aff = o;
  if (grad && nne == 10 && mdim == 3) o += sizeof(uint8_t) * te * nne;
  o = align_up(o, 16);
  L.conn = o;
  o += sizeof(int32_t) * te * nne;
  L.pairs = o;
  o += 2 * (nne * (nne + 1) / 2);
  L.total = align_up(o, 16);
  return L;
}

// Voigt row of B's nonzero for displacement component i and gradient
// direction m (xx, yy, zz, xy, xz, yz).
__host__ __device__ constexpr int voigt_sel(int i, int m) {
  return i == 0 ? (m == 0 ? 0 : (m == 1 ? 3 : 4))
                : (i == 1 ? (m == 0 ? 3 : (m == 1 ? 1 : 5)) : (m == 0 ? 4 : (m == 1 ? 5 : 2)));
}

// Arithmetic helpers.  In FP64 every product and sum is rounded on its own
// (no contraction into FMA), so the element arithmetic follows the
// reference's expressions operation by operation; in FP32 contraction is
// allowed (it only adds accuracy).
// EX selects the exact (uncontracted) FP64 form; the elasticity kernels,
// whose contraction order is their own anyway, use fused FP64 multiply-adds
// (half the FP64 instructions on a part whose FP64 rate is 1/64 of FP32).
template <typename C, bool EX = true>
__device__ __forceinline__ C mul(C a, C b) {
  if constexpr (std::is_same<C, double>::value && EX) return __dmul_rn(a, b);
  else return a * b;
}
template <typename C, bool EX = true>
__device__ __forceinline__ C add(C a, C b) {
  if constexpr (std::is_same<C, double>::value && EX) return __dadd_rn(a, b);
  else return a + b;
}
template <typename C, bool EX = true>
__device__ __forceinline__ C sub(C a, C b) {
  if constexpr (std::is_same<C, double>::value && EX) return __dsub_rn(a, b);
  else return a - b;
}
template <typename C, bool EX = true>
__device__ __forceinline__ C madd(C a, C b, C c) {  // c + a*b
  if constexpr (std::is_same<C, double>::value && EX) return __dadd_rn(c, __dmul_rn(a, b));
  else return fma(a, b, c);
}

// det J (returned) and, with INV, J^-1 of a 3 x 3 Jacobian by cofactors
// (Jacobian(), src/FESetModule.jl:426-435; gradN!, 507-544).
template <typename C, bool EX, bool INV>
__device__ __forceinline__ C det_inverse3(const C (&J)[3][3], C (&inv)[3][3]) {
  const C c0 = sub<C, EX>(mul<C, EX>(J[1][1], J[2][2]), mul<C, EX>(J[2][1], J[1][2]));
  const C c1 = sub<C, EX>(mul<C, EX>(J[1][0], J[2][2]), mul<C, EX>(J[1][2], J[2][0]));
  const C c2 = sub<C, EX>(mul<C, EX>(J[1][0], J[2][1]), mul<C, EX>(J[1][1], J[2][0]));
  const C det = add<C, EX>(sub<C, EX>(mul<C, EX>(J[0][0], c0), mul<C, EX>(J[0][1], c1)), mul<C, EX>(J[0][2], c2));
  if (INV) {
    const C id = C(1) / det;
    inv[0][0] = mul<C, EX>(c0, id);
    inv[0][1] = mul<C, EX>(-sub<C, EX>(mul<C, EX>(J[0][1], J[2][2]), mul<C, EX>(J[0][2], J[2][1])), id);
    inv[0][2] = mul<C, EX>(sub<C, EX>(mul<C, EX>(J[0][1], J[1][2]), mul<C, EX>(J[0][2], J[1][1])), id);
    inv[1][0] = mul<C, EX>(-c1, id);
    inv[1][1] = mul<C, EX>(sub<C, EX>(mul<C, EX>(J[0][0], J[2][2]), mul<C, EX>(J[0][2], J[2][0])), id);
    inv[1][2] = mul<C, EX>(-sub<C, EX>(mul<C, EX>(J[0][0], J[1][2]), mul<C, EX>(J[1][0], J[0][2])), id);
    inv[2][0] = mul<C, EX>(sub<C, EX>(mul<C, EX>(J[1][0], J[2][1]), mul<C, EX>(J[2][0], J[1][1])), id);
    inv[2][1] = mul<C, EX>(-sub<C, EX>(mul<C, EX>(J[0][0], J[2][1]), mul<C, EX>(J[2][0], J[0][1])), id);
    inv[2][2] = mul<C, EX>(sub<C, EX>(mul<C, EX>(J[0][0], J[1][1]), mul<C, EX>(J[1][0], J[0][1])), id);
  }
  return det;
}

// spatial gradients g_k = dN_k J^-1 (gradN!, src/FESetModule.jl:507-544)
template <int NNE, int MDIM, typename C, typename T, bool EX, typename XT>
__device__ __forceinline__ void gradients(const XT *dN, const C (&inv)[MDIM][MDIM], T *g) {
#pragma unroll
  for (int k = 0; k < NNE; ++k)
#pragma unroll
    for (int c = 0; c < MDIM; ++c) {
      C v = mul<C, EX>(C(dN[k * MDIM]), inv[0][c]);
#pragma unroll
      for (int m = 1; m < MDIM; ++m) v = madd<C, EX>(C(dN[k * MDIM + m]), inv[m][c], v);
      g[k * MDIM + c] = T(v);
    }
}

// Geometry at one quadrature point, computed in C (double or float):
// locjac! (J = X' dN, src/MatrixUtilityModule.jl:60-68), Jacobian()
// (src/FESetModule.jl:426-435, 479-489) and gradN! (453-470, 507-544).
// Writes the spatial gradients (as T) and returns the measure Jacobian
// (times the other dimension when a two-manifold is integrated as a volume).
template <int NNE, int MDIM, bool GRAD, typename C, typename T, bool EX = true, typename XT>
__device__ __forceinline__ C geometry_qp(const XT *X, const XT *dN, int sdim,
                                         int measure_volume, double otherdim, T *g,
                                         float *det_out, const XT *Nq = nullptr,
                                         int axisym = 0) {
  // coordinates: absolute in FP64; in FP32 relative to the element's first
  // node (computed once per element: the gradients of the basis sum to zero,
  // so J is unchanged)
  C J[3][MDIM];
#pragma unroll
  for (int s = 0; s < 3; ++s)
#pragma unroll
    for (int m = 0; m < MDIM; ++m) J[s][m] = C(0);
#pragma unroll
  for (int k = 0; k < NNE; ++k) {
    C x[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      if constexpr (std::is_same<C, XT>::value) x[s] = X[3 * k + s];
      else x[s] = C(X[3 * k + s] - X[s]);  // FP64 recompute from absolute coordinates
    }
#pragma unroll
    for (int m = 0; m < MDIM; ++m) {
      const C d = C(dN[k * MDIM + m]);
#pragma unroll
      for (int s = 0; s < 3; ++s) J[s][m] = madd<C, EX>(x[s], d, J[s][m]);
    }
  }
  C inv[MDIM][MDIM];
  C Jac;
  if constexpr (MDIM == 3) {
    Jac = det_inverse3<C, EX, GRAD>(J, inv);
  } else {
    if (sdim == 2) {
      Jac = sub<C, EX>(mul<C, EX>(J[0][0], J[1][1]), mul<C, EX>(J[1][0], J[0][1]));
    } else {  // |J1 x J2|
      const C c1 = sub<C, EX>(mul<C, EX>(J[1][0], J[2][1]), mul<C, EX>(J[2][0], J[1][1]));
      const C c2 = sub<C, EX>(mul<C, EX>(J[2][0], J[0][1]), mul<C, EX>(J[0][0], J[2][1]));
      const C c3 = sub<C, EX>(mul<C, EX>(J[0][0], J[1][1]), mul<C, EX>(J[1][0], J[0][1]));
      Jac = sqrt(add<C, EX>(add<C, EX>(mul<C, EX>(c1, c1), mul<C, EX>(c2, c2)), mul<C, EX>(c3, c3)));
    }
    if (GRAD) {
      const C id = C(1) / sub<C, EX>(mul<C, EX>(J[0][0], J[1][1]), mul<C, EX>(J[0][1], J[1][0]));
      inv[0][0] = mul<C, EX>(J[1][1], id);
      inv[0][1] = mul<C, EX>(-J[0][1], id);
      inv[1][0] = mul<C, EX>(-J[1][0], id);
      inv[1][1] = mul<C, EX>(J[0][0], id);
    }
    if (measure_volume) {
      if (axisym) {
        // Jacobianvolume on an axisymmetric domain: Jac * 2 * pi * loc[1]
        // (src/IntegDomainModule.jl:521-549), loc = N' X
        C r = C(0);
#pragma unroll
        for (int k = 0; k < NNE; ++k) r = madd<C, EX>(C(Nq[k]), C(X[3 * k]), r);
        Jac = mul<C, EX>(mul<C, EX>(mul<C, EX>(Jac, C(2)), C(3.14159265358979323846)), r);
      } else {
        Jac = mul<C, EX>(Jac, C(otherdim));
      }
    }
  }
  if (det_out) *det_out = float(Jac);
  if (GRAD) gradients<NNE, MDIM, C, T, EX>(dN, inv, g);
  return Jac;
}

// Per-form weighting of the gradients at one point (WG) and the stored
// per-point scalar (sJw):
//   diffusion (scalar c):  WG = ((c Jac) w) g            (add_mggt_ut_only!)
//   diffusion (kappa):     WG = (Jac w) (kappa g)         (add_gkgt_ut_only!)
//   elasticity (general D): WG = (Jac w) g               (Gram of the gradients)
//   elasticity (lam, mu):  WG = (s (Jac w)) g, s = mu (1 if mu = 0): the Gram
//                          sums come out scaled by mu, and sJw[e, 0] holds
//                          lam / s for the form map
//                          V = (lam/s) M' + M'^T + I tr M' (mu != 0),
//                          V = lam M' (mu = 0)
//   dot:                   sJw = Jac                      (factor formed per pair)
//   linform:               sJw = Jac w
template <int NNE, int MDIM, int FORM, typename T>
__device__ __forceinline__ void qp_weights(const KArgs &a, int64_t es, int q, int npts, T Jac,
                                           double wq, const T *g, T *wg, T *jw) {
  if constexpr (FORM == F_DIFF_ISO) {
    T c = T(1);
    if (a.coef_kind == FEGPU_COEF_CONST) c = T(a.cconst[0]);
    else if (a.coef_kind == FEGPU_COEF_PER_ELEMENT) c = T(a.coef[es]);
    else if (a.coef_kind == FEGPU_COEF_PER_QP) c = T(a.coef[es * npts + q]);
    const T mult = mul(mul(c, Jac), T(wq));
#pragma unroll
    for (int k = 0; k < NNE * MDIM; ++k) wg[k] = mul(mult, g[k]);
    *jw = mult;
  } else if constexpr (FORM == F_DIFF_GEN) {
    // kappa at this point: c = cf(loc, J, i, j) (src/FEMMBaseModule.jl:1497)
    const double *kap = a.coef_kind == FEGPU_COEF_PER_ELEMENT ? a.coef + es * MDIM * MDIM
                        : a.coef_kind == FEGPU_COEF_PER_QP   ? a.coef + (es * npts + q) * MDIM * MDIM
                                                             : a.cconst;
    const T Jw = mul(Jac, T(wq));
#pragma unroll
    for (int k = 0; k < NNE; ++k)
#pragma unroll
      for (int m = 0; m < MDIM; ++m) {
        T acc = mul(T(kap[m * MDIM]), g[k * MDIM]);
#pragma unroll
        for (int p = 1; p < MDIM; ++p) acc = madd(T(kap[m * MDIM + p]), g[k * MDIM + p], acc);
        wg[k * MDIM + m] = mul(Jw, acc);
      }
    *jw = Jw;
  } else if constexpr (FORM == F_ELAST_ISO) {
    T lam, mu;
    if (a.coef_kind == FEGPU_COEF_ISO_LAME) {
      lam = T(a.coef[2 * es]);
      mu = T(a.coef[2 * es + 1]);
    } else {
      lam = T(a.cconst[0]);
      mu = T(a.cconst[1]);
    }
    const T sc = mu != T(0) ? mu : T(1);
    const T Jw = sc * (Jac * T(wq));
#pragma unroll
    for (int k = 0; k < NNE * MDIM; ++k) wg[k] = Jw * g[k];
    if (q == 0) *jw = lam / sc;
  } else if constexpr (FORM == F_ELAST_GEN) {
    const T Jw = Jac * T(wq);
#pragma unroll
    for (int k = 0; k < NNE * MDIM; ++k) wg[k] = Jw * g[k];
    *jw = Jw;
  } else if constexpr (FORM == F_DOT) {
    *jw = Jac;
  } else {
    *jw = mul(Jac, T(wq));
  }
}

template <int ET, int FORM, typename T, int NDN>
__global__ void __launch_bounds__(kFormThreads) k_form(const KArgs a) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr bool GRAD = FORM <= F_ELAST_GEN;
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr bool EXACT = !(FORM == F_ELAST_ISO || FORM == F_ELAST_GEN);
  extern __shared__ __align__(16) unsigned char smem[];
  const int npts = a.npts, te = a.te;
  const SmemLayout L = smem_layout(NNE, MDIM, npts, te, sizeof(T), GRAD);
  double *sN = reinterpret_cast<double *>(smem + L.tab);
  double *sdN = sN + npts * NNE;
  double *sw = sdN + npts * NNE * MDIM;
  double *sX = reinterpret_cast<double *>(smem + L.X);
  T *sG = reinterpret_cast<T *>(smem + L.G);
  T *sWG = reinterpret_cast<T *>(smem + L.WG);
  T *sJw = reinterpret_cast<T *>(smem + L.Jw);
  float *sDet = reinterpret_cast<float *>(smem + L.det);
  int32_t *sConn = reinterpret_cast<int32_t *>(smem + L.conn);
  uint8_t *sPair = smem + L.pairs;
  // straight-sided T10 in the elasticity forms: J constant (per node, 1 when
  // the node is a mid-edge node off its edge's midpoint)
  constexpr bool AFF = NNE == 10 && MDIM == 3 && (FORM == F_ELAST_ISO || FORM == F_ELAST_GEN);
  uint8_t *sOff = smem + L.aff;
  const int tid = threadIdx.x, nth = blockDim.x;

  for (int i = tid; i < npts * NNE * (MDIM + 1) + npts; i += nth) {
    sN[i] = a.tab[i];
  }
  for (int i = tid; i < NBLK; i += nth) {
    int r = i, pa = 0;
    while (r >= NNE - pa) {
      r -= NNE - pa;
      ++pa;
    }
    sPair[2 * i] = static_cast<uint8_t>(pa);
    sPair[2 * i + 1] = static_cast<uint8_t>(pa + r);
  }
  const bool vol = (MDIM == 3) || (FORM <= F_ELAST_GEN) || a.measure_m == 3;
  const int64_t nel = a.e1 - a.e0;
  const int64_t ntiles = (nel + te - 1) / te;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t eb = a.e0 + tile * te;
    const int ne = static_cast<int>(min(static_cast<int64_t>(te), a.e1 - eb));
    __syncthreads();
    for (int i = tid; i < ne * NNE; i += nth) {
      const int32_t c = a.conn[eb * NNE + i];
      sConn[i] = dcheck(a.check, CK_CONN, c, a.nnodes) ? c : 0;  // debug builds
    }
    __syncthreads();
    for (int i = tid; i < ne * NNE; i += nth) {
      const double *p = a.xyz + 4 * static_cast<int64_t>(sConn[i]);
      sX[3 * i] = p[0];
      sX[3 * i + 1] = p[1];
      sX[3 * i + 2] = p[2];
      if constexpr (AFF) {
        // a T10 whose mid-edge nodes are exactly (FP64) at their edge
        // midpoints is the affine map x = X0 + r (X1 - X0) + s (X2 - X0) +
        // t (X3 - X0): its isoparametric J (ten terms per point) is the
        // constant [X1 - X0 | X2 - X0 | X3 - X0]
        const int e = i / NNE, k = i - e * NNE;
        uint8_t off = 0;
        if (k >= 4) {
          // edges of the mid-edge nodes 4..9: (0,1) (1,2) (2,0) (3,0) (3,1) (3,2)
          const int ea = k < 7 ? k - 4 : 3;
          const int eb = k < 7 ? (k == 6 ? 0 : k - 3) : k - 7;
          const double *pa = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE + ea]);
          const double *pb = a.xyz + 4 * static_cast<int64_t>(sConn[e * NNE + eb]);
#pragma unroll
          for (int c = 0; c < 3; ++c)
            off |= p[c] != __dmul_rn(0.5, __dadd_rn(pa[c], pb[c])) ? 1 : 0;
        }
        sOff[i] = off;
      }
    }
    __syncthreads();

    // ---- geometry per (element, quadrature point)
    for (int i = tid; i < ne * npts; i += nth) {
      const int e = i / npts, q = i - e * npts;
      T *g = sG + (static_cast<size_t>(e) * npts + q) * NNE * MDIM;
      T *wg = sWG + (static_cast<size_t>(e) * npts + q) * NNE * MDIM;
      if constexpr (AFF) {
        const uint8_t *off = sOff + e * NNE;
        if ((off[4] | off[5] | off[6] | off[7] | off[8] | off[9]) == 0) {
          const double *X = sX + e * NNE * 3;
          double J[3][3], inv[3][3];
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int m = 0; m < 3; ++m) J[c][m] = X[3 * (m + 1) + c] - X[c];
          const double det = det_inverse3<double, EXACT, true>(J, inv);
          // gradients from the constant barycentric gradients: the rows of
          // J^-1 are grad lambda_1..3, grad lambda_0 = -(their sum); the
          // T10 basis gives g_k = (4 lambda_k - 1) grad lambda_k at a corner
          // and 4 lambda_b grad lambda_a + 4 lambda_a grad lambda_b on edge
          // (a, b); f_k = 4 lambda_k - 1 read from the caller's table (the
          // parametric gradient of corner k is f_k d lambda_k)
          const double *d = sdN + q * NNE * MDIM;
          double gl[4][3], f[4];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            gl[1][c] = inv[0][c];
            gl[2][c] = inv[1][c];
            gl[3][c] = inv[2][c];
            gl[0][c] = -(inv[0][c] + inv[1][c] + inv[2][c]);
          }
          f[0] = -d[0];
          f[1] = d[3];
          f[2] = d[7];
          f[3] = d[11];
#pragma unroll
          for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int c = 0; c < 3; ++c) g[k * 3 + c] = T(f[k] * gl[k][c]);
#pragma unroll
          for (int k = 4; k < 10; ++k) {
            const int ea = k < 7 ? k - 4 : 3;
            const int eb = k < 7 ? (k == 6 ? 0 : k - 3) : k - 7;
            const double fa = f[ea] + 1.0, fb = f[eb] + 1.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) g[k * 3 + c] = T(fma(fb, gl[ea][c], fa * gl[eb][c]));
          }
          sDet[e * npts + q] = float(det);
          qp_weights<NNE, MDIM, FORM, T>(a, eb + e, q, npts, T(det), sw[q], g, wg,
                                         sJw + e * npts + q);
          continue;
        }
      }
      const T Jac = geometry_qp<NNE, MDIM, GRAD, double, T, EXACT>(
          sX + e * NNE * 3, sdN + q * NNE * MDIM, a.sdim, vol, a.otherdim, g, sDet + e * npts + q,
          sN + q * NNE, a.axisym);
      qp_weights<NNE, MDIM, FORM, T>(a, eb + e, q, npts, Jac, sw[q], g, wg, sJw + e * npts + q);
    }
    __syncthreads();

    if constexpr (FORM == F_LIN) {
      // ---- element load vector (linform_dot, src/FEMMBaseModule.jl:1221-1241):
      //      Fe[k, i] += (N_k (Jac w)) f_i, point by point
      for (int i = tid; i < ne * NNE; i += nth) {
        const int e = i / NNE, k = i - e * NNE;
        const int64_t es = eb + e;
        double fe[NDN];
#pragma unroll
        for (int c = 0; c < NDN; ++c) fe[c] = 0.0;
        for (int q = 0; q < npts; ++q) {
          const double nkf = mul(sN[q * NNE + k], double(sJw[e * npts + q]));
          const double *f = a.coef_kind == FEGPU_COEF_CONST ? a.cconst
                            : a.coef_kind == FEGPU_COEF_PER_ELEMENT
                                ? a.coef + es * NDN
                                : a.coef + (es * npts + q) * NDN;
#pragma unroll
          for (int c = 0; c < NDN; ++c) fe[c] = madd(nkf, f[c], fe[c]);
        }
        const int32_t A = sConn[e * NNE + k];
#pragma unroll
        for (int c = 0; c < NDN; ++c) {
          const int32_t r = a.dof[A * NDN + c];
          if (dcheck(a.check, CK_VECTOR, r, a.nnz)) a.val[r] += fe[c];  // debug builds
        }
      }
      continue;
    }

    // ---- node-pair blocks
    for (int i = tid; i < ne * NBLK; i += nth) {
      const int e = i / NBLK, blk = i - e * NBLK;
      const int pa = sPair[2 * blk], pb = sPair[2 * blk + 1];
      const int64_t es = eb + e;
      using VT = typename std::conditional<GRAD, T, double>::type;
      VT V[NDN][NDN];   // K[(A,i),(B,j)]
      VT Vt[NDN][NDN];  // K[(B,j),(A,i)] stored as [j][i]
      if constexpr (FORM == F_DIFF_ISO || FORM == F_DIFF_GEN) {
        // Ke[a, b] += g_a . WG_b, point by point (row a <= column b)
        const T *ga = sG + (static_cast<size_t>(e) * npts) * NNE * MDIM + pa * MDIM;
        const T *wb = sWG + (static_cast<size_t>(e) * npts) * NNE * MDIM + pb * MDIM;
        T s = T(0);
        for (int q = 0; q < npts; ++q) {
          const T *x = ga + q * NNE * MDIM;
          const T *y = wb + q * NNE * MDIM;
          if constexpr (FORM == F_DIFF_ISO) {
#pragma unroll
            for (int m = 0; m < MDIM; ++m) s = madd(x[m], y[m], s);
          } else {
            T acc = mul(x[0], y[0]);
#pragma unroll
            for (int m = 1; m < MDIM; ++m) acc = madd(x[m], y[m], acc);
            s = add(s, acc);
          }
        }
        V[0][0] = s;
        Vt[0][0] = s;
      } else if constexpr (FORM == F_ELAST_ISO || FORM == F_ELAST_GEN) {
        // Gram matrix of the gradients: M^{mn} = sum_q (Jac w) g_am g_bn
        T M[3][3];
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) M[m][n] = T(0);
        const T *wga = sWG + (static_cast<size_t>(e) * npts) * NNE * 3 + pa * 3;
        const T *gb = sG + (static_cast<size_t>(e) * npts) * NNE * 3 + pb * 3;
        for (int q = 0; q < npts; ++q) {
          T x[3], y[3];
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            x[m] = wga[q * NNE * 3 + m];
            y[m] = gb[q * NNE * 3 + m];
          }
#pragma unroll
          for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = 0; n < 3; ++n) M[m][n] = fma(x[m], y[n], M[m][n]);
        }
        if constexpr (FORM == F_ELAST_ISO) {
          // M holds mu M (the weights carry mu); r = lam / mu
          const bool fold =
              (a.coef_kind == FEGPU_COEF_ISO_LAME ? a.coef[2 * es + 1] : a.cconst[1]) != 0.0;
          const T r = sJw[e * npts];
          const T mtr = fold ? (M[0][0] + M[1][1]) + M[2][2] : T(0);
#pragma unroll
          for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) {
              T v = fma(r, M[ii][jj], fold ? M[jj][ii] : T(0));
              if (ii == jj) v += mtr;
              V[ii][jj] = v;
            }
        } else {
          const double *D = a.coef_kind == FEGPU_COEF_PER_ELEMENT ? a.coef + es * 36 : a.cconst;
#pragma unroll
          for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) {
              T v = T(0);
#pragma unroll
              for (int m = 0; m < 3; ++m)
#pragma unroll
                for (int n = 0; n < 3; ++n)
                  v = fma(T(D[voigt_sel(ii, m) * 6 + voigt_sel(jj, n)]), M[m][n], v);
              V[ii][jj] = v;
            }
        }
        if (pa == pb) {  // diagonal block: upper triangle mirrored (complete_lt!)
#pragma unroll
          for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < ii; ++jj) V[ii][jj] = V[jj][ii];
        }
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) Vt[jj][ii] = V[ii][jj];
      } else {  // F_DOT, src/FEMMBaseModule.jl:1357-1361
        const double *cA = (pa == pb) ? a.cdiag : a.cab;
#pragma unroll
        for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
          for (int jj = 0; jj < NDN; ++jj) {
            V[ii][jj] = 0.0;
            Vt[jj][ii] = 0.0;
          }
        for (int q = 0; q < npts; ++q) {
          // factor = N_k N_m Jac w[q], then elmat += factor * c[p, q]
          const double f =
              mul(mul(mul(sN[q * NNE + pa], sN[q * NNE + pb]), double(sJw[e * npts + q])), sw[q]);
          double sc = 1.0;
          if (a.coef_kind == FEGPU_COEF_PER_ELEMENT) sc = a.coef[es];
          else if (a.coef_kind == FEGPU_COEF_PER_QP) sc = a.coef[es * npts + q];
          if (a.coef_kind == FEGPU_COEF_CONST) {
#pragma unroll
            for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
              for (int jj = 0; jj < NDN; ++jj) {
                V[ii][jj] = madd(f, cA[ii * NDN + jj], V[ii][jj]);
                Vt[jj][ii] = madd(f, a.cba[jj * NDN + ii], Vt[jj][ii]);
              }
          } else {
#pragma unroll
            for (int ii = 0; ii < NDN; ++ii) {
              V[ii][ii] = madd(f, sc, V[ii][ii]);
              Vt[ii][ii] = madd(f, sc, Vt[ii][ii]);
            }
          }
        }
      }

      // ---- scatter (no atomics: one colour's elements share no node).  The
      // block's slots are distinct, so all row offsets, then all current
      // values are loaded before any store: independent loads in flight
      // together instead of one read-modify-write round trip per entry.
      const int32_t A = sConn[e * NNE + pa], B = sConn[e * NNE + pb];
      const bool off_diag = pa != pb;
      const int pAB = a.pos[(es * NNE + pa) * NNE + pb];
      const int pBA = off_diag ? a.pos[(es * NNE + pb) * NNE + pa] : 0;
      int64_t rA[NDN], rB[NDN], cA[NDN], cB[NDN];
#pragma unroll
      for (int ii = 0; ii < NDN; ++ii) {
        rA[ii] = a.rowptr[a.dof[A * NDN + ii]];
        rB[ii] = off_diag ? a.rowptr[a.dof[B * NDN + ii]] : 0;
        cA[ii] = a.colperm ? a.colperm[a.cpoff[A] * NDN + NDN * pAB + ii]
                           : static_cast<int64_t>(NDN * pAB + ii);
        cB[ii] = !off_diag ? 0
                 : a.colperm ? a.colperm[a.cpoff[B] * NDN + NDN * pBA + ii]
                             : static_cast<int64_t>(NDN * pBA + ii);
      }
      if constexpr (kDeviceChecks) {  // debug builds: every slot inside the values
        bool inside = true;
#pragma unroll
        for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
          for (int jj = 0; jj < NDN; ++jj) {
            inside = inside && dcheck(a.check, CK_SCATTER, rA[ii] + cA[jj], a.nnz);
            if (off_diag) inside = inside && dcheck(a.check, CK_SCATTER, rB[jj] + cB[ii], a.nnz);
          }
        if (!inside) continue;
      }
      double cur[NDN][NDN], curt[NDN][NDN];
#pragma unroll
      for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
        for (int jj = 0; jj < NDN; ++jj) {
          cur[ii][jj] = a.val[rA[ii] + cA[jj]];
          curt[jj][ii] = off_diag ? a.val[rB[jj] + cB[ii]] : 0.0;
        }
#pragma unroll
      for (int ii = 0; ii < NDN; ++ii)
#pragma unroll
        for (int jj = 0; jj < NDN; ++jj) a.val[rA[ii] + cA[jj]] = cur[ii][jj] + double(V[ii][jj]);
      if (off_diag) {
#pragma unroll
        for (int jj = 0; jj < NDN; ++jj)
#pragma unroll
          for (int ii = 0; ii < NDN; ++ii)
            a.val[rB[jj] + cB[ii]] = curt[jj][ii] + double(Vt[jj][ii]);
      }
    }
  }
}

// Host-side launcher for one instantiation.
template <int ET, int FORM, typename T, int NDN>
int launch_one(const KArgs &a, int num_sms, cudaStream_t s) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr bool GRAD = FORM <= F_ELAST_GEN;
  const SmemLayout L = smem_layout(NNE, MDIM, a.npts, a.te, sizeof(T), GRAD);
  auto kern = k_form<ET, FORM, T, NDN>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(L.total)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFormThreads, L.total));
  if (per_sm < 1) per_sm = 1;
  const int64_t nel = a.e1 - a.e0;
  if (nel <= 0) return 0;
  const int64_t ntiles = (nel + a.te - 1) / a.te;
  const int grid = static_cast<int>(std::min<int64_t>(ntiles, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kFormThreads, L.total, s>>>(a);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace fegpu
