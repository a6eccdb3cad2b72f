// Lumped (diagonal) mass: bilform_dot (src/FEMMBaseModule.jl:1335-1366)
// assembled by SysmatAssemblerSparseDiag (the element matrix's diagonal,
// src/AssemblyModule.jl:722-750) or SysmatAssemblerSparseHRZLumpingSymm (the
// diagonal scaled by the element total over the diagonal total,
// src/AssemblyModule.jl:1065-1095), on the device.
//
// One thread per element, one launch per colour (elements of a colour share
// no node, so the diagonal is updated without atomics and the sum over the
// elements of a DOF runs in colour order: reproducible).  FP64 throughout.
#include <algorithm>

#include "fegpu_internal.h"
#include "measure.cuh"

namespace fegpu {
namespace {

template <int NNE, int MDIM, int NDN>
__global__ void k_lumped_dot(const int32_t *conn, const double *xyz, const double *tab, int npts,
                             int sdim, double otherdim, int axisym, int measure_m, int coef_kind,
                             const double *cconst, const double *coef, const int32_t *dof,
                             int64_t e0, int64_t e1, int hrz, double *diag) {
  const double *N = tab;
  const double *dN = tab + npts * NNE;
  const double *w = dN + npts * NNE * MDIM;
  for (int64_t e = e0 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < e1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t *ce = conn + e * NNE;
    double dg[NNE][NDN];
#pragma unroll
    for (int k = 0; k < NNE; ++k)
#pragma unroll
      for (int p = 0; p < NDN; ++p) dg[k][p] = 0.0;
    double em2 = 0.0;
    for (int q = 0; q < npts; ++q) {
      double J[3][MDIM];
      jacobian_matrix<NNE, MDIM>(ce, xyz, dN + q * NNE * MDIM, J);
      const double rad = (MDIM == 2 && axisym) ? point_r<NNE>(ce, xyz, N + q * NNE) : 0.0;
      const double Jac = jacobian_mdim<MDIM>(J, sdim, otherdim, measure_m, axisym, rad);
      // coefficient c[p][q] at this point
      double c[NDN][NDN];
#pragma unroll
      for (int p = 0; p < NDN; ++p)
#pragma unroll
        for (int r = 0; r < NDN; ++r) {
          double v;
          if (coef_kind == FEGPU_COEF_CONST) v = cconst[p * NDN + r];
          else if (coef_kind == FEGPU_COEF_PER_ELEMENT) v = (p == r) ? coef[e] : 0.0;
          else v = (p == r) ? coef[e * npts + q] : 0.0;
          c[p][r] = v;
        }
      double csum = 0.0;
#pragma unroll
      for (int p = 0; p < NDN; ++p)
#pragma unroll
        for (int r = 0; r < NDN; ++r) csum += c[p][r];
      const double Jw = Jac * w[q];
      double nsum = 0.0;
#pragma unroll
      for (int k = 0; k < NNE; ++k) {
        const double nk = N[q * NNE + k];
        nsum += nk;
        const double factor = nk * nk * Jac * w[q];  // N_k N_k Jac w, as the reference
#pragma unroll
        for (int p = 0; p < NDN; ++p) dg[k][p] += factor * c[p][p];
      }
      em2 += nsum * nsum * Jw * csum;  // sum of every entry of the element matrix
    }
    double ff = 1.0;
    if (hrz) {
      double dem2 = 0.0;
#pragma unroll
      for (int k = 0; k < NNE; ++k)
#pragma unroll
        for (int p = 0; p < NDN; ++p) dem2 += dg[k][p];
      ff = em2 / dem2;
    }
#pragma unroll
    for (int k = 0; k < NNE; ++k)
#pragma unroll
      for (int p = 0; p < NDN; ++p) {
        const int32_t d = dof[static_cast<int64_t>(ce[k]) * NDN + p];
        diag[d] += hrz ? dg[k][p] * ff : dg[k][p];
      }
  }
}

template <int NNE, int MDIM, int NDN>
void launch_lumped(const fegpu_femm *fm, const fegpu_dofmap *dm, const double *cconst,
                   const double *coef, int coef_kind, int m, int hrz, double *diag,
                   cudaStream_t s) {
  const int ncol = static_cast<int>(fm->color_offsets.size()) - 1;
  for (int c = 0; c < ncol; ++c) {
    const int64_t e0 = fm->color_offsets[c], e1 = fm->color_offsets[c + 1];
    if (e1 <= e0) continue;
    const int grid = static_cast<int>(std::min<int64_t>((e1 - e0 + 127) / 128, 4096));
    k_lumped_dot<NNE, MDIM, NDN><<<grid, 128, 0, s>>>(
        fm->conn.as<int32_t>(), fm->xyz.as<double>(), fm->tab.as<double>(), fm->npts, fm->sdim,
        fm->otherdim, fm->axisym, m, coef_kind, cconst, coef, dm->dof.as<int32_t>(), e0, e1, hrz,
        diag);
    FEGPU_CUDA(cudaGetLastError());
  }
}

template <int NNE, int MDIM>
void dispatch_ndn(int ndn, const fegpu_femm *fm, const fegpu_dofmap *dm, const double *cconst,
                  const double *coef, int kind, int m, int hrz, double *diag, cudaStream_t s) {
  if (ndn == 1) launch_lumped<NNE, MDIM, 1>(fm, dm, cconst, coef, kind, m, hrz, diag, s);
  else if (ndn == 2) launch_lumped<NNE, MDIM, 2>(fm, dm, cconst, coef, kind, m, hrz, diag, s);
  else launch_lumped<NNE, MDIM, 3>(fm, dm, cconst, coef, kind, m, hrz, diag, s);
}

}  // namespace
}  // namespace fegpu

using namespace fegpu;

extern "C" int fegpu_bilform_dot_lumped(fegpu_dofmap *dm, const fegpu_coef *cf, int m, int hrz,
                                        double *diag) {
  try {
    FEGPU_REQUIRE(dm && cf && cf->data && diag, "null handle");
    fegpu_femm *fm = dm->femm;
    fegpu_context *ctx = fm->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
    else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    const int ndn = dm->ndn;
    cudaStream_t s = ctx->stream;
    DevBuf dconst, dcoef, dsorted, dd;
    int kind = cf->kind;
    dconst.alloc(sizeof(double) * 9);
    std::vector<double> hc(9, 0.0);
    if (kind == FEGPU_COEF_CONST) {
      if (cf->ncomp == 1) {
        for (int p = 0; p < ndn; ++p) hc[p * ndn + p] = cf->data[0];
      } else {
        FEGPU_REQUIRE(cf->ncomp == ndn * ndn, "dot: coefficient must be ndn x ndn");
        for (int i = 0; i < ndn * ndn; ++i) hc[i] = cf->data[i];
      }
    } else {
      FEGPU_REQUIRE(kind == FEGPU_COEF_PER_ELEMENT || kind == FEGPU_COEF_PER_QP,
                    "dot: bad coefficient kind");
      FEGPU_REQUIRE(cf->ncomp == 1, "dot: per-element / per-point coefficients are scalars");
      // element order -> colour order (the kernel walks colour-sorted elements)
      const int64_t width = kind == FEGPU_COEF_PER_QP ? fm->npts : 1;
      std::vector<double> sorted(static_cast<size_t>(std::max<int64_t>(width * fm->nelem, 1)));
      std::vector<int32_t> perm(static_cast<size_t>(std::max<int64_t>(fm->nelem, 1)));
      if (fm->nelem > 0)
        FEGPU_CUDA(cudaMemcpy(perm.data(), fm->perm.p, sizeof(int32_t) * fm->nelem,
                              cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < fm->nelem; ++i)
        for (int64_t k = 0; k < width; ++k) sorted[i * width + k] = cf->data[perm[i] * width + k];
      dcoef.alloc(sizeof(double) * sorted.size());
      FEGPU_CUDA(cudaMemcpy(dcoef.p, sorted.data(), sizeof(double) * sorted.size(),
                            cudaMemcpyHostToDevice));
    }
    FEGPU_CUDA(cudaMemcpyAsync(dconst.p, hc.data(), sizeof(double) * 9, cudaMemcpyHostToDevice, s));
    dd.alloc(sizeof(double) * std::max<int64_t>(dm->ndof, 1));
    FEGPU_CUDA(cudaMemsetAsync(dd.p, 0, sizeof(double) * dm->ndof, s));
    const double *cc = dconst.as<double>(), *cv = dcoef.as<double>();
    double *dg = dd.as<double>();
    switch (fm->etype) {
      case FEGPU_Q4: dispatch_ndn<4, 2>(ndn, fm, dm, cc, cv, kind, m, hrz, dg, s); break;
      case FEGPU_H8: dispatch_ndn<8, 3>(ndn, fm, dm, cc, cv, kind, m, hrz, dg, s); break;
      case FEGPU_H20: dispatch_ndn<20, 3>(ndn, fm, dm, cc, cv, kind, m, hrz, dg, s); break;
      case FEGPU_T4: dispatch_ndn<4, 3>(ndn, fm, dm, cc, cv, kind, m, hrz, dg, s); break;
      case FEGPU_T10: dispatch_ndn<10, 3>(ndn, fm, dm, cc, cv, kind, m, hrz, dg, s); break;
      default: throw Error{FEGPU_ERR_ARG, "unknown element type"};
    }
    ctx->launches += static_cast<int64_t>(fm->color_offsets.size()) - 1;
    FEGPU_CUDA(cudaMemcpyAsync(diag, dd.p, sizeof(double) * dm->ndof, cudaMemcpyDeviceToHost, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    set_error(e.what());
    return FEGPU_ERR_STATE;
  }
}
