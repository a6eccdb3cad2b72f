// bilform_masslike (src/FEMMBaseModule.jl:1865-1917) on the device: the
// rectangular matrix with nelem*ndn rows and nalldofs columns whose rows
// (i-1)*ndn+1 .. i*ndn belong to element i,
//   M[(i-1)*ndn + p, dof(b, q)] = sum over the points of N_b Jac w c[p, q],
// Jac = Jacobianmdim(m), assembled by SysmatAssemblerSparse (its default).
//
// One thread per element (element order) forms its ndn x nne*ndn block and
// writes it as COO keys (column << 32 | row) and values in the reference's
// triple order (columns outer, rows inner: assemble!, src/AssemblyModule.jl:
// 250-282); the generic assembler's device makematrix! (stable sort, runs
// summed in input order) turns them into the sorted CSC.  Rows belong to one
// element each, so no two elements meet in a row and no colouring is needed.
#include <algorithm>
#include <vector>

#include "fegpu_internal.h"
#include "measure.cuh"

namespace fegpu {
namespace {

template <int NNE, int MDIM, int NDN>
__global__ void k_masslike(const int32_t *conn, const double *xyz, const double *tab, int npts,
                           int sdim, double otherdim, int axisym, int measure_m, int coef_kind,
                           int ncomp, const double *coef, const int32_t *dof, int64_t nelem,
                           uint64_t *key, int64_t *idx, double *V) {
  const double *N = tab;
  const double *dN = tab + npts * NNE;
  const double *w = dN + npts * NNE * MDIM;
  constexpr int NC = NNE * NDN;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < nelem;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t *ce = conn + e * NNE;
    double Me[NDN][NC];
#pragma unroll
    for (int p = 0; p < NDN; ++p)
#pragma unroll
      for (int j = 0; j < NC; ++j) Me[p][j] = 0.0;
    for (int q = 0; q < npts; ++q) {
      double J[3][MDIM];
      jacobian_matrix<NNE, MDIM>(ce, xyz, dN + q * NNE * MDIM, J);
      const double rad = (MDIM == 2 && axisym) ? point_r<NNE>(ce, xyz, N + q * NNE) : 0.0;
      const double Jac = jacobian_mdim<MDIM>(J, sdim, otherdim, measure_m, axisym, rad);
      // c[p][r] at (element e, point q): constant, per element or per point;
      // a scalar stands for that multiple of the identity
      const double *cv = coef_kind == FEGPU_COEF_CONST ? coef
                         : coef_kind == FEGPU_COEF_PER_ELEMENT
                             ? coef + e * ncomp
                             : coef + (e * npts + q) * static_cast<int64_t>(ncomp);
      double c[NDN][NDN];
#pragma unroll
      for (int p = 0; p < NDN; ++p)
#pragma unroll
        for (int r = 0; r < NDN; ++r)
          c[p][r] = ncomp == 1 ? (p == r ? cv[0] : 0.0) : cv[p * NDN + r];
#pragma unroll
      for (int b = 0; b < NNE; ++b) {
        const double factor = N[q * NNE + b] * Jac * w[q];
#pragma unroll
        for (int p = 0; p < NDN; ++p)
#pragma unroll
          for (int r = 0; r < NDN; ++r) Me[p][b * NDN + r] += factor * c[p][r];
      }
    }
    const int64_t t0 = e * static_cast<int64_t>(NDN * NC);
#pragma unroll
    for (int b = 0; b < NNE; ++b)
#pragma unroll
      for (int r = 0; r < NDN; ++r) {
        const uint64_t col = static_cast<uint32_t>(dof[static_cast<int64_t>(ce[b]) * NDN + r]);
        const int j = b * NDN + r;
#pragma unroll
        for (int p = 0; p < NDN; ++p) {
          const int64_t t = t0 + j * NDN + p;
          key[t] = (col << 32) | static_cast<uint64_t>(e * NDN + p);
          idx[t] = t;
          V[t] = Me[p][j];
        }
      }
  }
}

template <int NNE, int MDIM, int NDN>
void launch_masslike(const fegpu_femm *fm, const fegpu_dofmap *dm, int m, int kind, int ncomp,
                     const double *coef, uint64_t *key, int64_t *idx, double *V, cudaStream_t s) {
  if (fm->nelem == 0) return;
  const int grid = static_cast<int>(std::min<int64_t>((fm->nelem + 127) / 128, 4096));
  k_masslike<NNE, MDIM, NDN><<<grid, 128, 0, s>>>(
      fm->conn_orig.as<int32_t>(), fm->xyz.as<double>(), fm->tab.as<double>(), fm->npts,
      fm->sdim, fm->otherdim, fm->axisym, m, kind, ncomp, coef, dm->dof.as<int32_t>(),
      fm->nelem, key, idx, V);
  FEGPU_CUDA(cudaGetLastError());
}

template <int NNE, int MDIM>
void dispatch_ndn(int ndn, const fegpu_femm *fm, const fegpu_dofmap *dm, int m, int kind,
                  int ncomp, const double *coef, uint64_t *key, int64_t *idx, double *V,
                  cudaStream_t s) {
  if (ndn == 1) launch_masslike<NNE, MDIM, 1>(fm, dm, m, kind, ncomp, coef, key, idx, V, s);
  else if (ndn == 2) launch_masslike<NNE, MDIM, 2>(fm, dm, m, kind, ncomp, coef, key, idx, V, s);
  else launch_masslike<NNE, MDIM, 3>(fm, dm, m, kind, ncomp, coef, key, idx, V, s);
}

}  // namespace
}  // namespace fegpu

using namespace fegpu;

extern "C" int fegpu_bilform_masslike(fegpu_dofmap *dm, const fegpu_coef *cf, int m,
                                      fegpu_assembler *a, int64_t *nnz) {
  try {
    FEGPU_REQUIRE(dm && cf && cf->data && a && nnz, "null handle");
    fegpu_femm *fm = dm->femm;
    fegpu_context *ctx = fm->ctx;
    FEGPU_REQUIRE(a->ctx == ctx, "the assembler belongs to another context");
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    if (fm->mdim == 3) FEGPU_REQUIRE(m == 3, "That is the only acceptable option here.");
    else FEGPU_REQUIRE(m == 2 || m == 3, "Those are the only acceptable options here.");
    const int ndn = dm->ndn;
    FEGPU_REQUIRE(ndn >= 1 && ndn <= 3, "masslike: 1 to 3 DOFs per node");
    FEGPU_REQUIRE(a->kind == FEGPU_ASM_SPARSE,
                  "masslike: the matrix is rectangular (SysmatAssemblerSparse)");
    FEGPU_REQUIRE(a->nrows == fm->nelem * ndn && a->ncols == dm->ndof,
                  "masslike: the assembler must be nelem*ndn x nalldofs");
    const int kind = cf->kind;
    FEGPU_REQUIRE(kind == FEGPU_COEF_CONST || kind == FEGPU_COEF_PER_ELEMENT ||
                      kind == FEGPU_COEF_PER_QP,
                  "masslike: bad coefficient kind");
    FEGPU_REQUIRE(cf->ncomp == 1 || cf->ncomp == ndn * ndn,
                  "masslike: the coefficient is a scalar or ndn x ndn");
    cudaStream_t s = ctx->stream;
    const int64_t per = kind == FEGPU_COEF_CONST ? 1
                        : kind == FEGPU_COEF_PER_ELEMENT ? fm->nelem
                                                         : fm->nelem * fm->npts;
    const int64_t ncoef = per * cf->ncomp;
    const int64_t n = fm->nelem * static_cast<int64_t>(ndn) * fm->nne * ndn;
    DevBuf dcoef, key, idx, V;
    dcoef.alloc(sizeof(double) * std::max<int64_t>(ncoef, 1));
    key.alloc(sizeof(uint64_t) * std::max<int64_t>(n, 1));
    idx.alloc(sizeof(int64_t) * std::max<int64_t>(n, 1));
    V.alloc(sizeof(double) * std::max<int64_t>(n, 1));
    if (ncoef > 0)
      FEGPU_CUDA(cudaMemcpyAsync(dcoef.p, cf->data, sizeof(double) * ncoef,
                                 cudaMemcpyHostToDevice, s));
    const double *cv = dcoef.as<double>();
    uint64_t *k = key.as<uint64_t>();
    int64_t *ix = idx.as<int64_t>();
    double *v = V.as<double>();
    switch (fm->etype) {
      case FEGPU_Q4: dispatch_ndn<4, 2>(ndn, fm, dm, m, kind, cf->ncomp, cv, k, ix, v, s); break;
      case FEGPU_H8: dispatch_ndn<8, 3>(ndn, fm, dm, m, kind, cf->ncomp, cv, k, ix, v, s); break;
      case FEGPU_H20: dispatch_ndn<20, 3>(ndn, fm, dm, m, kind, cf->ncomp, cv, k, ix, v, s); break;
      case FEGPU_T4: dispatch_ndn<4, 3>(ndn, fm, dm, m, kind, cf->ncomp, cv, k, ix, v, s); break;
      case FEGPU_T10: dispatch_ndn<10, 3>(ndn, fm, dm, m, kind, cf->ncomp, cv, k, ix, v, s); break;
      default: throw Error{FEGPU_ERR_ARG, "unknown element type"};
    }
    ctx->launches += 1;
    *nnz = assembler_reduce(a, key, idx, v, n);
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    set_error(e.what());
    return FEGPU_ERR_STATE;
  }
}
