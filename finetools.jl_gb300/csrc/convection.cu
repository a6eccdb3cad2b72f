// bilform_convection (src/FEMMBaseModule.jl:1583-1625) on the device:
// K[p, r] += N_p (u . grad N_r) Jac w summed over the points, u the velocity
// interpolated from its nodal values; a scalar field (one DOF per node); the
// unsymmetric element matrix goes into the structural CSR pattern (the
// reference's default SysmatAssemblerSparse).  The density rhof the
// reference evaluates does not enter its matrix, so it is not an input.
//
// One thread per element, one launch per colour: a colour's elements share
// no node, so the read-modify-write of the CSR values needs no atomics and
// every value sums its elements in colour order.  FP64 throughout.
#include <algorithm>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

template <int NNE, int MDIM>
__global__ void k_convection(const int32_t *conn, const double *xyz, const double *vel,
                             const double *tab, int npts, const uint16_t *pos, const int32_t *dof,
                             const int64_t *rowptr, const int32_t *colperm, const int64_t *cpoff,
                             double otherdim, int axisym, double *val, int64_t e0,
                             int64_t e1) {
  const double *N = tab;
  const double *dN = tab + npts * NNE;
  const double *w = dN + npts * NNE * MDIM;
  for (int64_t e = e0 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < e1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t *ce = conn + e * NNE;
    double Ke[NNE][NNE];
#pragma unroll
    for (int p = 0; p < NNE; ++p)
#pragma unroll
      for (int r = 0; r < NNE; ++r) Ke[p][r] = 0.0;
    for (int q = 0; q < npts; ++q) {
      const double *Nq = N + q * NNE, *dq = dN + q * NNE * MDIM;
      double J[MDIM][MDIM], u[MDIM];
#pragma unroll
      for (int s = 0; s < MDIM; ++s) {
        u[s] = 0.0;
#pragma unroll
        for (int m = 0; m < MDIM; ++m) J[s][m] = 0.0;
      }
      for (int k = 0; k < NNE; ++k) {
        const double *x = xyz + 4 * static_cast<int64_t>(ce[k]);
        const double *v = vel + 4 * static_cast<int64_t>(ce[k]);
#pragma unroll
        for (int s = 0; s < MDIM; ++s) {
          u[s] = fma(Nq[k], v[s], u[s]);
#pragma unroll
          for (int m = 0; m < MDIM; ++m) J[s][m] = fma(x[s], dq[k * MDIM + m], J[s][m]);
        }
      }
      double inv[MDIM][MDIM], det;
      if constexpr (MDIM == 3) {
        const double c0 = J[1][1] * J[2][2] - J[2][1] * J[1][2];
        const double c1 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
        const double c2 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c0 - J[0][1] * c1 + J[0][2] * c2;
        const double id = 1.0 / det;
        inv[0][0] = c0 * id;
        inv[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        inv[1][0] = -c1 * id;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        inv[1][2] = -(J[0][0] * J[1][2] - J[1][0] * J[0][2]) * id;
        inv[2][0] = c2 * id;
        inv[2][1] = -(J[0][0] * J[2][1] - J[2][0] * J[0][1]) * id;
        inv[2][2] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) * id;
      } else {
        det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
        const double id = 1.0 / det;
        inv[0][0] = J[1][1] * id;
        inv[0][1] = -J[0][1] * id;
        inv[1][0] = -J[1][0] * id;
        inv[1][1] = J[0][0] * id;
      }
      // Jacobianvolume: a two-manifold is scaled by the other dimension
      // Jacobianvolume: a two-manifold is scaled by the other dimension, or by
      // 2 pi r on an axisymmetric domain
      double od = otherdim;
      if (MDIM == 2 && axisym) {
        double r = 0.0;
        for (int k = 0; k < NNE; ++k) r = fma(Nq[k], xyz[4 * static_cast<int64_t>(ce[k])], r);
        od = 2.0 * 3.14159265358979323846 * r;
      }
      const double Jw = (MDIM == 2 ? det * od : det) * w[q];
      // (u . grad N_r) for every r
      double ug[NNE];
#pragma unroll
      for (int r = 0; r < NNE; ++r) {
        double a = 0.0;
#pragma unroll
        for (int c = 0; c < MDIM; ++c) {
          double gc = 0.0;
#pragma unroll
          for (int m = 0; m < MDIM; ++m) gc = fma(dq[r * MDIM + m], inv[m][c], gc);
          a = fma(u[c], gc, a);
        }
        ug[r] = a;
      }
#pragma unroll
      for (int p = 0; p < NNE; ++p) {
        const double np = Nq[p];
#pragma unroll
        for (int r = 0; r < NNE; ++r) Ke[p][r] += np * ug[r] * Jw;
      }
    }
    // scatter row by row (slots of a row are distinct: loads first, then stores)
    for (int p = 0; p < NNE; ++p) {
      const int32_t A = ce[p];
      const int64_t r0 = rowptr[dof[A]];
      const uint16_t *pr = pos + (e * NNE + p) * NNE;
      double cur[NNE];
      int64_t off[NNE];
#pragma unroll
      for (int r = 0; r < NNE; ++r) {
        off[r] = colperm ? colperm[cpoff[A] + pr[r]] : static_cast<int64_t>(pr[r]);
        cur[r] = val[r0 + off[r]];
      }
#pragma unroll
      for (int r = 0; r < NNE; ++r) val[r0 + off[r]] = cur[r] + Ke[p][r];
    }
  }
}

template <int NNE, int MDIM>
void launch_convection(const fegpu_femm *fm, const fegpu_dofmap *dm, const double *vel4,
                       double *val, cudaStream_t s) {
  const int ncol = static_cast<int>(fm->color_offsets.size()) - 1;
  for (int c = 0; c < ncol; ++c) {
    const int64_t e0 = fm->color_offsets[c], e1 = fm->color_offsets[c + 1];
    if (e1 <= e0) continue;
    const int grid = static_cast<int>(std::min<int64_t>((e1 - e0 + 63) / 64, 8192));
    k_convection<NNE, MDIM><<<grid, 64, 0, s>>>(
        fm->conn.as<int32_t>(), fm->xyz.as<double>(), vel4, fm->tab.as<double>(), fm->npts,
        dm->pos.as<uint16_t>(), dm->dof.as<int32_t>(), dm->rowptr.as<int64_t>(),
        dm->contiguous ? nullptr : dm->colperm.as<int32_t>(),
        dm->contiguous ? nullptr : dm->cpoff.as<int64_t>(), fm->otherdim, fm->axisym, val, e0,
        e1);
    FEGPU_CUDA(cudaGetLastError());
  }
}

}  // namespace
}  // namespace fegpu

using namespace fegpu;

extern "C" int fegpu_bilform_convection(fegpu_matrix *K, int nsd, const double *velocity) {
  try {
    FEGPU_REQUIRE(K && velocity, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    fegpu_context *ctx = fm->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    FEGPU_REQUIRE(dm->ndn == 1, "convection: the field must have one DOF per node");
    FEGPU_REQUIRE(fm->mdim == fm->sdim && nsd == fm->sdim,
                  "convection: velocity components = space dimension = manifold dimension");
    cudaStream_t s = ctx->stream;
    const int64_t n = fm->nnodes;
    DevBuf raw, vel4;
    raw.alloc(sizeof(double) * std::max<int64_t>(n * nsd, 1));
    vel4.alloc(sizeof(double) * 4 * std::max<int64_t>(n, 1));
    FEGPU_CUDA(cudaMemcpyAsync(raw.p, velocity, sizeof(double) * n * nsd, cudaMemcpyHostToDevice, s));
    pack_geometry(raw.as<double>(), n, nsd, vel4.as<double>(), s);  // column-major -> [N][4]
    await_export(K, s);
    FEGPU_CUDA(cudaMemsetAsync(K->val.p, 0, sizeof(double) * dm->nnz, s));
    K->unsym = true;
    switch (fm->etype) {
      case FEGPU_Q4: launch_convection<4, 2>(fm, dm, vel4.as<double>(), K->val.as<double>(), s); break;
      case FEGPU_H8: launch_convection<8, 3>(fm, dm, vel4.as<double>(), K->val.as<double>(), s); break;
      case FEGPU_H20: launch_convection<20, 3>(fm, dm, vel4.as<double>(), K->val.as<double>(), s); break;
      case FEGPU_T4: launch_convection<4, 3>(fm, dm, vel4.as<double>(), K->val.as<double>(), s); break;
      case FEGPU_T10: launch_convection<10, 3>(fm, dm, vel4.as<double>(), K->val.as<double>(), s); break;
      default: throw Error{FEGPU_ERR_ARG, "unknown element type"};
    }
    ctx->launches += static_cast<int64_t>(fm->color_offsets.size()) - 1;
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
