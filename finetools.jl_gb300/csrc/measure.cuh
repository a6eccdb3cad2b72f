// Geometry at a quadrature point for the one-thread-per-element kernels
// (lumped mass, masslike): the Jacobian matrix J = X' dN (locjac!,
// src/MatrixUtilityModule.jl:60-68) and the manifold Jacobian of
// Jacobianmdim (src/IntegDomainModule.jl:504-549, 567-602; Jacobian in
// src/FESetModule.jl:426-435, 479-489).  FP64.
#pragma once

#include <cstdint>

namespace fegpu {

constexpr double kPi = 3.14159265358979323846;  // pi as an FP64 number

// J[s][m] = sum_k x_k[s] dN_k[m] over the element's nodes (xyz: [nnodes][4])
template <int NNE, int MDIM>
__device__ inline void jacobian_matrix(const int32_t *ce, const double *xyz, const double *dNq,
                                       double (&J)[3][MDIM]) {
#pragma unroll
  for (int s = 0; s < 3; ++s)
#pragma unroll
    for (int m = 0; m < MDIM; ++m) J[s][m] = 0.0;
  for (int k = 0; k < NNE; ++k) {
    const double *x = xyz + 4 * static_cast<int64_t>(ce[k]);
#pragma unroll
    for (int m = 0; m < MDIM; ++m) {
      const double d = dNq[k * MDIM + m];
#pragma unroll
      for (int s = 0; s < 3; ++s) J[s][m] = fma(x[s], d, J[s][m]);
    }
  }
}

// the first coordinate of the point, sum_k N_k x_k (loc[1] of locjac!)
template <int NNE>
__device__ inline double point_r(const int32_t *ce, const double *xyz, const double *Nq) {
  double r = 0.0;
  for (int k = 0; k < NNE; ++k) r = fma(Nq[k], xyz[4 * static_cast<int64_t>(ce[k])], r);
  return r;
}

// Jacobianmdim: a 3-manifold's volume Jacobian (m = 3); a 2-manifold's
// surface Jacobian (the 2x2 determinant for planar coordinates, the norm of
// the tangents' cross product otherwise), for m = 3 times the other dimension
// or, on an axisymmetric domain, times 2 pi r (r: the point's first
// coordinate; src/IntegDomainModule.jl:504-549).
template <int MDIM>
__device__ inline double jacobian_mdim(const double (&J)[3][MDIM], int sdim, double otherdim,
                                       int m, int axisym = 0, double r = 0.0) {
  double Jac;
  if constexpr (MDIM == 3) {
    Jac = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
          J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  } else {
    if (sdim == 2) {
      Jac = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    } else {
      const double c1 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
      const double c2 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
      const double c3 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
      Jac = sqrt(c1 * c1 + c2 * c2 + c3 * c3);
    }
    if (m == 3) Jac = axisym ? Jac * 2.0 * kPi * r : Jac * otherdim;
  }
  return Jac;
}

}  // namespace fegpu
