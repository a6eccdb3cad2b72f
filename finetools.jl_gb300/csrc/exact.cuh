// FP64 element blocks in the reference's own operation order, and the row
// gather that sums them in the reference's own order.
//
// The reference evaluates every element matrix with separately rounded IEEE
// double operations in a fixed order, appends the lower triangle (by local
// index) of each one to a COO list in element order, sums duplicates in that
// order (sparse(I, J, V)) and completes the symmetric matrix as S + S' with
// the diagonal halved (src/AssemblyModule.jl:500-583).  This path repeats each
// of those roundings, so the assembled matrix equals the reference algorithm's
// bit for bit -- including which entries come out exactly zero and are left
// out of the S + S' result:
//
//   element phase (k_blocks_exact): one tile of elements per CTA, element
//     order; per point locjac!/Jacobian/gradN! (src/MatrixUtilityModule.jl:
//     60-68, src/FESetModule.jl:479-544) with no contraction into FMA, then
//       diffusion  add_mggt_ut_only! / add_gkgt_ut_only!
//                  (src/MatrixUtilityModule.jl:84-153),
//       elasticity DB = (Jac w) (D B) and Ke += B' DB, upper triangle,
//                  add_btdb_ut_only! (src/MatrixUtilityModule.jl:189-216)
//                  with B from blmat! (src/DeforModelRedModule.jl:447-472);
//     B's structural zeros (and, for an isotropic D, D's) are skipped: a
//     product with an exact zero adds nothing but the sign of a zero sum, so
//     every nonzero result is unchanged.  The upper node-pair blocks (the
//     diagonal ones mirrored, complete_lt!) go to an FP64 ring, chunk by
//     chunk of elements.
//   gather phase (gather_node_exact): one warp per node; its rows are summed
//     over the incident elements in element order into two buckets per entry:
//     contributions whose local row index is >= the local column index are
//     the reference's S(r, c) triples, the others its S(c, r) triples.  The
//     stored value is S(r, c) + S(c, r), on the diagonal (S + S) / 2: the
//     reference's S + S' step.  An unsymmetric assembly (SysmatAssemblerSparse)
//     keeps one bucket: S(r, c).
#pragma once

#include "elements.cuh"
#include "softf64.cuh"

namespace fegpu {

constexpr int kExactThreads = 256;

// separately rounded FP64 products and sums on the FP64 unit (xm, xa), and
// sums over the quadrature points (xs<SOFT>): with SOFT on the integer units
// (sf_add, bit-identical to the FP64 unit's sum), so that GB300's narrow FP64
// pipe and its integer issue share the element blocks.  That pays where the
// block kernel keeps enough warps per SM to cover the integer chains' latency:
// T10 elasticity, two CTAs of 256 threads (35.3 -> 31.3 ms at 60^3), and H20
// elasticity with one element per tile, three CTAs per SM (34.9 -> 31.3 ms at
// 40^3; with three elements per tile and one CTA per SM the integer sums
// made it slower, 40.0 ms).  Where the sums are all point sums (H8
// diffusion) the FP64 unit alone is faster.
__device__ __forceinline__ double xm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xa(double a, double b) { return __dadd_rn(a, b); }
template <bool SOFT>
__device__ __forceinline__ double xs(double a, double b) {
  if constexpr (SOFT) return sf_add(a, b);
  else return __dadd_rn(a, b);
}

// values kept per (element, point, node) for the block phase: the weighted
// gradients (diffusion), or the nonzeros of the node's three DB columns
// (elasticity: 9 for an isotropic D, 18 for a general one)
__host__ __device__ constexpr int exact_node_values(int form) {
  return form == F_ELAST_ISO ? 9 : (form == F_ELAST_GEN ? 18 : 3);
}

struct ExactLayout {
  size_t tab, X, G, V, Jw, conn, pairs, total;
};

__host__ __device__ inline ExactLayout exact_layout(int nne, int mdim, int npts, int te, int form) {
  ExactLayout L;
  size_t o = 0;
  L.tab = o;
  o += sizeof(double) * (npts * nne + npts * nne * mdim + npts);
  o = align_up(o, 16);
  L.X = o;
  o += sizeof(double) * te * nne * 3;
  L.G = o;
  o += sizeof(double) * te * npts * nne * mdim;
  L.V = o;
  o += sizeof(double) * te * npts * nne * exact_node_values(form);
  L.Jw = o;
  o += sizeof(double) * te * npts;
  L.conn = o;
  o += sizeof(int32_t) * te * nne;
  L.pairs = o;
  o += 2 * (nne * (nne + 1) / 2);
  L.total = align_up(o, 16);
  return L;
}

// Isotropic D entries of element es: D[j][j], D[m][j] (m != j), D[3][3].
// A per-element (lambda, mu) pair gives lambda + 2 mu, lambda, mu, formed as
// the 6x6 D is (2 mu exact, one rounding of the sum).
__device__ __forceinline__ void exact_iso_entries(const KArgs &a, int64_t es, double &d0,
                                                  double &d1, double &d3) {
  if (a.coef_kind == FEGPU_COEF_ISO_LAME) {
    const double lam = a.coef[2 * es], mu = a.coef[2 * es + 1];
    d0 = xa(lam, xm(2.0, mu));
    d1 = lam;
    d3 = mu;
  } else {
    d0 = a.cconst[0];
    d1 = a.cconst[1];
    d3 = a.cconst[2];
  }
}

template <int ET, int FORM>
__global__ void __launch_bounds__(kExactThreads) k_blocks_exact(const KArgs a) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  constexpr bool ELAST = FORM == F_ELAST_ISO || FORM == F_ELAST_GEN;
  constexpr bool SOFT = ELAST && (ET == FEGPU_T10 || ET == FEGPU_H20);  // point sums on the integer units
  constexpr int NDN = ELAST ? 3 : 1;
  constexpr int BS = NDN * NDN;
  constexpr int NBLK = NNE * (NNE + 1) / 2;
  constexpr int NV = exact_node_values(FORM);
  static_assert(!ELAST || MDIM == 3, "elasticity needs a solid element");
  extern __shared__ __align__(16) unsigned char smem[];
  const int npts = a.npts, te = a.te;
  const ExactLayout L = exact_layout(NNE, MDIM, npts, te, FORM);
  double *sN = reinterpret_cast<double *>(smem + L.tab);
  double *sdN = sN + npts * NNE;
  double *sw = sdN + npts * NNE * MDIM;
  double *sX = reinterpret_cast<double *>(smem + L.X);
  double *sG = reinterpret_cast<double *>(smem + L.G);
  double *sV = reinterpret_cast<double *>(smem + L.V);
  double *sJw = reinterpret_cast<double *>(smem + L.Jw);
  int32_t *sConn = reinterpret_cast<int32_t *>(smem + L.conn);
  uint8_t *sPair = smem + L.pairs;
  const int tid = threadIdx.x, nth = blockDim.x;

  for (int i = tid; i < npts * NNE * (MDIM + 1) + npts; i += nth) sN[i] = a.tab[i];
  for (int i = tid; i < NBLK; i += nth) {
    int r = i, pa = 0;
    while (r >= NNE - pa) {
      r -= NNE - pa;
      ++pa;
    }
    sPair[2 * i] = static_cast<uint8_t>(pa);
    sPair[2 * i + 1] = static_cast<uint8_t>(pa + r);
  }
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
    }
    __syncthreads();

    // ---- geometry per (element, point): gradients and the point factors
    for (int i = tid; i < ne * npts; i += nth) {
      const int e = i / npts, q = i - e * npts;
      double *g = sG + (static_cast<size_t>(e) * npts + q) * NNE * MDIM;
      const double Jac = geometry_qp<NNE, MDIM, true, double, double, true>(
          sX + e * NNE * 3, sdN + q * NNE * MDIM, a.sdim, 1, a.otherdim, g, nullptr,
          sN + q * NNE, a.axisym);
      if constexpr (ELAST) {
        sJw[e * npts + q] = xm(Jac, sw[q]);  // Jac * w[j]
      } else {
        // mult = (c Jac) w, av = mult g (add_mggt_ut_only!), or
        // kg = (Jac w) (kappa g) (add_gkgt_ut_only!)
        double *wg = sV + (static_cast<size_t>(e) * npts + q) * NNE * MDIM;
        qp_weights<NNE, MDIM, FORM, double>(a, eb + e, q, npts, Jac, sw[q], g, wg,
                                            sJw + e * npts + q);
      }
    }
    __syncthreads();

    if constexpr (ELAST) {
      // ---- DB columns of every node: DB[m][(b,j)] = (Jac w) sum_p D[m][p] B[p][(b,j)]
      for (int i = tid; i < ne * npts * NNE; i += nth) {
        const int eq = i / NNE, b = i - eq * NNE;
        const int e = eq / npts, q = eq - e * npts;
        const int64_t es = eb + e;
        const double *gb = sG + (static_cast<size_t>(eq) * NNE + b) * 3;
        const double gx = gb[0], gy = gb[1], gz = gb[2];
        const double Jw = sJw[eq];
        double *v = sV + (static_cast<size_t>(eq) * NNE + b) * NV;
        if constexpr (FORM == F_ELAST_ISO) {
          // P_j = Jw (D[j][j] g_j), Q_j = Jw (D[m][j] g_j) (m != j),
          // S_k = Jw (D[3][3] g_k): the nonzeros of DB's columns (b, j)
          double d0, d1, d3;
          exact_iso_entries(a, es, d0, d1, d3);
          v[0] = xm(Jw, xm(d0, gx));
          v[1] = xm(Jw, xm(d0, gy));
          v[2] = xm(Jw, xm(d0, gz));
          v[3] = xm(Jw, xm(d1, gx));
          v[4] = xm(Jw, xm(d1, gy));
          v[5] = xm(Jw, xm(d1, gz));
          v[6] = xm(Jw, xm(d3, gx));
          v[7] = xm(Jw, xm(d3, gy));
          v[8] = xm(Jw, xm(d3, gz));
        } else {
          // column (b,x) of B: rows 0 (g_x), 3 (g_y), 4 (g_z); (b,y): 1 (g_y),
          // 3 (g_x), 5 (g_z); (b,z): 2 (g_z), 4 (g_x), 5 (g_y)
          // D at this point: C = cf(loc, J, i, j) is evaluated at every point
          // (src/FEMMBaseModule.jl:1802); constant, per element or per point
          const double *D = a.coef_kind == FEGPU_COEF_PER_ELEMENT ? a.coef + es * 36
                            : a.coef_kind == FEGPU_COEF_PER_QP   ? a.coef + (es * npts + q) * 36
                                                                 : a.cconst;
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            const double *Dm = D + 6 * m;
            v[3 * m + 0] = xm(Jw, xa(xa(xm(Dm[0], gx), xm(Dm[3], gy)), xm(Dm[4], gz)));
            v[3 * m + 1] = xm(Jw, xa(xa(xm(Dm[1], gy), xm(Dm[3], gx)), xm(Dm[5], gz)));
            v[3 * m + 2] = xm(Jw, xa(xa(xm(Dm[2], gz), xm(Dm[4], gx)), xm(Dm[5], gy)));
          }
        }
      }
      __syncthreads();
    }

    // ---- node-pair blocks (a <= b), summed over the points in point order
    for (int i = tid; i < ne * NBLK; i += nth) {
      const int e = i / NBLK, blk = i - e * NBLK;
      const int pa = sPair[2 * blk], pb = sPair[2 * blk + 1];
      double *out = a.ke64 + ((eb + e - a.e0) * NBLK + blk) * BS;
      if constexpr (!ELAST) {
        const double *ga = sG + static_cast<size_t>(e) * npts * NNE * MDIM + pa * MDIM;
        const double *wb = sV + static_cast<size_t>(e) * npts * NNE * MDIM + pb * MDIM;
        double s = 0.0;
        for (int q = 0; q < npts; ++q) {
          const double *x = ga + q * NNE * MDIM;
          const double *y = wb + q * NNE * MDIM;
          if constexpr (FORM == F_DIFF_ISO) {
            // Ke[a][b] += g[a][p] * av[b][p], one p at a time
#pragma unroll
            for (int m = 0; m < MDIM; ++m) s = xs<SOFT>(s, xm(x[m], y[m]));
          } else {
            double acc = xm(x[0], y[0]);
#pragma unroll
            for (int m = 1; m < MDIM; ++m) acc = xa(acc, xm(x[m], y[m]));
            s = xs<SOFT>(s, acc);
          }
        }
        out[0] = s;
      } else {
        double K[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) K[r][c] = 0.0;
        const bool diag = pa == pb;
        for (int q = 0; q < npts; ++q) {
          const double *ga = sG + ((static_cast<size_t>(e) * npts + q) * NNE + pa) * 3;
          const double *v = sV + ((static_cast<size_t>(e) * npts + q) * NNE + pb) * NV;
          const double ax = ga[0], ay = ga[1], az = ga[2];
          // Ke[(a,i)][(b,j)] += sum over B column (a,i)'s rows p, in increasing
          // order, of B[p][(a,i)] * DB[p][(b,j)]
          if constexpr (FORM == F_ELAST_ISO) {
            const double Px = v[0], Py = v[1], Pz = v[2];
            const double Qx = v[3], Qy = v[4], Qz = v[5];
            const double Sx = v[6], Sy = v[7], Sz = v[8];
            // (the first sum of each diagonal entry's three products on the
            // integer units too: 30.2 -> 29.4 ms at T10 60^3)
            K[0][0] = xs<SOFT>(K[0][0], xa(xs<SOFT>(xm(ax, Px), xm(ay, Sy)), xm(az, Sz)));
            K[0][1] = xs<SOFT>(K[0][1], xa(xm(ax, Qy), xm(ay, Sx)));
            K[0][2] = xs<SOFT>(K[0][2], xa(xm(ax, Qz), xm(az, Sx)));
            K[1][1] = xs<SOFT>(K[1][1], xa(xs<SOFT>(xm(ay, Py), xm(ax, Sx)), xm(az, Sz)));
            K[1][2] = xs<SOFT>(K[1][2], xa(xm(ay, Qz), xm(az, Sy)));
            K[2][2] = xs<SOFT>(K[2][2], xa(xs<SOFT>(xm(az, Pz), xm(ax, Sx)), xm(ay, Sy)));
            if (!diag) {
              K[1][0] = xs<SOFT>(K[1][0], xa(xm(ay, Qx), xm(ax, Sy)));
              K[2][0] = xs<SOFT>(K[2][0], xa(xm(az, Qx), xm(ax, Sz)));
              K[2][1] = xs<SOFT>(K[2][1], xa(xm(az, Qy), xm(ay, Sz)));
            }
          } else {
            // v[3 m + j] = DB[m][(b,j)]; column (a,x): rows 0, 3, 4;
            // (a,y): 1, 3, 5; (a,z): 2, 4, 5
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              if (!diag || j >= 0) {
                K[0][j] = xs<SOFT>(K[0][j], xa(xa(xm(ax, v[j]), xm(ay, v[9 + j])), xm(az, v[12 + j])));
              }
              if (!diag || j >= 1) {
                K[1][j] = xs<SOFT>(K[1][j], xa(xa(xm(ay, v[3 + j]), xm(ax, v[9 + j])), xm(az, v[15 + j])));
              }
              if (!diag || j >= 2) {
                K[2][j] = xs<SOFT>(K[2][j], xa(xa(xm(az, v[6 + j]), xm(ax, v[12 + j])), xm(ay, v[15 + j])));
              }
            }
          }
        }
        if (diag) {  // complete_lt!: the lower triangle mirrors the upper
          K[1][0] = K[0][1];
          K[2][0] = K[0][2];
          K[2][1] = K[1][2];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) out[r * 3 + c] = K[r][c];
      }
    }
  }
}

template <int ET, int FORM>
int launch_blocks_exact_t(const KArgs &a, int num_sms, cudaStream_t s) {
  constexpr int NNE = ElemT<ET>::NNE, MDIM = ElemT<ET>::MDIM;
  const ExactLayout L = exact_layout(NNE, MDIM, a.npts, a.te, FORM);
  auto kern = k_blocks_exact<ET, FORM>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(L.total)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kExactThreads, L.total));
  if (per_sm < 1) per_sm = 1;
  const int64_t nel = a.e1 - a.e0;
  if (nel <= 0) return 0;
  const int64_t ntiles = (nel + a.te - 1) / a.te;
  const int grid = static_cast<int>(std::min<int64_t>(ntiles, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kExactThreads, L.total, s>>>(a);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace fegpu
