// Conjugate gradients on the resident CSR matrix: conjugategradient
// (src/AlgoBaseModule.jl:425-445), run on the device.
//
// The iteration is the reference's, step for step:
//   gt = A x0 - b;  d = gt
//   repeat maxiter times:
//     Ad = A d;  rho = d.Ad;  alpha = -(gt.d) / rho;  x += alpha d
//     gt = A x - b;  beta = (gt.Ad) / rho;  d = beta d - gt
// The scalars stay on the device (no host round trip per iteration); dot
// products are reduced in a fixed order (per-block trees, then one block over
// the partial sums), so results are reproducible run to run.  Element-wise
// updates use separately rounded multiply and add, as the reference's
// broadcasts.
#include <algorithm>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

constexpr int kThreads = 256;
constexpr int kDotBlocks = 456;  // 3 x 152 SMs

enum Scalar { S_RHO = 0, S_ALPHA = 1, S_BETA = 2, S_TMP = 3, S_COUNT = 4 };

__global__ void k_dot_partial(const double *a, const double *b, int64_t n, double *part) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    s = fma(a[i], b[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// op 0: scal[S_RHO] = sum; op 1: scal[S_ALPHA] = -sum / rho; op 2: scal[S_BETA] = sum / rho
__global__ void k_dot_final(const double *part, int nparts, double *scal, int op) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kThreads) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double v = sh[0];
    if (op == 0) scal[S_RHO] = v;
    else if (op == 1) scal[S_ALPHA] = -v / scal[S_RHO];
    else scal[S_BETA] = v / scal[S_RHO];
  }
}

// y = A x - b (warp per row; fixed lane order and shuffle tree)
__global__ void k_residual(const int64_t *rowptr, const int32_t *colind, const double *val,
                           int64_t nrows, const double *__restrict__ x, const double *b,
                           double *y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t r = w0; r < nrows; r += nw) {
    double s = 0.0;
    for (int64_t p = rowptr[r] + lane; p < rowptr[r + 1]; p += 32) s = fma(val[p], x[colind[p]], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) y[r] = b ? __dsub_rn(s, b[r]) : s;
  }
}

__global__ void k_axpy(double *x, const double *d, const double *scal, int64_t n) {
  const double alpha = scal[S_ALPHA];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] = __dadd_rn(x[i], __dmul_rn(alpha, d[i]));
}

__global__ void k_new_direction(double *d, const double *gt, const double *scal, int64_t n) {
  const double beta = scal[S_BETA];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    d[i] = __dsub_rn(__dmul_rn(beta, d[i]), gt[i]);
}

int blocks_for(int64_t n) {
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16)));
}

}  // namespace
}  // namespace fegpu

using namespace fegpu;

extern "C" int fegpu_matrix_cg(fegpu_matrix *K, const double *b, const double *x0, int maxiter,
                               double *x) {
  try {
    FEGPU_REQUIRE(K && b && x0 && x, "null handle");
    FEGPU_REQUIRE(maxiter >= 0, "maxiter must be non-negative");
    const fegpu_dofmap *dm = K->dm;
    fegpu_context *ctx = dm->femm->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = dm->ndof;
    DevBuf vb, vx, vgt, vd, vAd, part, scal;
    for (DevBuf *v : {&vb, &vx, &vgt, &vd, &vAd}) v->alloc(sizeof(double) * std::max<int64_t>(n, 1));
    part.alloc(sizeof(double) * kDotBlocks);
    scal.alloc(sizeof(double) * S_COUNT);
    FEGPU_CUDA(cudaMemcpyAsync(vb.p, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    FEGPU_CUDA(cudaMemcpyAsync(vx.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    const int64_t *rp = dm->rowptr.as<int64_t>();
    const int32_t *ci = dm->colind.as<int32_t>();
    const double *val = K->val.as<double>();
    const int gspmv = blocks_for(n * 32), gvec = blocks_for(n);
    auto residual = [&](const double *xin, const double *bin, double *y) {
      k_residual<<<gspmv, kThreads, 0, s>>>(rp, ci, val, n, xin, bin, y);
      FEGPU_CUDA(cudaGetLastError());
    };
    auto dot = [&](const double *u, const double *v, int op) {
      k_dot_partial<<<kDotBlocks, kThreads, 0, s>>>(u, v, n, part.as<double>());
      k_dot_final<<<1, kThreads, 0, s>>>(part.as<double>(), kDotBlocks, scal.as<double>(), op);
      FEGPU_CUDA(cudaGetLastError());
    };
    residual(vx.as<double>(), vb.as<double>(), vgt.as<double>());  // gt = A x - b
    FEGPU_CUDA(cudaMemcpyAsync(vd.p, vgt.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    for (int it = 0; it < maxiter; ++it) {
      residual(vd.as<double>(), nullptr, vAd.as<double>());         // Ad = A d
      dot(vd.as<double>(), vAd.as<double>(), 0);                     // rho = d.Ad
      dot(vgt.as<double>(), vd.as<double>(), 1);                     // alpha = -(gt.d)/rho
      k_axpy<<<gvec, kThreads, 0, s>>>(vx.as<double>(), vd.as<double>(), scal.as<double>(), n);
      residual(vx.as<double>(), vb.as<double>(), vgt.as<double>());  // gt = A x - b
      dot(vgt.as<double>(), vAd.as<double>(), 2);                    // beta = (gt.Ad)/rho
      k_new_direction<<<gvec, kThreads, 0, s>>>(vd.as<double>(), vgt.as<double>(),
                                                scal.as<double>(), n);
      FEGPU_CUDA(cudaGetLastError());
      ctx->launches += 9;
    }
    FEGPU_CUDA(cudaMemcpyAsync(x, vx.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
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
