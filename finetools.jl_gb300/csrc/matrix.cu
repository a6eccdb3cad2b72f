// Matrix utilities: SpMV, CSC export (with the exact-zero dropping of the
// symmetric assembler), and the generic COO assembler for element matrices
// formed on the host.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

int grid_of(int64_t n, int per = 256) {
  return static_cast<int>(std::min<int64_t>(std::max<int64_t>((n + per - 1) / per, 1), 1 << 20));
}

template <typename F>
void cub_call(fegpu_context *ctx, DevBuf &tmp, F &&f) {
  size_t bytes = 0;
  FEGPU_CUDA(f(nullptr, bytes));
  tmp.alloc(bytes);
  FEGPU_CUDA(f(tmp.p, bytes));
  (void)ctx;
}

// y = K x, one warp per row.
__global__ void k_spmv(const int64_t *rowptr, const int32_t *colind, const double *val,
                       int64_t nrows, const double *__restrict__ x, double *y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < nrows; r += nw) {
    double s = 0.0;
    for (int64_t p = rowptr[r] + lane; p < rowptr[r + 1]; p += 32) s = fma(val[p], x[colind[p]], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) y[r] = s;
  }
}

// nonzeros per row (one warp per row)
__global__ void k_row_nonzeros(const int64_t *rowptr, const double *val, int64_t nrows,
                               int64_t *cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < nrows; r += nw) {
    int64_t c = 0;
    for (int64_t p = rowptr[r] + lane; p < rowptr[r + 1]; p += 32) c += (val[p] != 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[r] = c;
  }
}

// compaction of one row per warp; keeps the column order
__global__ void k_compact(const int64_t *rowptr, const int32_t *colind, const double *val,
                          int64_t nrows, const int64_t *newptr, int64_t *rowval1, double *nzval) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < nrows; r += nw) {
    int64_t out = newptr[r];
    for (int64_t p0 = rowptr[r]; p0 < rowptr[r + 1]; p0 += 32) {
      const int64_t p = p0 + lane;
      const bool keep = p < rowptr[r + 1] && val[p] != 0.0;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int64_t o = out + __popc(m & ((1u << lane) - 1u));
        rowval1[o] = static_cast<int64_t>(colind[p]) + 1;
        nzval[o] = val[p];
      }
      out += __popc(m);
    }
  }
}

__global__ void k_widen1(const int32_t *src, int64_t n, int64_t *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = static_cast<int64_t>(src[i]) + 1;
}

__global__ void k_plus1(const int64_t *src, int64_t n, int64_t *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] + 1;
}

}  // namespace

void spmv(const fegpu_dofmap *dm, const double *val, const double *x, double *y, cudaStream_t s) {
  const int64_t n = dm->ndof;
  k_spmv<<<grid_of(n * 32), 256, 0, s>>>(dm->rowptr.as<int64_t>(), dm->colind.as<int32_t>(), val,
                                         n, x, y);
  FEGPU_CUDA(cudaGetLastError());
}

int64_t count_nonzeros(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val) {
  cudaStream_t s = ctx->stream;
  const int64_t n = dm->ndof;
  DevBuf cnt, sum, tmp;
  cnt.alloc(sizeof(int64_t) * (n + 1));
  sum.alloc(sizeof(int64_t));
  k_row_nonzeros<<<grid_of(n * 32), 256, 0, s>>>(dm->rowptr.as<int64_t>(), val, n,
                                                 cnt.as<int64_t>());
  FEGPU_CUDA(cudaGetLastError());
  cub_call(ctx, tmp, [&](void *t, size_t &b) {
    return cub::DeviceReduce::Sum(t, b, cnt.as<int64_t>(), sum.as<int64_t>(), n, s);
  });
  int64_t h = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&h, sum.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  return h;
}

// CSC (== CSR of the symmetric matrix), 1-based.  val == nullptr: pattern only.
namespace {
// warp per row i: each entry (i, j) finds i in row j (sorted columns) and
// writes its value there
__global__ void k_transpose_vals(const int64_t *rowptr, const int32_t *colind, const double *val,
                                 int64_t nrows, double *out) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = w0; i < nrows; i += nw) {
    for (int64_t p = rowptr[i] + lane; p < rowptr[i + 1]; p += 32) {
      const int32_t j = colind[p];
      int64_t lo = rowptr[j], hi = rowptr[j + 1] - 1;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (colind[mid] < i) lo = mid + 1;
        else hi = mid;
      }
      out[lo] = val[p];
    }
  }
}
}  // namespace

namespace {
__device__ __forceinline__ int64_t lower_bound32(const int32_t *a, int64_t lo, int64_t hi, int32_t v) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// per column j in [c0, c1): the slice of its (sorted) row list in [r0, r1)
// and the entries it keeps (all, or the nonzero ones when drop_zeros)
__global__ void k_block_count(const int64_t *rowptr, const int32_t *colind, const double *val,
                              int64_t c0, int64_t c1, int32_t r0, int32_t r1, int drop_zeros,
                              int64_t *first, int64_t *last, int64_t *cnt) {
  for (int64_t j = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < c1;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = lower_bound32(colind, rowptr[j], rowptr[j + 1], r0);
    const int64_t b = lower_bound32(colind, a, rowptr[j + 1], r1);
    first[j - c0] = a;
    last[j - c0] = b;
    int64_t n = b - a;
    if (drop_zeros) {
      n = 0;
      for (int64_t p = a; p < b; ++p) n += (val[p] != 0.0);
    }
    cnt[j - c0] = n;
  }
}

// one warp per column; ballot compaction keeps the row order
__global__ void k_block_copy(const int32_t *colind, const double *val, const int64_t *first,
                             const int64_t *last, const int64_t *ptr, int64_t ncols, int32_t r0,
                             int drop_zeros, int64_t *rowval, double *nzval) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w0; j < ncols; j += nw) {
    int64_t out = ptr[j];
    for (int64_t p0 = first[j]; p0 < last[j]; p0 += 32) {
      const int64_t p = p0 + lane;
      const bool keep = p < last[j] && (!drop_zeros || val[p] != 0.0);
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int64_t o = out + __popc(m & ((1u << lane) - 1u));
        rowval[o] = static_cast<int64_t>(colind[p]) - r0 + 1;
        nzval[o] = val[p];
      }
      out += __popc(m);
    }
  }
}
}  // namespace

int64_t copy_block_csc(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val, int64_t r0,
                       int64_t r1, int64_t c0, int64_t c1, int drop_zeros, int64_t *colptr,
                       int64_t *rowval, double *nzval) {
  cudaStream_t s = ctx->stream;
  const int64_t nc = c1 - c0;
  DevBuf first, last, cnt, ptr, tmp, rv, nz;
  first.alloc(sizeof(int64_t) * (nc + 1));
  last.alloc(sizeof(int64_t) * (nc + 1));
  cnt.alloc(sizeof(int64_t) * (nc + 1));
  ptr.alloc(sizeof(int64_t) * (nc + 1));
  FEGPU_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int64_t) * (nc + 1), s));
  if (nc > 0) {
    k_block_count<<<grid_of(nc), 256, 0, s>>>(dm->rowptr.as<int64_t>(), dm->colind.as<int32_t>(),
                                              val, c0, c1, static_cast<int32_t>(r0),
                                              static_cast<int32_t>(r1), drop_zeros,
                                              first.as<int64_t>(), last.as<int64_t>(),
                                              cnt.as<int64_t>());
    FEGPU_CUDA(cudaGetLastError());
  }
  cub_call(ctx, tmp, [&](void *t, size_t &b) {
    return cub::DeviceScan::ExclusiveSum(t, b, cnt.as<int64_t>(), ptr.as<int64_t>(), nc + 1, s);
  });
  int64_t nnz = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&nnz, ptr.as<int64_t>() + nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  if (!colptr) return nnz;  // size query
  rv.alloc(sizeof(int64_t) * (nnz + 1));
  nz.alloc(sizeof(double) * (nnz + 1));
  if (nnz > 0)
    k_block_copy<<<grid_of(nc * 32), 256, 0, s>>>(dm->colind.as<int32_t>(), val, first.as<int64_t>(),
                                                  last.as<int64_t>(), ptr.as<int64_t>(), nc,
                                                  static_cast<int32_t>(r0), drop_zeros,
                                                  rv.as<int64_t>(), nz.as<double>());
  FEGPU_CUDA(cudaGetLastError());
  k_plus1<<<grid_of(nc + 1), 256, 0, s>>>(ptr.as<int64_t>(), nc + 1, first.as<int64_t>());
  FEGPU_CUDA(cudaGetLastError());
  FEGPU_CUDA(cudaMemcpyAsync(colptr, first.p, sizeof(int64_t) * (nc + 1), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaMemcpyAsync(rowval, rv.p, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaMemcpyAsync(nzval, nz.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  return nnz;
}

void transpose_values(const fegpu_dofmap *dm, const double *val, double *out, cudaStream_t s) {
  const int64_t n = dm->ndof;
  if (n <= 0) return;
  k_transpose_vals<<<grid_of(n * 32), 256, 0, s>>>(dm->rowptr.as<int64_t>(),
                                                   dm->colind.as<int32_t>(), val, n, out);
  FEGPU_CUDA(cudaGetLastError());
}

void copy_csc(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val, int drop_zeros,
              int64_t *colptr, int64_t *rowval, double *nzval) {
  cudaStream_t s = ctx->stream;
  const int64_t n = dm->ndof, nnz = dm->nnz;
  DevBuf ptr, rv, nz, tmp;
  ptr.alloc(sizeof(int64_t) * (n + 1));
  if (!drop_zeros || val == nullptr) {
    rv.alloc(sizeof(int64_t) * (nnz + 1));
    k_plus1<<<grid_of(n + 1), 256, 0, s>>>(dm->rowptr.as<int64_t>(), n + 1, ptr.as<int64_t>());
    k_widen1<<<grid_of(nnz), 256, 0, s>>>(dm->colind.as<int32_t>(), nnz, rv.as<int64_t>());
    FEGPU_CUDA(cudaGetLastError());
    FEGPU_CUDA(cudaMemcpyAsync(colptr, ptr.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
    FEGPU_CUDA(cudaMemcpyAsync(rowval, rv.p, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, s));
    if (val && nzval)
      FEGPU_CUDA(cudaMemcpyAsync(nzval, val, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
    return;
  }
  DevBuf cnt;
  cnt.alloc(sizeof(int64_t) * (n + 1));
  FEGPU_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int64_t) * (n + 1), s));
  k_row_nonzeros<<<grid_of(n * 32), 256, 0, s>>>(dm->rowptr.as<int64_t>(), val, n,
                                                 cnt.as<int64_t>());
  FEGPU_CUDA(cudaGetLastError());
  cub_call(ctx, tmp, [&](void *t, size_t &b) {
    return cub::DeviceScan::ExclusiveSum(t, b, cnt.as<int64_t>(), ptr.as<int64_t>(), n + 1, s);
  });
  int64_t kept = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&kept, ptr.as<int64_t>() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  rv.alloc(sizeof(int64_t) * (kept + 1));
  nz.alloc(sizeof(double) * (kept + 1));
  k_compact<<<grid_of(n * 32), 256, 0, s>>>(dm->rowptr.as<int64_t>(), dm->colind.as<int32_t>(),
                                            val, n, ptr.as<int64_t>(), rv.as<int64_t>(),
                                            nz.as<double>());
  DevBuf ptr1;
  ptr1.alloc(sizeof(int64_t) * (n + 1));
  k_plus1<<<grid_of(n + 1), 256, 0, s>>>(ptr.as<int64_t>(), n + 1, ptr1.as<int64_t>());
  FEGPU_CUDA(cudaGetLastError());
  FEGPU_CUDA(cudaMemcpyAsync(colptr, ptr1.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaMemcpyAsync(rowval, rv.p, sizeof(int64_t) * kept, cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaMemcpyAsync(nzval, nz.p, sizeof(double) * kept, cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fegpu
// ---------------------------------------------------------------------------
// Generic assembler: startassembly!/assemble!/makematrix! of
// SysmatAssemblerSparse(Symm) (src/AssemblyModule.jl:209-329, 454-583) for
// element matrices formed by the caller.  makematrix! runs on the device: a
// stable radix sort of (column, row) keys keeps duplicates in input order,
// and each run of equal keys is summed left to right, which is the combine
// order of Julia's sparse(I, J, V).  The symmetric variant then forms S + S'
// (exact zeros not stored) and halves the diagonal.  Device forms that
// produce rectangular COO data (bilform_masslike) hand their keys and values
// to the same reduction.

namespace fegpu {
namespace {

__global__ void k_make_keys(const int64_t *I, const int64_t *J, int64_t n, uint64_t *key,
                            int64_t *idx) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    key[t] = (static_cast<uint64_t>(J[t] - 1) << 32) | static_cast<uint64_t>(I[t] - 1);
    idx[t] = t;
  }
}

__global__ void k_iota(int64_t n, int64_t *idx) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    idx[t] = t;
}

__global__ void k_heads(const uint64_t *key, int64_t n, int64_t *head) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    head[t] = (t == 0 || key[t] != key[t - 1]) ? 1 : 0;
}

// sum each run of equal keys left to right (input order)
__global__ void k_reduce_runs(const uint64_t *key, const int64_t *order, const double *V,
                              const int64_t *seg, int64_t n, uint64_t *ukey, double *uval) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t != 0 && key[t] == key[t - 1]) continue;
    double s = V[order[t]];
    int64_t u = t + 1;
    while (u < n && key[u] == key[t]) {
      s = s + V[order[u]];
      ++u;
    }
    const int64_t o = seg[t];
    ukey[o] = key[t];
    uval[o] = s;
  }
}

// S + S': entries of S are tagged 0..n-1, mirrored entries n..2n-1
__global__ void k_mirror(const uint64_t *key, const double *val, int64_t n, uint64_t *k2,
                         double *v2, int64_t *tag) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = key[t] >> 32, r = key[t] & 0xffffffffu;
    k2[t] = key[t];
    v2[t] = val[t];
    tag[t] = t;
    k2[n + t] = (r << 32) | c;
    v2[n + t] = val[t];
    tag[n + t] = n + t;
  }
}

// after the stable sort a run is (S) or (S, S') or (S'): v = s + t with the
// missing one as 0.0; exact zeros are not kept, the diagonal is halved
__global__ void k_symm_runs(const uint64_t *key, const double *v2, const int64_t *order,
                            int64_t n2, int64_t nS, uint64_t *okey, double *oval, int64_t *keep) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2;
       t += (int64_t)gridDim.x * blockDim.x) {
    keep[t] = 0;
    if (t != 0 && key[t] == key[t - 1]) continue;
    double sv = 0.0, tv = 0.0;
    bool hs = false, ht = false;
    for (int64_t u = t; u < n2 && key[u] == key[t]; ++u) {
      if (order[u] < nS) { sv = v2[order[u]]; hs = true; }
      else { tv = v2[order[u]]; ht = true; }
    }
    double v = hs && ht ? sv + tv : (hs ? sv + 0.0 : 0.0 + tv);
    const uint64_t c = key[t] >> 32, r = key[t] & 0xffffffffu;
    if (v != 0.0) {
      if (r == c) v *= 0.5;
      keep[t] = 1;
    }
    okey[t] = key[t];
    oval[t] = v;
  }
}

__global__ void k_scatter_kept(const uint64_t *okey, const double *oval, const int64_t *keep,
                               const int64_t *pos, int64_t n, uint64_t *key, double *val) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    if (keep[t]) {
      key[pos[t]] = okey[t];
      val[pos[t]] = oval[t];
    }
}

// CSC export: colptr[c] = 1 + (first entry of a column >= c), rows 1-based
__global__ void k_colptr(const uint64_t *key, int64_t nnz, int64_t ncols, int64_t *colptr) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c <= ncols;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = nnz;
    const uint64_t target = static_cast<uint64_t>(c) << 32;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (key[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    colptr[c] = lo + 1;
  }
}

__global__ void k_rowval(const uint64_t *key, int64_t nnz, int64_t *rowval) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz;
       t += (int64_t)gridDim.x * blockDim.x)
    rowval[t] = static_cast<int64_t>(key[t] & 0xffffffffu) + 1;
}

int key_bits(int64_t ncols) {
  int b = 0;
  while (b < 32 && (int64_t(1) << b) < ncols) ++b;
  return 32 + b;
}

int64_t read_count(const int64_t *a, const int64_t *b, cudaStream_t s) {
  int64_t h[2] = {0, 0};
  FEGPU_CUDA(cudaMemcpyAsync(&h[0], a, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  if (b) FEGPU_CUDA(cudaMemcpyAsync(&h[1], b, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  return h[0] + h[1];
}

// S + S' of the reduced entries in a->keys / a->vals (nu of them)
int64_t symmetric_completion(fegpu_assembler *a, int64_t nu) {
  fegpu_context *ctx = a->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n2 = 2 * nu;
  DevBuf k2, v2, k3, o2, o3, okey, oval, keep, pos, tmp;
  k2.alloc(sizeof(uint64_t) * n2);
  v2.alloc(sizeof(double) * n2);
  k3.alloc(sizeof(uint64_t) * n2);
  o2.alloc(sizeof(int64_t) * n2);
  o3.alloc(sizeof(int64_t) * n2);
  okey.alloc(sizeof(uint64_t) * n2);
  oval.alloc(sizeof(double) * n2);
  keep.alloc(sizeof(int64_t) * (n2 + 1));
  pos.alloc(sizeof(int64_t) * (n2 + 1));
  k_mirror<<<grid_of(nu), 256, 0, s>>>(a->keys.as<uint64_t>(), a->vals.as<double>(), nu,
                                       k2.as<uint64_t>(), v2.as<double>(), o2.as<int64_t>());
  const int bits = std::max(key_bits(a->ncols), key_bits(a->nrows));
  cub_call(ctx, tmp, [&](void *t, size_t &b) {
    return cub::DeviceRadixSort::SortPairs(t, b, k2.as<uint64_t>(), k3.as<uint64_t>(),
                                           o2.as<int64_t>(), o3.as<int64_t>(), n2, 0, bits, s);
  });
  FEGPU_CUDA(cudaMemsetAsync(keep.as<int64_t>() + n2, 0, sizeof(int64_t), s));
  k_symm_runs<<<grid_of(n2), 256, 0, s>>>(k3.as<uint64_t>(), v2.as<double>(), o3.as<int64_t>(),
                                           n2, nu, okey.as<uint64_t>(), oval.as<double>(),
                                           keep.as<int64_t>());
  cub_call(ctx, tmp, [&](void *t, size_t &b) {
    return cub::DeviceScan::ExclusiveSum(t, b, keep.as<int64_t>(), pos.as<int64_t>(), n2 + 1, s);
  });
  const int64_t kept = read_count(pos.as<int64_t>() + n2, nullptr, s);
  a->keys.alloc(sizeof(uint64_t) * (kept + 1));
  a->vals.alloc(sizeof(double) * (kept + 1));
  k_scatter_kept<<<grid_of(n2), 256, 0, s>>>(okey.as<uint64_t>(), oval.as<double>(),
                                              keep.as<int64_t>(), pos.as<int64_t>(), n2,
                                              a->keys.as<uint64_t>(), a->vals.as<double>());
  FEGPU_CUDA(cudaGetLastError());
  FEGPU_CUDA(cudaStreamSynchronize(s));
  return kept;
}

}  // namespace

int64_t assembler_reduce(fegpu_assembler *a, DevBuf &key, DevBuf &idx, const double *V,
                         int64_t n) {
  fegpu_context *ctx = a->ctx;
  cudaStream_t s = ctx->stream;
  int64_t nu = 0;
  if (n > 0) {
    DevBuf key2, idx2, head, seg, tmp;
    key2.alloc(sizeof(uint64_t) * n);
    idx2.alloc(sizeof(int64_t) * n);
    head.alloc(sizeof(int64_t) * n);
    seg.alloc(sizeof(int64_t) * n);
    const int bits = key_bits(a->ncols);
    cub_call(ctx, tmp, [&](void *t, size_t &b) {
      return cub::DeviceRadixSort::SortPairs(t, b, key.as<uint64_t>(), key2.as<uint64_t>(),
                                             idx.as<int64_t>(), idx2.as<int64_t>(), n, 0, bits, s);
    });
    k_heads<<<grid_of(n), 256, 0, s>>>(key2.as<uint64_t>(), n, head.as<int64_t>());
    cub_call(ctx, tmp, [&](void *t, size_t &b) {
      return cub::DeviceScan::ExclusiveSum(t, b, head.as<int64_t>(), seg.as<int64_t>(), n, s);
    });
    nu = read_count(seg.as<int64_t>() + n - 1, head.as<int64_t>() + n - 1, s);
    a->keys.alloc(sizeof(uint64_t) * (nu + 1));
    a->vals.alloc(sizeof(double) * (nu + 1));
    k_reduce_runs<<<grid_of(n), 256, 0, s>>>(key2.as<uint64_t>(), idx2.as<int64_t>(), V,
                                             seg.as<int64_t>(), n, a->keys.as<uint64_t>(),
                                             a->vals.as<double>());
    FEGPU_CUDA(cudaGetLastError());
  }
  if (a->symmetric && nu > 0) nu = symmetric_completion(a, nu);
  FEGPU_CUDA(cudaStreamSynchronize(s));
  a->nnz = nu;
  a->I.clear();
  a->J.clear();
  a->V.clear();  // buffer pointer back to 1: ready for the next assembly
  return nu;
}

}  // namespace fegpu

using namespace fegpu;

extern "C" {

int fegpu_assembler_create(fegpu_context *ctx, int kind, int64_t nrows, int64_t ncols,
                           fegpu_assembler **out) {
  try {
    if (!ctx || !out) throw Error{FEGPU_ERR_ARG, "null handle"};
    if (kind < FEGPU_ASM_SPARSE || kind > FEGPU_ASM_HRZ_LUMPING_SYMM)
      throw Error{FEGPU_ERR_ARG, "unknown assembler kind"};
    const int symmetric = kind == FEGPU_ASM_SPARSE_SYMM;
    if (kind != FEGPU_ASM_SPARSE && nrows != ncols)
      throw Error{FEGPU_ERR_ARG, "Row and column info do not agree"};
    if (nrows < 1 || ncols < 1 || nrows >= (int64_t(1) << 32) || ncols >= (int64_t(1) << 32))
      throw Error{FEGPU_ERR_ARG, "bad matrix size"};
    auto *a = new fegpu_assembler();
    a->ctx = ctx;
    a->symmetric = symmetric;
    a->kind = kind;
    a->nrows = nrows;
    a->ncols = ncols;
    *out = a;
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  }
}

int fegpu_assembler_destroy(fegpu_assembler *a) {
  if (a) {
    cudaSetDevice(a->ctx->device);
    cudaStreamSynchronize(a->ctx->stream);
    delete a;
  }
  return FEGPU_OK;
}

int fegpu_assembler_assemble(fegpu_assembler *a, const double *mat, int nr, int nc,
                             const int64_t *rows, const int64_t *cols) {
  try {
    if (!a || !mat || !rows || !cols) throw Error{FEGPU_ERR_ARG, "null handle"};
    if (a->kind != FEGPU_ASM_SPARSE && nr != nc) throw Error{FEGPU_ERR_ARG, "Size mismatch"};
    if (a->kind == FEGPU_ASM_SPARSE_DIAG || a->kind == FEGPU_ASM_HRZ_LUMPING_SYMM) {
      // the element's diagonal (times, for HRZ, the element total -- column
      // sums, then their sum -- over the diagonal total)
      double ff = 1.0;
      if (a->kind == FEGPU_ASM_HRZ_LUMPING_SYMM) {
        double em2 = 0.0, dem2 = 0.0;
        for (int j = 0; j < nc; ++j) {
          double cs = 0.0;
          for (int i = 0; i < nr; ++i) cs += mat[static_cast<size_t>(j) * nr + i];
          em2 += cs;
        }
        for (int i = 0; i < nr; ++i) dem2 += mat[static_cast<size_t>(i) * nr + i];
        ff = em2 / dem2;
      }
      for (int j = 0; j < nc; ++j) {
        const int64_t dj = cols[j];
        if (dj < 1) throw Error{FEGPU_ERR_ARG, "Column degree of freedom < 1"};
        if (dj > a->ncols) throw Error{FEGPU_ERR_ARG, "Column degree of freedom > size"};
        const double v = mat[static_cast<size_t>(j) * nr + j];
        a->I.push_back(dj);
        a->J.push_back(dj);
        a->V.push_back(a->kind == FEGPU_ASM_HRZ_LUMPING_SYMM ? v * ff : v);
      }
      return FEGPU_OK;
    }
    for (int j = 0; j < nc; ++j) {
      const int64_t dj = cols[j];
      if (dj < 1) throw Error{FEGPU_ERR_ARG, "Column degree of freedom < 1"};
      if (dj > a->ncols) throw Error{FEGPU_ERR_ARG, "Column degree of freedom > size"};
      for (int i = a->symmetric ? j : 0; i < nr; ++i) {
        const int64_t di = rows[i];
        if (di < 1) throw Error{FEGPU_ERR_ARG, "Row degree of freedom < 1"};
        if (di > a->nrows) throw Error{FEGPU_ERR_ARG, "Row degree of freedom > size"};
        a->I.push_back(di);
        a->J.push_back(dj);
        a->V.push_back(mat[static_cast<size_t>(j) * nr + i]);
      }
    }
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc &) {
    set_error("host allocation failed");
    return FEGPU_ERR_MEMORY;
  }
}

int fegpu_assembler_make(fegpu_assembler *a, int64_t *nnz) {
  try {
    if (!a || !nnz) throw Error{FEGPU_ERR_ARG, "null handle"};
    fegpu_context *ctx = a->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = static_cast<int64_t>(a->V.size());
    DevBuf dI, dJ, dV, key, idx;
    dI.alloc(sizeof(int64_t) * (n + 1));
    dJ.alloc(sizeof(int64_t) * (n + 1));
    dV.alloc(sizeof(double) * (n + 1));
    key.alloc(sizeof(uint64_t) * (n + 1));
    idx.alloc(sizeof(int64_t) * (n + 1));
    if (n > 0) {
      FEGPU_CUDA(cudaMemcpyAsync(dI.p, a->I.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
      FEGPU_CUDA(cudaMemcpyAsync(dJ.p, a->J.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
      FEGPU_CUDA(cudaMemcpyAsync(dV.p, a->V.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      k_make_keys<<<grid_of(n), 256, 0, s>>>(dI.as<int64_t>(), dJ.as<int64_t>(), n,
                                             key.as<uint64_t>(), idx.as<int64_t>());
      FEGPU_CUDA(cudaGetLastError());
    }
    *nnz = assembler_reduce(a, key, idx, dV.as<double>(), n);
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc &) {
    set_error("host allocation failed");
    return FEGPU_ERR_MEMORY;
  }
}

int fegpu_assembler_copy_csc(fegpu_assembler *a, int64_t *colptr, int64_t *rowval, double *nzval) {
  try {
    if (!a || !colptr || !rowval || !nzval) throw Error{FEGPU_ERR_ARG, "null handle"};
    if (a->nnz < 0) throw Error{FEGPU_ERR_STATE, "makematrix! has not run"};
    fegpu_context *ctx = a->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t nnz = a->nnz;
    DevBuf cp, rv;
    cp.alloc(sizeof(int64_t) * (a->ncols + 1));
    rv.alloc(sizeof(int64_t) * (nnz + 1));
    k_colptr<<<grid_of(a->ncols + 1), 256, 0, s>>>(a->keys.as<uint64_t>(), nnz, a->ncols,
                                                   cp.as<int64_t>());
    if (nnz > 0) k_rowval<<<grid_of(nnz), 256, 0, s>>>(a->keys.as<uint64_t>(), nnz, rv.as<int64_t>());
    FEGPU_CUDA(cudaGetLastError());
    FEGPU_CUDA(cudaMemcpyAsync(colptr, cp.p, sizeof(int64_t) * (a->ncols + 1), cudaMemcpyDeviceToHost, s));
    if (nnz > 0) {
      FEGPU_CUDA(cudaMemcpyAsync(rowval, rv.p, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, s));
      FEGPU_CUDA(cudaMemcpyAsync(nzval, a->vals.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
    }
    FEGPU_CUDA(cudaStreamSynchronize(s));
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  }
}

}  // extern "C"
