// Device construction of the CSR pattern of the global matrix.
//
// The reference gets its pattern as a by-product of sparse(I, J, V) over the
// element COO triples (src/AssemblyModule.jl:319, 567).  Here the pattern is
// built once per (mesh, DOF numbering) from the connectivity alone:
//   1. node pairs (A, B) of every element -> 64-bit keys (A, rank(B)), where
//      rank orders nodes by their smallest DOF number;
//   2. radix sort + unique -> node adjacency lists, sorted by DOF number;
//   3. every DOF row of node A holds ndn * deg(A) columns (all DOFs of all
//      neighbours), so row lengths and the row pointer follow by a scan;
//   4. column indices are written directly when every node's DOFs are
//      consecutive (the numbering numberdofs! produces without EBCs); for any
//      other numbering the rows are segment-sorted and a per-node column
//      permutation maps (neighbour, component) to the position in the row;
//   5. pos[e][a][b] = position of node b in node a's adjacency list, for every
//      element in colour order: the element kernels turn it into a CSR slot.
// The structure equals that of SparseMatrixCSC returned by makematrix!
// (node adjacency x ndn^2), before any exact-zero values are dropped.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

constexpr int kThreads = 256;
inline int grid_for(int64_t n, int per = kThreads) {
  int64_t g = (n + per - 1) / per;
  return static_cast<int>(std::min<int64_t>(std::max<int64_t>(g, 1), 1 << 20));
}

__global__ void k_node_key(const int32_t *dof, int ndn, int64_t nnodes, uint32_t *key,
                           int32_t *idx) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nnodes;
       n += (int64_t)gridDim.x * blockDim.x) {
    int32_t m = dof[n * ndn];
    for (int j = 1; j < ndn; ++j) m = min(m, dof[n * ndn + j]);
    key[n] = static_cast<uint32_t>(m);
    idx[n] = static_cast<int32_t>(n);
  }
}

__global__ void k_rank(const int32_t *order, int64_t n, int32_t *rank) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    rank[order[i]] = static_cast<int32_t>(i);
}

__global__ void k_pair_keys(const int32_t *conn, int64_t nelem, int nne, const int32_t *rank,
                            uint64_t *keys) {
  const int64_t total = nelem * nne * nne;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / (nne * nne);
    const int r = static_cast<int>(t - e * nne * nne);
    const int a = r / nne, b = r - a * nne;
    const uint32_t A = static_cast<uint32_t>(conn[e * nne + a]);
    const uint32_t B = static_cast<uint32_t>(conn[e * nne + b]);
    keys[t] = (static_cast<uint64_t>(A) << 32) | static_cast<uint32_t>(rank[B]);
  }
}

__global__ void k_degree(const uint64_t *ukeys, const int64_t *nu, int32_t *deg, uint32_t *nbr) {
  const int64_t n = *nu;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = ukeys[t];
    atomicAdd(&deg[k >> 32], 1);  // integer counts: order-independent
    nbr[t] = static_cast<uint32_t>(k & 0xffffffffu);
  }
}

__global__ void k_contig(const int32_t *dof, int ndn, int64_t nnodes, const int32_t *deg,
                         int *flag) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nnodes;
       n += (int64_t)gridDim.x * blockDim.x) {
    if (deg[n] == 0) continue;
    for (int j = 1; j < ndn; ++j)
      if (dof[n * ndn + j] != dof[n * ndn] + j) atomicExch(flag, 0);
  }
}

// One warp per node: write the columns of the node's ndn rows.
__global__ void k_colind(const int32_t *dof, int ndn, int64_t nnodes, const int64_t *nptr,
                         const uint32_t *nbr, const int32_t *order, const int64_t *rowptr,
                         int32_t *colind) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t n = warp; n < nnodes; n += nwarps) {
    const int64_t b0 = nptr[n], deg = nptr[n + 1] - b0;
    if (deg == 0) continue;
    for (int i = 0; i < ndn; ++i) {
      const int64_t r0 = rowptr[dof[n * ndn + i]];
      for (int64_t k = lane; k < deg; k += 32) {
        const int32_t B = order[nbr[b0 + k]];
        for (int j = 0; j < ndn; ++j) colind[r0 + ndn * k + j] = dof[B * ndn + j];
      }
    }
  }
}

// General numbering: position of dof(B_k, j) inside the (sorted) rows of node A.
__global__ void k_colperm(const int32_t *dof, int ndn, int64_t nnodes, const int64_t *nptr,
                          const uint32_t *nbr, const int32_t *order, const int64_t *rowptr,
                          const int32_t *colind, int32_t *colperm) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nnodes;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = nptr[n], deg = nptr[n + 1] - b0;
    if (deg == 0) continue;
    const int64_t r0 = rowptr[dof[n * ndn]];
    const int64_t len = ndn * deg;
    for (int64_t k = 0; k < deg; ++k) {
      const int32_t B = order[nbr[b0 + k]];
      for (int j = 0; j < ndn; ++j) {
        const int32_t c = dof[B * ndn + j];
        int64_t lo = 0, hi = len;  // lower_bound
        while (lo < hi) {
          const int64_t mid = (lo + hi) >> 1;
          if (colind[r0 + mid] < c) lo = mid + 1; else hi = mid;
        }
        colperm[b0 * ndn + k * ndn + j] = static_cast<int32_t>(lo);
      }
    }
  }
}

// pos[e][a][b]: index of node b in node a's adjacency list (binary search on rank).
__global__ void k_pos(const int32_t *conn, int64_t nelem, int nne, const int32_t *rank,
                      const int64_t *nptr, const uint32_t *nbr, uint16_t *pos) {
  const int64_t total = nelem * nne * nne;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / (nne * nne);
    const int r = static_cast<int>(t - e * nne * nne);
    const int a = r / nne, b = r - a * nne;
    const int32_t A = conn[e * nne + a];
    const uint32_t key = static_cast<uint32_t>(rank[conn[e * nne + b]]);
    int64_t lo = nptr[A], hi = nptr[A + 1];
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (nbr[mid] < key) lo = mid + 1; else hi = mid;
    }
    pos[t] = static_cast<uint16_t>(lo - nptr[A]);
  }
}

template <typename F>
void cub_call(fegpu_context *ctx, F &&f) {
  size_t bytes = 0;
  FEGPU_CUDA(f(nullptr, bytes));
  ctx->scratch.alloc(bytes);
  FEGPU_CUDA(f(ctx->scratch.p, bytes));
}

int bits_for(uint64_t v) {
  int b = 1;
  while (b < 64 && (v >> b) != 0) ++b;
  return b;
}

}  // namespace

void build_pattern(fegpu_dofmap *dm, const std::vector<int32_t> &hdof) {
  fegpu_femm *fm = dm->femm;
  fegpu_context *ctx = fm->ctx;
  cudaStream_t s = ctx->stream;
  const int ndn = dm->ndn, nne = fm->nne;
  const int64_t N = fm->nnodes, E = fm->nelem, ndof = dm->ndof;

  dm->dof.alloc(sizeof(int32_t) * N * ndn);
  FEGPU_CUDA(cudaMemcpyAsync(dm->dof.p, hdof.data(), sizeof(int32_t) * N * ndn,
                             cudaMemcpyHostToDevice, s));

  // 1. node ranks by smallest DOF number
  DevBuf key, keyo, idx, order, rank;
  key.alloc(sizeof(uint32_t) * N);
  keyo.alloc(sizeof(uint32_t) * N);
  idx.alloc(sizeof(int32_t) * N);
  order.alloc(sizeof(int32_t) * N);
  rank.alloc(sizeof(int32_t) * N);
  k_node_key<<<grid_for(N), kThreads, 0, s>>>(dm->dof.as<int32_t>(), ndn, N, key.as<uint32_t>(),
                                              idx.as<int32_t>());
  FEGPU_CUDA(cudaGetLastError());
  cub_call(ctx, [&](void *t, size_t &b) {
    return cub::DeviceRadixSort::SortPairs(t, b, key.as<uint32_t>(), keyo.as<uint32_t>(),
                                           idx.as<int32_t>(), order.as<int32_t>(), N, 0,
                                           bits_for(ndof), s);
  });
  k_rank<<<grid_for(N), kThreads, 0, s>>>(order.as<int32_t>(), N, rank.as<int32_t>());

  // 2. node pairs -> sorted unique adjacency
  const int64_t np = E * nne * nne;
  DevBuf keys, keys2, ucount;
  keys.alloc(sizeof(uint64_t) * np);
  keys2.alloc(sizeof(uint64_t) * np);
  ucount.alloc(sizeof(int64_t));
  k_pair_keys<<<grid_for(np), kThreads, 0, s>>>(fm->conn_orig.as<int32_t>(), E, nne,
                                                rank.as<int32_t>(), keys.as<uint64_t>());
  FEGPU_CUDA(cudaGetLastError());
  const int endbit = 32 + bits_for(static_cast<uint64_t>(N));
  cub_call(ctx, [&](void *t, size_t &b) {
    return cub::DeviceRadixSort::SortKeys(t, b, keys.as<uint64_t>(), keys2.as<uint64_t>(), np, 0,
                                          endbit, s);
  });
  cub_call(ctx, [&](void *t, size_t &b) {
    return cub::DeviceSelect::Unique(t, b, keys2.as<uint64_t>(), keys.as<uint64_t>(),
                                     ucount.as<int64_t>(), np, s);
  });
  int64_t nu = 0;
  FEGPU_CUDA(cudaMemcpyAsync(&nu, ucount.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  keys2.release();

  DevBuf deg, nbr;
  DevBuf &nptr = dm->nptr;
  deg.alloc(sizeof(int32_t) * (N + 1));
  nptr.alloc(sizeof(int64_t) * (N + 1));
  nbr.alloc(sizeof(uint32_t) * (nu + 1));
  FEGPU_CUDA(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * (N + 1), s));
  k_degree<<<grid_for(nu), kThreads, 0, s>>>(keys.as<uint64_t>(), ucount.as<int64_t>(),
                                             deg.as<int32_t>(), nbr.as<uint32_t>());
  keys.release();
  DevBuf degl;
  degl.alloc(sizeof(int64_t) * (N + 1));
  {
    // widen to int64 and scan -> nptr
    std::vector<int32_t> hdeg(N);
    FEGPU_CUDA(cudaMemcpyAsync(hdeg.data(), deg.p, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
    std::vector<int64_t> hp(N + 1, 0);
    int mx = 0;
    for (int64_t n = 0; n < N; ++n) {
      hp[n + 1] = hp[n] + hdeg[n];
      mx = std::max(mx, hdeg[n]);
    }
    dm->maxdeg = mx;
    FEGPU_REQUIRE(mx < 65536, "node degree too large for the 16-bit slot map");
    FEGPU_CUDA(cudaMemcpyAsync(nptr.p, hp.data(), sizeof(int64_t) * (N + 1),
                               cudaMemcpyHostToDevice, s));
    // 3. DOF row lengths and row pointer
    std::vector<int64_t> rl(ndof + 1, 0);
    for (int64_t n = 0; n < N; ++n)
      if (hdeg[n] > 0)
        for (int i = 0; i < ndn; ++i) rl[hdof[n * ndn + i]] = static_cast<int64_t>(ndn) * hdeg[n];
    std::vector<int64_t> rp(ndof + 1, 0);
    for (int64_t r = 0; r < ndof; ++r) rp[r + 1] = rp[r] + rl[r];
    dm->nnz = rp[ndof];
    FEGPU_REQUIRE(dm->nnz < (int64_t(1) << 31) * 16, "matrix too large");
    dm->rowptr.alloc(sizeof(int64_t) * (ndof + 1));
    FEGPU_CUDA(cudaMemcpyAsync(dm->rowptr.p, rp.data(), sizeof(int64_t) * (ndof + 1),
                               cudaMemcpyHostToDevice, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
  }

  // contiguity of the numbering
  DevBuf flag;
  flag.alloc(sizeof(int));
  int one = 1;
  FEGPU_CUDA(cudaMemcpyAsync(flag.p, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  if (ndn > 1)
    k_contig<<<grid_for(N), kThreads, 0, s>>>(dm->dof.as<int32_t>(), ndn, N, deg.as<int32_t>(),
                                              flag.as<int>());
  int contig = 1;
  FEGPU_CUDA(cudaMemcpyAsync(&contig, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  FEGPU_CUDA(cudaStreamSynchronize(s));
  dm->contiguous = contig != 0;

  // 4. column indices
  dm->colind.alloc(sizeof(int32_t) * (dm->nnz + 1));
  k_colind<<<grid_for(N * 32), kThreads, 0, s>>>(
      dm->dof.as<int32_t>(), ndn, N, nptr.as<int64_t>(), nbr.as<uint32_t>(), order.as<int32_t>(),
      dm->rowptr.as<int64_t>(), dm->colind.as<int32_t>());
  FEGPU_CUDA(cudaGetLastError());
  if (!dm->contiguous) {
    DevBuf sorted;
    sorted.alloc(sizeof(int32_t) * (dm->nnz + 1));
    cub_call(ctx, [&](void *t, size_t &b) {
      return cub::DeviceSegmentedSort::SortKeys(
          t, b, dm->colind.as<int32_t>(), sorted.as<int32_t>(), dm->nnz, ndof,
          dm->rowptr.as<int64_t>(), dm->rowptr.as<int64_t>() + 1, s);
    });
    FEGPU_CUDA(cudaMemcpyAsync(dm->colind.p, sorted.p, sizeof(int32_t) * dm->nnz,
                               cudaMemcpyDeviceToDevice, s));
    FEGPU_CUDA(cudaStreamSynchronize(s));
    dm->colperm.alloc(sizeof(int32_t) * (nu * ndn + 1));
    k_colperm<<<grid_for(N), kThreads, 0, s>>>(
        dm->dof.as<int32_t>(), ndn, N, nptr.as<int64_t>(), nbr.as<uint32_t>(),
        order.as<int32_t>(), dm->rowptr.as<int64_t>(), dm->colind.as<int32_t>(),
        dm->colperm.as<int32_t>());
    FEGPU_CUDA(cudaGetLastError());
    // cpoff[A] = nptr[A] * ndn: the kernels compute it from nptr
    dm->cpoff.alloc(sizeof(int64_t) * (N + 1));
    FEGPU_CUDA(cudaMemcpyAsync(dm->cpoff.p, dm->nptr.p, sizeof(int64_t) * (N + 1),
                               cudaMemcpyDeviceToDevice, s));
  }

  // 5. slot maps for the colour-sorted elements
  dm->pos.alloc(sizeof(uint16_t) * np);
  k_pos<<<grid_for(np), kThreads, 0, s>>>(fm->conn.as<int32_t>(), E, nne, rank.as<int32_t>(),
                                          nptr.as<int64_t>(), nbr.as<uint32_t>(),
                                          dm->pos.as<uint16_t>());
  FEGPU_CUDA(cudaGetLastError());
  FEGPU_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fegpu
