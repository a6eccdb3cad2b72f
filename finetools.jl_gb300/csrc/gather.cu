// Mixed-precision assembly by row gather.
//
// On this GPU an FP64 add or an f32->f64 conversion runs at ~0.5 T/s, so one
// FP64 add per element contribution (230 M for an H20 40^3 block, 1.17 G for
// a T10 60^3 block) costs more than streaming the whole CSR through HBM.  The
// mixed path therefore never adds into the global matrix element by element:
//   1. element phase: the FP32 node-pair blocks of a chunk of elements (in
//      element order) go to a ring buffer that stays L2-resident;
//   2. gather phase: one warp per node accumulates the blocks of its incident
//      elements (in element order: deterministic) into its rows with
//      compensated FP32 sums (two-sum, ~48-bit significand), converts each
//      entry to FP64 with integer operations only, and writes every CSR value
//      of the node's rows exactly once (plain coalesced stores, no RMW).
// A node is gathered right after the chunk holding its last element, so the
// ring needs only (span of a node's elements in chunks) + 1 chunks.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "gather.cuh"

namespace fegpu {
namespace {

template <int NNE, int NDN, bool INLINE_SLOT>
__global__ void __launch_bounds__(kGatherWarps * 32) k_gather(const GArgs g) {
  extern __shared__ __align__(16) float gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per-warp region padded to a multiple of 4 floats: every warp's region
  // starts on a 16-byte boundary (the zeroing stores float4)
  const int wstride = gather_warp_stride(NDN, g.maxdeg);
  float *acc = gsm + static_cast<size_t>(warp) * wstride;
  for (int64_t t = g.n0 + static_cast<int64_t>(blockIdx.x) * kGatherWarps + warp; t < g.n1;
       t += static_cast<int64_t>(gridDim.x) * kGatherWarps)
    gather_node<NNE, NDN, INLINE_SLOT>(g, g.nodes[t], acc, lane);
}

template <int NNE, int NDN, bool INLINE_SLOT = false>
int launch_t(const GArgs &g, int num_sms, cudaStream_t s) {
  const int64_t n = g.n1 - g.n0;
  if (n <= 0) return 0;
  const size_t smem = sizeof(float) * static_cast<size_t>(gather_warp_stride(NDN, g.maxdeg)) * kGatherWarps;
  FEGPU_REQUIRE(smem <= 227 * 1024, "node degree too large for the row gather");
  auto kern = k_gather<NNE, NDN, INLINE_SLOT>;
  FEGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  int per_sm = 0;
  FEGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGatherWarps * 32, smem));
  per_sm = std::max(per_sm, 1);
  const int64_t ctas = (n + kGatherWarps - 1) / kGatherWarps;
  const int grid = static_cast<int>(std::min<int64_t>(ctas, static_cast<int64_t>(num_sms) * per_sm));
  kern<<<grid, kGatherWarps * 32, smem, s>>>(g);
  FEGPU_CUDA(cudaGetLastError());
  return 1;
}

__global__ void k_unsort_pos(const uint16_t *pos_sorted, const int32_t *perm, int64_t nelem,
                             int nn2, uint16_t *pos_orig) {
  const int64_t total = nelem * nn2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t es = t / nn2;
    pos_orig[static_cast<int64_t>(perm[es]) * nn2 + (t - es * nn2)] = pos_sorted[t];
  }
}

}  // namespace

int launch_gather(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_H8: return ndn == 1 ? launch_t<8, 1>(g, num_sms, s) : launch_t<8, 3>(g, num_sms, s);
    case FEGPU_H20: return ndn == 1 ? launch_t<20, 1>(g, num_sms, s) : launch_t<20, 3>(g, num_sms, s);
    case FEGPU_T4: return ndn == 1 ? launch_t<4, 1>(g, num_sms, s) : launch_t<4, 3>(g, num_sms, s);
    case FEGPU_T10: return ndn == 1 ? launch_t<10, 1>(g, num_sms, s) : launch_t<10, 3>(g, num_sms, s);
    case FEGPU_Q4: return ndn == 1 ? launch_t<4, 1>(g, num_sms, s) : launch_t<4, 3>(g, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

int launch_gather_inline_slot(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s) {
  switch (etype) {
    case FEGPU_H8: return ndn == 1 ? launch_t<8, 1, true>(g, num_sms, s) : launch_t<8, 3, true>(g, num_sms, s);
    case FEGPU_H20: return ndn == 1 ? launch_t<20, 1, true>(g, num_sms, s) : launch_t<20, 3, true>(g, num_sms, s);
    case FEGPU_T4: return ndn == 1 ? launch_t<4, 1, true>(g, num_sms, s) : launch_t<4, 3, true>(g, num_sms, s);
    case FEGPU_T10: return ndn == 1 ? launch_t<10, 1, true>(g, num_sms, s) : launch_t<10, 3, true>(g, num_sms, s);
    case FEGPU_Q4: return ndn == 1 ? launch_t<4, 1, true>(g, num_sms, s) : launch_t<4, 3, true>(g, num_sms, s);
  }
  throw Error{FEGPU_ERR_ARG, "unknown element type"};
}

// Node -> element lists (incident elements in element order, with the node's
// local index) and the element-order slot maps: built once per dofmap, shared
// by the mixed and the reference-order chunk plans.  elem_out (optional)
// receives the host copy of the element lists.
void build_node_lists(fegpu_dofmap *dm, std::vector<int32_t> *elem_out) {
  fegpu_femm *fm = dm->femm;
  fegpu_context *ctx = fm->ctx;
  cudaStream_t s = ctx->stream;
  const int nne = fm->nne;
  const int64_t N = fm->nnodes, E = fm->nelem;
  const std::vector<int32_t> &c0 = fm->conn_host;
  std::vector<int64_t> ptr(N + 1, 0);
  for (int64_t i = 0; i < E * nne; ++i) ptr[c0[i] + 1]++;
  for (int64_t n = 0; n < N; ++n) ptr[n + 1] += ptr[n];
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  std::vector<int32_t> elem(static_cast<size_t>(E) * nne);
  std::vector<uint8_t> loc(static_cast<size_t>(E) * nne);
  for (int64_t e = 0; e < E; ++e)
    for (int a = 0; a < nne; ++a) {
      const int64_t q = fill[c0[e * nne + a]]++;
      elem[q] = static_cast<int32_t>(e);
      loc[q] = static_cast<uint8_t>(a);
    }
  dm->node_first.assign(N, -1);
  dm->node_last.assign(N, -1);
  for (int64_t n = 0; n < N; ++n)
    if (ptr[n + 1] > ptr[n]) {
      dm->node_first[n] = elem[ptr[n]];
      dm->node_last[n] = elem[ptr[n + 1] - 1];
    }
  if (!dm->lists_ready) {
    dm->n2e_ptr.alloc(sizeof(int64_t) * (N + 1));
    dm->n2e_elem.alloc(sizeof(int32_t) * std::max<size_t>(elem.size(), 1));
    dm->n2e_loc.alloc(std::max<size_t>(loc.size(), 1));
    FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_ptr.p, ptr.data(), sizeof(int64_t) * (N + 1),
                               cudaMemcpyHostToDevice, s));
    if (!elem.empty()) {
      FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_elem.p, elem.data(), sizeof(int32_t) * elem.size(),
                                 cudaMemcpyHostToDevice, s));
      FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_loc.p, loc.data(), loc.size(), cudaMemcpyHostToDevice,
                                 s));
    }
    const int64_t np = E * nne * nne;
    dm->pos_orig.alloc(sizeof(uint16_t) * std::max<int64_t>(np, 1));
    if (np > 0) {
      const int grid = static_cast<int>(std::min<int64_t>((np + 255) / 256, 1 << 20));
      k_unsort_pos<<<grid, 256, 0, s>>>(dm->pos.as<uint16_t>(), fm->perm.as<int32_t>(), E,
                                        nne * nne, dm->pos_orig.as<uint16_t>());
      FEGPU_CUDA(cudaGetLastError());
      ctx->launches++;
    }
    FEGPU_CUDA(cudaStreamSynchronize(s));  // the host vectors leave scope
    dm->lists_ready = true;
  }
  if (elem_out) elem_out->swap(elem);
}

// Chunk plan for chunks of `chunk` elements: a node is gathered right after
// the chunk holding its last incident element; `order` lists the nodes by
// that chunk (ranges in chunk_nodes); span is the largest chunk distance
// between a node's first and last element; the ring holds span + 2 chunks
// (the chunks one gather reads, plus the one the next element tiles write).
void plan_chunks(const fegpu_dofmap *dm, int64_t chunk, std::vector<int64_t> &chunk_nodes,
                 std::vector<int32_t> &order, int &span_out, int &ring_out) {
  const int64_t E = dm->femm->nelem;
  const int64_t N = static_cast<int64_t>(dm->node_first.size());
  const int64_t nch = (E + chunk - 1) / chunk;
  std::vector<int64_t> cnt(nch + 1, 0);
  int64_t span = 0;
  for (int64_t n = 0; n < N; ++n) {
    if (dm->node_first[n] < 0) continue;
    const int64_t cmin = dm->node_first[n] / chunk, cmaxc = dm->node_last[n] / chunk;
    span = std::max(span, cmaxc - cmin);
    cnt[cmaxc + 1]++;
  }
  for (int64_t c = 0; c < nch; ++c) cnt[c + 1] += cnt[c];
  std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
  order.assign(nch > 0 ? cnt[nch] : 0, 0);
  for (int64_t n = 0; n < N; ++n) {
    if (dm->node_first[n] < 0) continue;
    order[at[dm->node_last[n] / chunk]++] = static_cast<int32_t>(n);
  }
  chunk_nodes = cnt;
  span_out = static_cast<int>(span);
  // (at least one slot: a mesh without elements has no chunk but keeps the
  // per-slot events and slot arithmetic defined)
  ring_out = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(span + 2, nch)));
}

// The mixed path's plan: node lists, chunks of ~24 MB of FP32 blocks (at
// least 1024 elements), ring slots of the incident elements, the FP32 ring.
void build_gather_plan(fegpu_dofmap *dm, int block_values) {
  fegpu_femm *fm = dm->femm;
  cudaStream_t s = fm->ctx->stream;
  const int64_t E = fm->nelem;
  std::vector<int32_t> elem;
  build_node_lists(dm, &elem);
  const int64_t per_elem = static_cast<int64_t>(block_values) * 4;
  dm->chunk = std::max<int64_t>(1024, (24ll << 20) / std::max<int64_t>(per_elem, 1));
  dm->chunk = std::min<int64_t>(dm->chunk, std::max<int64_t>(E, 1));
  std::vector<int32_t> order;
  plan_chunks(dm, dm->chunk, dm->chunk_nodes, order, dm->span, dm->ring);
  std::vector<int32_t> slot(elem.size());
  for (size_t q = 0; q < elem.size(); ++q) {
    const int64_t ce = elem[q] / dm->chunk;
    slot[q] = static_cast<int32_t>((ce % dm->ring) * dm->chunk + (elem[q] - ce * dm->chunk));
  }
  dm->n2e_slot.alloc(sizeof(int32_t) * std::max<size_t>(slot.size(), 1));
  if (!slot.empty())
    FEGPU_CUDA(cudaMemcpyAsync(dm->n2e_slot.p, slot.data(), sizeof(int32_t) * slot.size(),
                               cudaMemcpyHostToDevice, s));
  dm->gnodes.alloc(sizeof(int32_t) * std::max<size_t>(order.size(), 1));
  if (!order.empty())
    FEGPU_CUDA(cudaMemcpyAsync(dm->gnodes.p, order.data(), sizeof(int32_t) * order.size(),
                               cudaMemcpyHostToDevice, s));
  dm->ke.alloc(sizeof(float) * static_cast<size_t>(dm->ring) * dm->chunk * block_values);
  FEGPU_CUDA(cudaStreamSynchronize(s));
  dm->gather_ready = true;
}

}  // namespace fegpu
