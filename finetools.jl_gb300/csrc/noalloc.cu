// Allocation-free mixed-precision linear-elasticity assembly.
//
// Some callers cannot call cudaMalloc once they are running: a framework
// whose own pool allocator has already reserved the GPU's memory (and would
// be starved or fragmented by allocations behind its back), or a time-step
// loop that must not pay cudaMalloc's device-wide synchronisation and its
// failure modes after start-up.  fegpu_bilform_lin_elastic_noalloc serves
// them: it runs the mixed-precision path (FP32 element blocks + row gather)
// with all of its scratch -- the element-block ring, the gather order of the
// nodes and the per-element coefficients -- in the file-scope array below,
// and calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array has a fixed size (FEGPU_NOALLOC_SCRATCH_BYTES, 64 MiB) and every
// GPU on which a library context is created holds it until the process exits
// (fegpu_context_create looks its address up, which loads it).  All calls
// share it and it keeps the last call's contents; nothing in it needs to
// start at zero (every block, order entry and coefficient is written before
// it is read).  Calls whose GPU work overlaps (two streams, or two host
// threads) race on it.
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[FEGPU_NOALLOC_SCRATCH_BYTES];
// status word of the tensor-core element kernel (0 = ok)
static __device__ int g_noalloc_status;

// Device address of the array, looked up once per device with that device
// current (in host code the symbol is only a host-side stand-in).
void *scratch_address(int device) {
  static std::mutex mu;
  static void *addr[256] = {};
  std::lock_guard<std::mutex> lock(mu);
  FEGPU_REQUIRE(device >= 0 && device < 256, "device ordinal out of range");
  if (!addr[device]) {
    void *p = nullptr;
    FEGPU_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[device] = p;
  }
  return addr[device];
}

int *status_address(int device) {
  static std::mutex mu;
  static void *addr[256] = {};
  std::lock_guard<std::mutex> lock(mu);
  FEGPU_REQUIRE(device >= 0 && device < 256, "device ordinal out of range");
  if (!addr[device]) {
    void *p = nullptr;
    FEGPU_CUDA(cudaGetSymbolAddress(&p, g_noalloc_status));
    addr[device] = p;
  }
  return static_cast<int *>(addr[device]);
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace

// Called by fegpu_context_create with the device current: looking the two
// symbols up loads this file's module, and with it the static array, before
// the caller's own allocator reserves the GPU's memory.
void noalloc_prepare(int device) {
  scratch_address(device);
  status_address(device);
}

namespace {

// ring chunks needed when elements are cut in chunks of c: a node's incident
// elements span (last / c - first / c + 1) chunks
int ring_for(const fegpu_dofmap *dm, int64_t c) {
  int64_t span = 0;
  for (size_t n = 0; n < dm->node_first.size(); ++n)
    if (dm->node_first[n] >= 0)
      span = std::max<int64_t>(span, dm->node_last[n] / c - dm->node_first[n] / c);
  return static_cast<int>(span + 1);
}

}  // namespace
}  // namespace fegpu

using namespace fegpu;

extern "C" int fegpu_bilform_lin_elastic_noalloc(fegpu_matrix *K, const fegpu_coef *cf) {
  try {
    FEGPU_REQUIRE(K && cf && cf->data, "null handle");
    fegpu_dofmap *dm = K->dm;
    fegpu_femm *fm = dm->femm;
    fegpu_context *ctx = fm->ctx;
    FEGPU_CUDA(cudaSetDevice(ctx->device));
    FEGPU_REQUIRE(fm->has_geometry, "geometry not set (fegpu_femm_set_geometry)");
    FEGPU_REQUIRE(fm->mdim == 3 && fm->sdim == 3, "lin_elastic: 3-D solid elements only");
    FEGPU_REQUIRE(dm->ndn == 3, "lin_elastic: the field must have three DOFs per node");
    if (!dm->gather_ready)
      throw Error{FEGPU_ERR_STATE,
                  "run one mixed-precision assembly on this matrix first "
                  "(fegpu_bilform_lin_elastic with FEGPU_MIXED builds the node-to-element "
                  "tables this entry point reads)"};
    void *base = scratch_address(ctx->device);  // looked up when the context was created
    K->unsym = false;
    const int64_t E = fm->nelem;
    const int nne = fm->nne;
    const int nblk = nne * (nne + 1) / 2;
    const size_t block_bytes = sizeof(float) * nblk * 9;

    KArgs a = base_args(K, dm);
    int form;
    int64_t coef_width = 0;
    if (cf->kind == FEGPU_COEF_ISO_LAME) {
      form = F_ELAST_ISO;
      coef_width = 2;
    } else if (cf->kind == FEGPU_COEF_PER_ELEMENT && cf->ncomp == 36) {
      form = F_ELAST_GEN;
      coef_width = 36;
    } else if (cf->kind == FEGPU_COEF_CONST && cf->ncomp == 36) {
      double lam, mu;
      if (is_isotropic(cf->data, lam, mu)) {
        form = F_ELAST_ISO;
        a.cconst[0] = lam;
        a.cconst[1] = mu;
      } else {
        form = F_ELAST_GEN;
        for (int i = 0; i < 36; ++i) a.cconst[i] = cf->data[i];
      }
    } else {
      throw Error{FEGPU_ERR_ARG,
                  "lin_elastic: coefficient must be a 6x6 D (constant or per element) or "
                  "per-element (lambda, mu)"};
    }
    a.coef_kind = cf->kind;
    // the same kernel arguments as fegpu_bilform_lin_elastic: an isotropic
    // constant D travels as its (lambda, mu) pair
    a.ncomp = (form == F_ELAST_ISO && cf->kind == FEGPU_COEF_CONST) ? 2 : cf->ncomp;

    // chunk size: the largest (from the regular plan's down) whose ring,
    // node order and coefficients fit in the static array
    const int64_t nactive = dm->chunk_nodes.empty() ? 0 : dm->chunk_nodes.back();
    const size_t order_bytes = align256(sizeof(int32_t) * std::max<int64_t>(nactive, 1));
    const size_t coef_bytes = align256(sizeof(double) * E * coef_width);
    if (dm->na_chunk == 0 || dm->na_coef_bytes != coef_bytes) {
      dm->na_coef_bytes = coef_bytes;
      int64_t c = std::max<int64_t>(1, std::min<int64_t>(dm->chunk, E));
      for (;;) {
        const int ring = ring_for(dm, c);
        const size_t need = align256(static_cast<size_t>(ring) * c * block_bytes) + order_bytes;
        if (need + coef_bytes <= FEGPU_NOALLOC_SCRATCH_BYTES || c <= 64) {
          dm->na_chunk = c;
          dm->na_ring = ring;
          break;
        }
        c /= 2;
      }
      // node order by the chunk of the node's last element
      const int64_t nch = (E + dm->na_chunk - 1) / dm->na_chunk;
      std::vector<int64_t> cnt(nch + 1, 0);
      for (size_t n = 0; n < dm->node_last.size(); ++n)
        if (dm->node_first[n] >= 0) cnt[dm->node_last[n] / dm->na_chunk + 1]++;
      for (int64_t c2 = 0; c2 < nch; ++c2) cnt[c2 + 1] += cnt[c2];
      std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
      dm->na_order.assign(cnt[nch], 0);
      for (size_t n = 0; n < dm->node_last.size(); ++n)
        if (dm->node_first[n] >= 0)
          dm->na_order[at[dm->node_last[n] / dm->na_chunk]++] = static_cast<int32_t>(n);
      dm->na_chunk_nodes = cnt;
    }
    const int64_t chunk = dm->na_chunk;
    const int ring = dm->na_ring;
    const size_t ring_bytes = align256(static_cast<size_t>(ring) * chunk * block_bytes);
    const size_t total = ring_bytes + order_bytes + coef_bytes;
    if (total > FEGPU_NOALLOC_SCRATCH_BYTES) {
      throw Error{FEGPU_ERR_ARG,
                  "mesh too large for the allocation-free assembly: it needs " +
                      std::to_string((total + (1u << 20) - 1) >> 20) + " MiB of scratch, the "
                      "static array holds " + std::to_string(FEGPU_NOALLOC_SCRATCH_BYTES >> 20) +
                      " MiB (use fegpu_bilform_lin_elastic with FEGPU_MIXED)"};
    }

    unsigned char *sbase = static_cast<unsigned char *>(base);
    float *ke = reinterpret_cast<float *>(sbase);
    int32_t *order = reinterpret_cast<int32_t *>(sbase + ring_bytes);
    double *coef = reinterpret_cast<double *>(sbase + ring_bytes + order_bytes);
    cudaStream_t s = ctx->stream;
    if (nactive > 0)
      FEGPU_CUDA(cudaMemcpyAsync(order, dm->na_order.data(), sizeof(int32_t) * nactive,
                                 cudaMemcpyHostToDevice, s));
    if (coef_width > 0) {
      FEGPU_CUDA(cudaMemcpyAsync(coef, cf->data, sizeof(double) * E * coef_width,
                                 cudaMemcpyHostToDevice, s));
      a.coef = coef;  // element order, as the block kernel reads it
    }

    a.conn = fm->conn_orig.as<int32_t>();
    a.te = mixed_tile_for(fm->etype, form, fm->npts, false);  // the single-call tile
    FEGPU_REQUIRE(mixed_smem_for(fm->etype, form, fm->npts, a.te) <= 227 * 1024,
                  "quadrature rule too large for the element kernel");
    GArgs g;
    g.n2e_ptr = dm->n2e_ptr.as<int64_t>();
    g.n2e_elem = dm->n2e_elem.as<int32_t>();
    g.n2e_loc = dm->n2e_loc.as<uint8_t>();
    g.n2e_slot = nullptr;  // slots computed from chunk and ring
    g.nodes = order;
    g.nptr = dm->nptr.as<int64_t>();
    g.pos = dm->pos_orig.as<uint16_t>();
    g.ke = ke;
    g.chunk = chunk;
    g.ring = ring;
    g.dof = dm->dof.as<int32_t>();
    g.rowptr = dm->rowptr.as<int64_t>();
    g.colperm = dm->contiguous ? nullptr : dm->colperm.as<int32_t>();
    g.cpoff = dm->contiguous ? nullptr : dm->cpoff.as<int64_t>();
    g.val = K->val.as<double>();
    g.maxdeg = dm->maxdeg;
    g.check = a.check;
    g.nnz = dm->nnz;
    await_export(K, s);
    a.status = status_address(ctx->device);  // enables the tensor-core element blocks
    const int64_t nch = static_cast<int64_t>(dm->na_chunk_nodes.size()) - 1;
    for (int64_t c = 0; c < nch; ++c) {
      a.e0 = c * chunk;
      a.e1 = std::min(E, (c + 1) * chunk);
      a.ke = ke + (c % ring) * chunk * nblk * 9;
      ctx->launches += launch_mixed(fm->etype, form, a, ctx->num_sms, s);
      g.n0 = dm->na_chunk_nodes[c];
      g.n1 = dm->na_chunk_nodes[c + 1];
      ctx->launches += launch_gather_inline_slot(fm->etype, 3, g, ctx->num_sms, s);
    }
    FEGPU_CUDA(cudaStreamSynchronize(s));
    int st = 0;
    FEGPU_CUDA(cudaMemcpy(&st, a.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) {
      FEGPU_CUDA(cudaMemset(a.status, 0, sizeof(int)));
      throw Error{FEGPU_ERR_DEVICE, "mixed path: tensor-core completion wait ran out"};
    }
    return FEGPU_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    set_error(e.what());
    return FEGPU_ERR_STATE;
  }
}
