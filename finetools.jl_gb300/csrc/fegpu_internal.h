// Internal declarations of libfegpu: handle layouts, kernel argument blocks and
// the launchers that api.cu dispatches to.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fegpu.h"

namespace fegpu {

// ---- error plumbing --------------------------------------------------------
void set_error(const std::string &msg);
struct Error {
  int code;
  std::string msg;
};
#define FEGPU_CUDA(call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess)                                                      \
      throw ::fegpu::Error{e_ == cudaErrorMemoryAllocation ? FEGPU_ERR_MEMORY   \
                                                           : FEGPU_ERR_CUDA,    \
                           std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)
#define FEGPU_REQUIRE(cond, msg)                              \
  do {                                                        \
    if (!(cond)) throw ::fegpu::Error{FEGPU_ERR_ARG, (msg)}; \
  } while (0)

// ---- device buffer ----------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    if (n <= bytes && p) return;
    release();
    if (n == 0) n = 16;
    FEGPU_CUDA(cudaMalloc(&p, n));
    bytes = n;
  }
  template <typename T>
  T *as() const { return static_cast<T *>(p); }
};

// ---- element facts ---------------------------------------------------------
inline int nodes_per_elem(int et) {
  switch (et) {
    case FEGPU_Q4: return 4;
    case FEGPU_H8: return 8;
    case FEGPU_H20: return 20;
    case FEGPU_T4: return 4;
    case FEGPU_T10: return 10;
  }
  return 0;
}
inline int manif_dim(int et) { return et == FEGPU_Q4 ? 2 : 3; }
// quadrature points accepted per element type: the reference's Gauss rules of
// orders 1-10 (tensor products) and tet rules of 1, 4 and 5 points; rules
// whose per-element tables do not fit a kernel's shared memory are refused
// when the form runs
inline int max_qp(int et) {
  switch (et) {
    case FEGPU_Q4: return 100;
    case FEGPU_H8: return 1000;
    case FEGPU_H20: return 1000;
    case FEGPU_T4: return 5;
    case FEGPU_T10: return 5;
  }
  return 0;
}

// ---- device index checks (debug builds, -DFEGPU_DEVICE_CHECKS) ---------------
// The kernels check the node numbers they read and the CSR slots they write;
// the first violation (site << 56 | index) goes to the context's check word,
// the access is skipped, and the entry point returns FEGPU_ERR_DEVICE.  Off in
// regular builds: the checks then compile to nothing.
enum CheckSite { CK_CONN = 1, CK_SCATTER = 2, CK_GATHER = 3, CK_VECTOR = 4 };
#if defined(FEGPU_DEVICE_CHECKS)
constexpr bool kDeviceChecks = true;
#else
constexpr bool kDeviceChecks = false;
#endif
#if defined(__CUDACC__)
// true when 0 <= i < n; otherwise records (site, i) as the first violation
__device__ __forceinline__ bool dcheck(unsigned long long *word, int site, int64_t i, int64_t n) {
  if constexpr (!kDeviceChecks) {
    return true;
  } else {
    if (i >= 0 && i < n) return true;
    if (word)
      atomicCAS(word, 0ull,
                (static_cast<unsigned long long>(site) << 56) |
                    (static_cast<unsigned long long>(i) & ((1ull << 56) - 1ull)));
    return false;
  }
}
#endif

}  // namespace fegpu

// ---- handles (opaque to callers) -------------------------------------------
struct fegpu_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  fegpu::DevBuf scratch;   // CUB temporaries, compaction buffers
  fegpu::DevBuf scratch2;
  bool timing = false;      // events around the element-kernel launches
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double kernel_ms = 0.0;   // accumulated element-kernel time
  int64_t launches = 0;     // kernels launched by the library
  // mixed path: a second stream for the element blocks, so chunk c+1's blocks
  // overlap chunk c's gather; events per ring slot order them (created on use)
  cudaStream_t side = nullptr;
  std::vector<cudaEvent_t> ev_blocks, ev_gather;
  // copies of finished matrices to host memory (fegpu_matrix_copy_values_async)
  cudaStream_t export_stream = nullptr;
  // status word of the tensor-core element kernel (0 = ok), made on first use
  fegpu::DevBuf tc_status;
  // first device index-check violation (builds with device checks only)
  fegpu::DevBuf check_word;
};

struct fegpu_femm {
  fegpu_context *ctx = nullptr;
  int etype = 0, nne = 0, mdim = 0, npts = 0, sdim = 0;
  int64_t nelem = 0, nnodes = 0;
  double otherdim = 1.0;
  int axisym = 0;                      // axisymmetric domain (two-manifolds: 2 pi r)
  std::vector<int64_t> colors;         // element order, 1-based
  std::vector<int64_t> color_offsets;  // sorted-element ranges per colour
  fegpu::DevBuf conn_orig;             // int32 nelem x nne, 0-based, element order
  fegpu::DevBuf conn;                  // int32 nelem x nne, colour-sorted
  fegpu::DevBuf perm;                  // int32 sorted position -> element
  fegpu::DevBuf tab;                   // double: N[q][k], dN[q][k][m], w[q]
  fegpu::DevBuf tab32;                 // float: N[q][k], dN[q][k][m], w[q]
  fegpu::DevBuf xyz;                   // double [nnodes][4]
  bool has_geometry = false;
  std::vector<int32_t> conn_host;      // element order, 0-based
};

struct fegpu_dofmap {
  fegpu_femm *femm = nullptr;
  int ndn = 0;
  int64_t ndof = 0, nnz = 0;
  int maxdeg = 0;
  bool contiguous = true;   // every node's DOFs are consecutive numbers
  fegpu::DevBuf dof;        // int32 [nnodes][ndn], 0-based
  fegpu::DevBuf rowptr;     // int64 [ndof + 1]
  fegpu::DevBuf colind;     // int32 [nnz]
  fegpu::DevBuf pos;        // uint16 [nelem][nne][nne], colour-sorted elements
  fegpu::DevBuf colperm;    // int32 per node block, only if !contiguous
  fegpu::DevBuf cpoff;      // int64 [nnodes], only if !contiguous
  fegpu::DevBuf nptr;       // int64 [nnodes + 1]: node adjacency offsets
  // node -> element lists in element order (gather.cu), built on first use
  bool lists_ready = false;
  // row-gather plan (mixed precision), built on first use
  bool gather_ready = false;
  int64_t chunk = 0;        // elements per chunk of the block ring
  int ring = 0;             // chunks held by the ring
  int span = 0;             // max chunk distance between a node's first and last element
  std::vector<int64_t> chunk_nodes;  // gather node ranges per chunk
  fegpu::DevBuf n2e_ptr;    // int64 [nnodes + 1]
  fegpu::DevBuf n2e_elem;   // int32: incident elements, increasing
  fegpu::DevBuf n2e_loc;    // uint8: local index of the node in that element
  fegpu::DevBuf n2e_slot;   // int32: block-ring slot of that element
  fegpu::DevBuf gnodes;     // int32: nodes in gather order
  fegpu::DevBuf pos_orig;   // uint16 [nelem][nne][nne], element order
  fegpu::DevBuf ke;         // float ring of element blocks
  std::vector<int32_t> node_first, node_last;  // first / last incident element (-1: none)
  // reference-order FP64 path (exact.cu): its own chunk plan over the same
  // node-to-element lists, and an FP64 block ring
  bool exact_ready = false;
  int64_t x_chunk = 0;
  int x_ring = 0, x_span = 0, x_tile = 0;
  std::vector<int64_t> x_chunk_nodes;
  fegpu::DevBuf x_gnodes;   // int32: nodes in gather order
  fegpu::DevBuf x_ke;       // double ring of element blocks
  // plan of the allocation-free variant (noalloc.cu), cached per chunk size
  int64_t na_chunk = 0;
  int na_ring = 0;
  size_t na_coef_bytes = 0;
  std::vector<int32_t> na_order;
  std::vector<int64_t> na_chunk_nodes;
};

struct fegpu_matrix {
  fegpu_dofmap *dm = nullptr;
  fegpu::DevBuf val;    // double [nnz], CSR order (row = test DOF)
  bool unsym = false;   // values not symmetric: the CSC export transposes them
  bool symm_asm = true; // SysmatAssemblerSparseSymm (S + S') or SysmatAssemblerSparse (S)
  // asynchronous export: `ready` marks the values on the context stream,
  // `exported` the end of their copy on the export stream
  cudaEvent_t ready = nullptr, exported = nullptr;
  bool export_pending = false;
};

namespace fegpu {

// ---- element-kernel forms ----------------------------------------------------
enum Form {
  F_DIFF_ISO = 0,   // scalar conductivity
  F_DIFF_GEN = 1,   // mdim x mdim conductivity
  F_ELAST_ISO = 2,  // lambda, mu
  F_ELAST_GEN = 3,  // 6x6 D
  F_DOT = 4,        // N N' c
  F_LIN = 5,        // N f  (vector)
};

// Kernel argument block (passed by value; < 1 KB).
struct KArgs {
  const int32_t *conn;     // colour-sorted nelem x nne
  const double *xyz;       // [nnodes][4]
  const double *tab;       // N, dN, w tables
  const float *tab32;      // FP32 N, dN and w tables (mixed path)
  const uint16_t *pos;     // colour-sorted nelem x nne x nne
  const int32_t *dof;      // [nnodes][ndn]
  const int64_t *rowptr;   // CSR rows
  const int32_t *colperm;  // null when the numbering is node-contiguous
  const int64_t *cpoff;
  double *val;             // CSR values, or the dense vector for F_LIN
  const double *coef;      // device coefficient array (colour-sorted) or null
  int coef_kind;           // FEGPU_COEF_*
  int ncomp;
  double cconst[36];       // constant coefficient
  double cab[9], cba[9], cdiag[9];  // bilform_dot block coefficients
  int npts, sdim, te;
  int measure_m;           // manifold dimension of the measure (dot, linform)
  double otherdim;
  int axisym;              // axisymmetric domain: 2 pi r instead of otherdim
  double distort_tol;      // mixed path: det_min/det_max below -> FP64 geometry
  int t10_affine;          // mixed path, T10: straight-sided elements take the FP32
                           // corner Jacobian, curved ones FP64 geometry
  int64_t e0, e1;          // colour range of sorted elements
  int *status;             // device status word (0 = ok)
  float *ke;               // block-output mode: element blocks of elements e0.. (or null)
  double *ke64;            // reference-order path: FP64 blocks of elements e0..
  unsigned long long *check;  // device index checks: first violation (or null)
  int64_t nnz;             // values behind val (CSR values, or the vector's length)
  int64_t nnodes;          // node count (coordinates behind xyz)
};

// Launch one colour of one form.  Returns the number of kernel launches made.
int launch_form(int etype, int form, int precision, int ndn, const KArgs &a,
                int num_sms, cudaStream_t s);
size_t form_smem_bytes(int etype, int form, int precision, int npts, int te);
int choose_tile(int etype, int form, int precision, int npts);

// ---- host colouring (element_coloring!) ---------------------------------------
int64_t greedy_element_coloring(int64_t nelem, int nne, const int32_t *conn0,
                                int64_t nnodes, std::vector<int64_t> &colors);

// ---- pattern build on the device ------------------------------------------------
void build_pattern(fegpu_dofmap *dm, const std::vector<int32_t> &hdof);

// ---- row gather (mixed precision) ------------------------------------------------
struct GArgs {
  const int64_t *n2e_ptr;
  const int32_t *n2e_elem;
  const uint8_t *n2e_loc;
  const int32_t *n2e_slot;  // ring slot of each incident element
  const int32_t *nodes;     // nodes in gather order
  int64_t n0, n1;           // range of nodes[] handled by this launch
  const int64_t *nptr;      // adjacency offsets (degree)
  const uint16_t *pos;      // element-order slot maps
  const float *ke;          // ring of element blocks
  const double *ke64;       // ring of FP64 element blocks (reference-order path)
  int64_t chunk;            // elements per ring chunk
  int ring;                 // chunks in the ring
  const int32_t *dof;
  const int64_t *rowptr;
  const int32_t *colperm;
  const int64_t *cpoff;
  double *val;
  int maxdeg;
  unsigned long long *check;  // device index checks: first violation (or null)
  int64_t nnz;
};
void build_gather_plan(fegpu_dofmap *dm, int nblk_values);
// node -> element lists and element-order slot maps (once per dofmap); the
// host copy of the lists goes to elem_out when given
void build_node_lists(fegpu_dofmap *dm, std::vector<int32_t> *elem_out);
// gather order and ring size for chunks of `chunk` elements
void plan_chunks(const fegpu_dofmap *dm, int64_t chunk, std::vector<int64_t> &chunk_nodes,
                 std::vector<int32_t> &order, int &span, int &ring);
int launch_gather(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s);
// variant that computes each element's ring slot from chunk and ring
// (g.n2e_slot unused)
int launch_gather_inline_slot(int etype, int ndn, const GArgs &g, int num_sms, cudaStream_t s);
int launch_mixed(int etype, int form, const KArgs &a, int sms, cudaStream_t s);
// reference-order FP64 path (exact.cu): elements per tile of its block kernel,
// and the whole assembly (blocks + element-order two-bucket gather) into a.val
int exact_tile(int etype, int form, int npts);
void run_exact(fegpu_dofmap *dm, int form, KArgs &a, bool symmetric);
// D has the isotropic zero pattern with equal normal diagonal (d0), normal
// off-diagonal (d1) and shear diagonal (d3) entries
bool iso_pattern(const double *D, double &d0, double &d1, double &d3);
// elements per tile and the tile's shared memory for a form of the mixed path
// elements per mixed tile: wide = the persistent batch kernel's tile shape
int mixed_tile_for(int etype, int form, int npts, bool wide = true);
size_t mixed_smem_for(int etype, int form, int npts, int te);

// Node coordinates: column-major nnodes x sdim (device) -> [nnodes][4] (device).
void pack_geometry(const double *src_colmajor, int64_t nnodes, int sdim, double *xyz4,
                   cudaStream_t s);

// ---- shared by the entry points -----------------------------------------------------
KArgs base_args(fegpu_matrix *K, fegpu_dofmap *dm);
// builds with device checks: reads (and clears) the context's check word and
// throws FEGPU_ERR_DEVICE naming the first violation; otherwise nothing
void device_checks(fegpu_context *ctx, cudaStream_t s);
// work queued on s after this call may overwrite K's values: it first waits
// (on the device) for a copy of them still in flight to the host
void await_export(fegpu_matrix *K, cudaStream_t s);
bool is_isotropic(const double *D, double &lam, double &mu);
// loads the allocation-free entry point's static array on the current device
// and looks its address up (noalloc.cu); called when a context is created
void noalloc_prepare(int device);

// ---- matrix utilities -----------------------------------------------------------
void spmv(const fegpu_dofmap *dm, const double *val, const double *x, double *y,
          cudaStream_t s);
int64_t count_nonzeros(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val);
// CSR values -> the values of the same (symmetric) pattern read by columns:
// out[slot of (j, i) in row j] = val[slot of (i, j) in row i]
void transpose_values(const fegpu_dofmap *dm, const double *val, double *out, cudaStream_t s);
// CSC (1-based) of the block rows [r0, r1) x columns [c0, c1) of a matrix of the
// dofmap's pattern whose values are given by columns (exact zeros left out when
// drop_zeros); colptr == nullptr: only returns the block's stored entries
int64_t copy_block_csc(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val, int64_t r0,
                       int64_t r1, int64_t c0, int64_t c1, int drop_zeros, int64_t *colptr,
                       int64_t *rowval, double *nzval);
void copy_csc(fegpu_context *ctx, const fegpu_dofmap *dm, const double *val,
              int drop_zeros, int64_t *colptr, int64_t *rowval, double *nzval);
}  // namespace fegpu

// Generic COO assembler (matrix.cu): the triples of assemble! (host), or
// keys and values formed on the device; makematrix! leaves the result as
// sorted unique keys (column << 32 | row, 0-based) and values.
struct fegpu_assembler {
  fegpu_context *ctx = nullptr;
  int symmetric = 0;  // S + S^T completion (SparseSymm)
  int kind = 0;       // FEGPU_ASM_*
  int64_t nrows = 0, ncols = 0;
  std::vector<int64_t> I, J;
  std::vector<double> V;
  int64_t nnz = -1;
  fegpu::DevBuf keys, vals;
};

namespace fegpu {
// makematrix! on device COO data: key[t] = column << 32 | row (0-based),
// idx[t] = t, V[t] the value of triple t in assembly order; the stable sort
// sums duplicates in that order (sparse(I, J, V)), then the symmetric
// completion if the assembler is SparseSymm.  Returns the stored entries.
int64_t assembler_reduce(fegpu_assembler *a, DevBuf &key, DevBuf &idx, const double *V,
                         int64_t n);

}  // namespace fegpu
