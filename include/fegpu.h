/*
 * fegpu.h -- C ABI of the GB300 finite-element assembly library (libfegpu.so).
 *
 * The library replaces the element-by-element form evaluation and the sparse
 * COO->CSC assembly of FinEtools.jl (v8.2.11) for one GPU.  Every entry point
 * is plain C: opaque handles, host pointers and sizes; no CUDA or torch types.
 * A Julia caller reaches it through `ccall`; Python through ctypes.
 *
 * Conventions (identical to the Julia objects the reference passes around):
 *   - node and DOF numbers are 1-based;
 *   - connectivity is nelem x nne, row-major (Vector{NTuple{nne,Int}});
 *   - nodal values (geometry) and DOF numbers are nnodes x k, column-major
 *     (NodalField.values / NodalField.dofnums);
 *   - results are SparseMatrixCSC{Float64,Int64} arrays (colptr, rowval,
 *     nzval), 1-based.
 * Every function returns FEGPU_OK (0) or a nonzero status; the message of the
 * most recent failure on the calling thread is fegpu_last_error().
 * Handles are externally synchronised: one thread at a time per context.
 */
#ifndef FEGPU_H
#define FEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FEGPU_OK 0
#define FEGPU_ERR_ARG 1      /* invalid argument (sizes, numbers, kinds)     */
#define FEGPU_ERR_CUDA 2     /* CUDA runtime failure                          */
#define FEGPU_ERR_MEMORY 3   /* device allocation failed                      */
#define FEGPU_ERR_STATE 4    /* handle used out of order                      */
#define FEGPU_ERR_DEVICE 5   /* a device-side check failed (bad data)         */

/* element types (src/FESetModule.jl: FESetQ4 711, FESetH8 953, FESetH20
 * 1028, FESetT4 1342, FESetT10 1393) */
#define FEGPU_Q4 0
#define FEGPU_H8 1
#define FEGPU_H20 2
#define FEGPU_T4 3
#define FEGPU_T10 4

/* coefficient kinds: the DataCache forms a caller can hand over
 * (src/DataCacheModule.jl:65-112) */
#define FEGPU_COEF_CONST 0        /* one value set, as DataCache(data)        */
#define FEGPU_COEF_PER_ELEMENT 1  /* nelem x ncomp, row-major (per feid)      */
#define FEGPU_COEF_PER_QP 2       /* nelem x npts x ncomp (per feid, qpid)    */
#define FEGPU_COEF_ISO_LAME 3     /* nelem x 2 (lambda, mu): per-element      */
                                  /* isotropic elasticity                     */

/* arithmetic of the element kernels */
#define FEGPU_FP64 0   /* FP64 in the reference's own operation order: for    */
                       /* bilform_diffusion and bilform_lin_elastic the       */
                       /* matrix equals the reference algorithm's bit for     */
                       /* bit (element arithmetic without FMA contraction,    */
                       /* sums in element order, S + S' completion), so the   */
                       /* exact zeros makematrix! leaves out are the same     */
#define FEGPU_MIXED 1  /* FP32 bulk (FP64 geometry for distorted elements,    */
                       /* FP64 global accumulation)                           */
#define FEGPU_FP64_FAST 2 /* FP64 with fused multiply-adds and Gram-sum       */
                       /* element blocks, colour-ordered sums: within         */
                       /* 1e-12 |K_ij| + 1e-14 max_k |K_ik| of FEGPU_FP64,    */
                       /* several times faster; entries the reference forms   */
                       /* by exact cancellation may come out as ~1e-17        */
                       /* residues instead of exact zeros                     */

typedef struct fegpu_context fegpu_context;
typedef struct fegpu_femm fegpu_femm;
typedef struct fegpu_dofmap fegpu_dofmap;
typedef struct fegpu_matrix fegpu_matrix;
typedef struct fegpu_vector_assembler fegpu_vector_assembler;
typedef struct fegpu_assembler fegpu_assembler;

typedef struct {
  int kind;            /* FEGPU_COEF_*                                       */
  int ncomp;           /* values per element / quadrature point              */
  const double *data;  /* host pointer                                       */
} fegpu_coef;

/* Message of the last failed call on this thread ("" if none). */
const char *fegpu_last_error(void);

/* ---- context: one GPU, one CUDA stream ---------------------------------- */
int fegpu_context_create(int device, fegpu_context **out);
int fegpu_context_destroy(fegpu_context *ctx);
int fegpu_context_synchronize(fegpu_context *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or record events around library calls.  No reference counterpart:
 * interoperability only. */
int fegpu_context_stream(fegpu_context *ctx, void **stream);
/* Kernel accounting (no reference counterpart): with timing enabled, every
 * form records CUDA events around its element-kernel launches on the
 * context's stream; kernel_stats returns the accumulated element-kernel time
 * (ms) and the number of kernels the library launched, and resets them when
 * reset != 0. */
int fegpu_context_timing(fegpu_context *ctx, int enable);
/* Whether the loaded library checks device indices (no reference counterpart: the
 * reference's assemble! bounds-checks every DOF, src/AssemblyModule.jl:
 * 519-524).  A library built with FEGPU_DEVICE_CHECKS (build.py
 * --device-checks, libfegpu_checked.so) checks in its kernels the node
 * numbers they read and the CSR slots and vector entries they write, skips an
 * access out of range and records the first one; the entry point then
 * returns FEGPU_ERR_DEVICE naming it.  Regular builds compile the checks
 * away. */
int fegpu_context_device_checks(fegpu_context *ctx, int *enabled);
/* Self-test of the integer-unit FP64 addition that the reference-order path
 * uses for part of its sums (no reference counterpart): n operand pairs
 * (uniform bit patterns, close exponents, near-cancellations, ties to even)
 * from the seed, each summed by the routine and by the FP64 unit on the
 * device; the number of results that differ in any bit (0 expected) and the
 * index of the first (-1 if none). */
int fegpu_selftest_soft_add(fegpu_context *ctx, int64_t n, uint64_t seed, int64_t *mismatches,
                            int64_t *first);
int fegpu_context_kernel_stats(fegpu_context *ctx, double *kernel_ms, int64_t *launches,
                               int reset);

/* ---- FEMMBase: element set + integration data, resident on the device ---
 * Replaces FEMMBase(IntegDomain(fes, rule[, otherdimension]))
 * (src/FEMMBaseModule.jl:72-84, src/IntegDomainModule.jl:43-143) together
 * with integrationdata() (src/IntegDomainModule.jl:610-648): the caller
 * passes the basis-function tables the reference computes at the quadrature
 * points (Ns: npts x nne, gradNparams: npts x nne x mdim, row-major; w: npts)
 * so that the kernels use exactly the caller's rule.  Builds the node ->
 * element map and the greedy element colouring of element_coloring!
 * (src/FENodeToFEMapModule.jl:44-74, src/MeshModificationModule.jl:1287-1365). */
int fegpu_femm_create(fegpu_context *ctx, int etype, int64_t nelem,
                      const int64_t *conn, int64_t nnodes, int npts,
                      const double *Ns, const double *gradNparams,
                      const double *w, double otherdimension,
                      fegpu_femm **out);
int fegpu_femm_destroy(fegpu_femm *femm);
/* geometry NodalField values (nnodes x sdim, column-major), uploaded and kept
 * resident; call again to move the nodes (re-assembly on new coordinates). */
int fegpu_femm_set_geometry(fegpu_femm *femm, int sdim, const double *xyz);
/* IntegDomain(fes, rule, axisymmetric = true) (src/IntegDomainModule.jl:43-143):
 * a two-manifold measured as a volume is scaled by 2 pi r at each point (r:
 * the point's first coordinate, src/IntegDomainModule.jl:521-549) instead of
 * the other dimension.  Default 0. */
int fegpu_femm_set_axisymmetric(fegpu_femm *femm, int axisymmetric);
/* element colours (1-based, element order) and their count. */
int fegpu_femm_colors(fegpu_femm *femm, int64_t *colors, int64_t *ncolors);

/* ---- DOF map: NodalField dofnums -> CSR pattern built on the device ------
 * Replaces the structure half of makematrix! (the sparse() call,
 * src/AssemblyModule.jl:319, 567) and connectionmatrix
 * (src/FEMMBaseModule.jl:490-510).  dofnums: nnodes x ndn column-major,
 * 1-based, every DOF numbered (src/FieldModule.jl:328-377); nalldofs as
 * returned by nalldofs(u).  Reports the structural nnz. */
int fegpu_dofmap_create(fegpu_femm *femm, int ndn, const int64_t *dofnums,
                        int64_t nalldofs, fegpu_dofmap **out, int64_t *nnz);
int fegpu_dofmap_destroy(fegpu_dofmap *dm);
/* structural pattern as CSC (symmetric, so CSC == CSR), 1-based. */
int fegpu_dofmap_copy_pattern(fegpu_dofmap *dm, int64_t *colptr, int64_t *rowval);

/* ---- global matrix resident on the device --------------------------------
 * The device-side counterpart of SysmatAssemblerSparseSymm / Sparse
 * (src/AssemblyModule.jl:88-583): values live in the dofmap's CSR pattern. */
int fegpu_matrix_create(fegpu_dofmap *dm, fegpu_matrix **out);
int fegpu_matrix_destroy(fegpu_matrix *K);
/* The assembler the matrix stands for: symmetric = 1 (the default)
 * SysmatAssemblerSparseSymm, 0 SysmatAssemblerSparse
 * (src/AssemblyModule.jl:88-329, 454-583).  The FEGPU_FP64 forms group their
 * sums as that assembler does (S + S' of the lower-triangle triples, or S of
 * all triples), which decides the last bits of the values. */
int fegpu_matrix_set_symmetric_assembly(fegpu_matrix *K, int symmetric);

/* The forms.  Each one assembles every element into K deterministically:
 * FEGPU_FP64 by the element-ordered row gather (the reference's own sums,
 * bit for bit), FEGPU_FP64_FAST by the colour-ordered scatter, FEGPU_MIXED by
 * the float-float row gather.
 *   bilform_diffusion: src/FEMMBaseModule.jl:1462-1545 (scalar ncomp = 1 ->
 *     _bilform_diffusion_iso, mdim x mdim -> _bilform_diffusion_general);
 *   bilform_lin_elastic(DeforModelRed3D): src/FEMMBaseModule.jl:1774-1824
 *     (ncomp = 36: 6x6 D in Voigt order xx,yy,zz,xy,xz,yz, row-major,
 *     constant, per element, or per point with FEGPU_FP64 only (the other
 *     precisions apply one D per element to its point-summed gradient
 *     products); or FEGPU_COEF_ISO_LAME);
 *   bilform_dot: src/FEMMBaseModule.jl:1335-1376 (ncomp = ndn*ndn; m is the
 *     manifold dimension of the measure, as in Jacobianmdim).
 * symmetric = 1 reproduces SysmatAssemblerSparseSymm (the element matrix's
 * lower triangle by local index, mirrored), 0 reproduces SysmatAssemblerSparse. */
int fegpu_bilform_diffusion(fegpu_matrix *K, const fegpu_coef *cf, int precision);
int fegpu_bilform_lin_elastic(fegpu_matrix *K, const fegpu_coef *cf, int precision);
/* bilform_convection: src/FEMMBaseModule.jl:1583-1625, scalar field (one DOF
 * per node); velocity: nnodes x nsd column-major (NodalField values), nsd =
 * the space = manifold dimension.  The reference's default assembler is
 * SysmatAssemblerSparse (copy out with drop_zeros = 0); its density rhof
 * does not enter the matrix and is not an argument. */
int fegpu_bilform_convection(fegpu_matrix *K, int nsd, const double *velocity);
/* bilform_div_grad: src/FEMMBaseModule.jl:1672-1723 (3-D, ndn = 3; scalar
 * viscosity, constant or per element).  The reference's default assembler is
 * SysmatAssemblerSparse: copy out with drop_zeros = 0. */
int fegpu_bilform_div_grad(fegpu_matrix *K, const fegpu_coef *cf, int precision);
int fegpu_bilform_dot(fegpu_matrix *K, const fegpu_coef *cf, int m, int symmetric,
                      int precision);

/* linform_dot / distribloads (src/FEMMBaseModule.jl:1207-1297) into a dense
 * vector, SysvecAssembler semantics (src/AssemblyModule.jl:853-917).
 * f: ncomp = ndn.  F: nalldofs doubles (host). */
int fegpu_linform_dot(fegpu_dofmap *dm, const fegpu_coef *f, int m, double *F);
/* bilform_dot assembled by SysmatAssemblerSparseDiag (hrz = 0,
 * src/AssemblyModule.jl:722-750) or SysmatAssemblerSparseHRZLumpingSymm
 * (hrz = 1, src/AssemblyModule.jl:1065-1095): the diagonal of the lumped
 * matrix (nalldofs values; the matrix is diag(diag) on the DOFs of the
 * element set).  Coefficient: scalar (constant, per element, per point) or a
 * constant ndn x ndn matrix. */
int fegpu_bilform_dot_lumped(fegpu_dofmap *dm, const fegpu_coef *f, int m, int hrz,
                             double *diag);

/* makematrix! output.  drop_zeros = 1 leaves out entries that are exactly
 * zero, as the S + transpose(S) step of SysmatAssemblerSparseSymm does
 * (src/AssemblyModule.jl:576); 0 keeps the structural pattern (as
 * SysmatAssemblerSparse's sparse() does). */
int fegpu_matrix_nnz(fegpu_matrix *K, int drop_zeros, int64_t *nnz);
int fegpu_matrix_copy_csc(fegpu_matrix *K, int drop_zeros, int64_t *colptr,
                          int64_t *rowval, double *nzval);
/* values only, in the structural pattern order (re-assembly on a fixed mesh) */
int fegpu_matrix_copy_values(fegpu_matrix *K, double *nzval);
/* The same copy without waiting for it (no reference counterpart: the
 * reference's makematrix! hands back a host matrix at once): queued on the
 * context's export stream behind the work already queued for K, it overlaps
 * what the caller queues next (the next assembly into another matrix, a
 * coordinate upload).
 * nzval should be page-locked host memory and stays in use until
 * fegpu_matrix_wait_export(K) returns.  A form that writes K again waits on
 * the device for the copy first, so two matrices of one dofmap used in turn
 * pipeline the assembly of one with the export of the other. */
int fegpu_matrix_copy_values_async(fegpu_matrix *K, double *nzval);
int fegpu_matrix_wait_export(fegpu_matrix *K);
/* A block of the matrix as CSC (1-based, (row1-row0) x (col1-col0)): rows
 * [row0, row1) x columns [col0, col1), 0-based half-open -- matrix_blocked_ff
 * / _fd / _df / _dd and the makematrix! of SysmatAssemblerFFBlock
 * (src/MatrixUtilityModule.jl:675-806, src/AssemblyModule.jl:1229-1236) with
 * the free DOFs numbered first.  drop_zeros = 0 keeps the stored entries
 * (explicit zeros included: a SysmatAssemblerSparse matrix), 1 leaves out
 * exact zeros (a SysmatAssemblerSparseSymm matrix, whose S + S' stores
 * none).  Call with colptr = rowval = nzval = NULL for the entry count, then
 * again with arrays of (col1 - col0 + 1) and *nnz entries. */
int fegpu_matrix_copy_block_csc(fegpu_matrix *K, int64_t row0, int64_t row1, int64_t col0,
                                int64_t col1, int drop_zeros, int64_t *nnz, int64_t *colptr,
                                int64_t *rowval, double *nzval);
/* y = K x on the device (host vectors of length nalldofs) */
int fegpu_matrix_spmv(fegpu_matrix *K, const double *x, double *y);
/* conjugategradient(K, b, x0, maxiter) (src/AlgoBaseModule.jl:425-445): the
 * reference's iteration, every step on the device; host vectors of length
 * nalldofs; the result goes to x. */
int fegpu_matrix_cg(fegpu_matrix *K, const double *b, const double *x0, int maxiter,
                    double *x);

/* Allocation-free mixed-precision bilform_lin_elastic.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory once they
 * run -- a framework whose pool allocator has reserved the GPU, or a
 * time-step loop that must not hit cudaMalloc's device-wide synchronisation.
 * Same arguments and result as fegpu_bilform_lin_elastic(K, cf, FEGPU_MIXED);
 * all scratch (element-block ring, node gather order, per-element
 * coefficients) lives in one static device array of
 * FEGPU_NOALLOC_SCRATCH_BYTES, which fegpu_context_create loads (and looks
 * its device address up) on its device, so that GPU holds it from then until
 * the process exits; meshes whose scratch would not fit are rejected with an
 * error.  Calls no cudaMalloc or cudaFree.  Preconditions: one regular
 * FEGPU_MIXED assembly on the same matrix has run (it builds the
 * node-to-element tables read here).  The call blocks the host until its
 * work is done.  Calls share the array (it keeps the last call's contents):
 * calls whose GPU work overlaps race. */
#define FEGPU_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int fegpu_bilform_lin_elastic_noalloc(fegpu_matrix *K, const fegpu_coef *cf);

/* ---- batches: many assemblies in one persistent launch ---------------------
 * A batch replaces a host loop of bilform calls over many FEMMs -- each one
 * bilform_diffusion (src/FEMMBaseModule.jl:1462-1545), bilform_lin_elastic
 * (1774-1824) or bilform_dot (1335-1376) with SysmatAssemblerSparseSymm --
 * by one persistent kernel over a work queue of element tiles and row-gather
 * ranges of all of them (any mix of element types and sizes), replayed as a
 * CUDA graph.  Every job is evaluated as the FEGPU_MIXED path and its matrix
 * is identical to fegpu_bilform_*(K, cf, FEGPU_MIXED) (bilform_dot: the
 * symmetric arrangement).  Batched kinds: diffusion (scalar coefficient:
 * constant, per element or per point) on Q4/H8/H20/T4/T10; linear elasticity
 * (isotropic D or per-element Lame pairs) on H8/H20/T4/T10; dot (scalar
 * coefficient, or a constant ndn x ndn matrix; ndn 1 or 3) on Q4 (m = 2 or
 * 3) and H8.  Each matrix takes part in at most one job of a batch.
 * Waits inside the kernel are bounded (default 5 s each,
 * fegpu_batch_set_wait_limit): one that runs out makes fegpu_batch_wait /
 * run return FEGPU_ERR_DEVICE. */
#define FEGPU_FORM_DIFFUSION 0
#define FEGPU_FORM_LIN_ELASTIC 1
#define FEGPU_FORM_DOT 2
typedef struct fegpu_batch fegpu_batch;
int fegpu_batch_create(fegpu_context *ctx, fegpu_batch **out);
int fegpu_batch_destroy(fegpu_batch *b);
/* adds a job; its index goes to *job (may be null).  m: dot manifold
 * dimension (ignored by the other forms).  Coefficient values are copied. */
int fegpu_batch_add(fegpu_batch *b, fegpu_matrix *K, int form, const fegpu_coef *cf,
                    int m, int64_t *job);
/* new coefficient values for a job (same form); the captured graph stays */
int fegpu_batch_set_coef(fegpu_batch *b, int64_t job, const fegpu_coef *cf);
/* autotuner: elements per tile for each job kind, timed on the largest job
 * of that kind; cache_path (or null) keeps "<kind> <tile>" lines across runs */
int fegpu_batch_tune(fegpu_batch *b, const char *cache_path);
int fegpu_batch_tile(fegpu_batch *b, int64_t job, int *elements_per_tile);
int fegpu_batch_set_wait_limit(fegpu_batch *b, double seconds);
/* Test of the failure path (no reference counterpart): job >= 0 withholds the
 * completion count of that job's first element stage, a counter nothing else
 * raises, so the items that depend on it wait until the wait limit, the
 * kernel skips the rest and ends, and fegpu_batch_wait returns
 * FEGPU_ERR_DEVICE; job = -1 restores normal runs.  No device fault is
 * involved: every wait is bounded. */
int fegpu_batch_withhold(fegpu_batch *b, int64_t job);
/* launch (asynchronous, on the context stream) / wait and check / both */
int fegpu_batch_launch(fegpu_batch *b);
int fegpu_batch_wait(fegpu_batch *b);
int fegpu_batch_run(fegpu_batch *b);
int fegpu_batch_stats(fegpu_batch *b, int64_t *jobs, int64_t *items);

/* ---- serving loop: re-assembly requests on resident meshes -----------------
 * No reference counterpart (the reference assembles on demand, one call per
 * matrix): a server keeps meshes resident on the device -- the handles of a
 * matrix (femm, dofmap, matrix) plus its form and coefficient, registered once
 * -- and accepts requests that carry new per-element coefficients
 * (FEGPU_REQUEST_COEF: the same layout as the coefficient the mesh was added
 * with) or new node coordinates (FEGPU_REQUEST_COORDS: nnodes x sdim,
 * column-major, as geom.values).  A worker thread launches the persistent
 * kernel on `lanes` CUDA streams.  When a lane is free its next launch holds
 * the next slice of every request running on it (a slice: at most
 * slice_elements of the mesh's elements in whole chunks,
 * fegpu_server_set_slice, default 16384) and the oldest waiting request of
 * every mesh with none running, up to max_jobs; a launch covers 1/(1 + lanes
 * running) of the GPU (all of it when the other lanes are idle).  A large
 * request therefore runs over several launches of its lane, and requests that
 * arrive meanwhile start on another lane or join its next launch.  Requests of
 * one mesh complete in submission order; a
 * request's result is the mesh's matrix (values on the device, read with
 * fegpu_matrix_copy_values before the mesh's next request completes).  Every
 * request is evaluated as the batch path (FEGPU_MIXED) and its matrix does
 * not depend on what else shared its launches.  Latency = completion (host
 * callback behind the kernel) - submit.  The data passed to
 * fegpu_server_submit is copied; the matrices must outlive the server; a
 * coordinates request also changes the femm's geometry. */
#define FEGPU_REQUEST_COEF 0
#define FEGPU_REQUEST_COORDS 1
typedef struct fegpu_server fegpu_server;
int fegpu_server_create(fegpu_context *ctx, int lanes, int max_jobs, fegpu_server **out);
int fegpu_server_destroy(fegpu_server *s);
/* FEGPU_MIXED (default) or, before the first mesh is added, FEGPU_FP64 /
 * FEGPU_FP64_FAST: the worker then runs each request by itself through the
 * single-call form on the context's stream, in arrival order (the caller does
 * not use that context meanwhile). */
int fegpu_server_set_precision(fegpu_server *s, int precision);
int fegpu_server_set_slice(fegpu_server *s, int64_t elements);
/* Admission: fegpu_server_add_mesh returns FEGPU_ERR_MEMORY when the device
 * memory the mesh still needs to be served (gather plan, block ring,
 * coefficient and staging buffers) exceeds the free memory less a 256 MB
 * reserve, or when a limit is set (bytes > 0) and the meshes' total device
 * memory (their femm, pattern and values included) would exceed it; meshes
 * can be added and removed while requests stream. */
int fegpu_server_set_memory_limit(fegpu_server *s, int64_t bytes);
int fegpu_server_add_mesh(fegpu_server *s, fegpu_matrix *K, int form, const fegpu_coef *cf,
                          int m, int64_t *mesh_id);
/* stops serving a mesh (none of its requests waiting or in flight, else
 * FEGPU_ERR_STATE) and frees what serving it added; the caller then destroys
 * its matrix, dofmap and femm. */
int fegpu_server_remove_mesh(fegpu_server *s, int64_t mesh_id);
/* device bytes a served mesh holds (mesh_id < 0: all of them) */
int fegpu_server_mesh_bytes(fegpu_server *s, int64_t mesh_id, int64_t *bytes);
/* device bytes a mesh of this size needs to be created and served (femm,
 * pattern, values, serving structures), from the average node degree of the
 * element type: an estimate for admission before anything is allocated */
int fegpu_estimate_mesh_bytes(int etype, int64_t nelem, int64_t nnodes, int ndn,
                              int64_t *bytes);
int fegpu_server_submit(fegpu_server *s, int64_t mesh_id, int kind, const double *data,
                        int64_t count, int64_t *request_id);
/* a request still waiting is withdrawn (its wait returns FEGPU_ERR_STATE);
 * one already running or done: FEGPU_ERR_STATE */
int fegpu_server_cancel(fegpu_server *s, int64_t request_id);
/* blocks until the request completed; its latency in ms; collects it */
int fegpu_server_wait(fegpu_server *s, int64_t request_id, double *latency_ms);
/* blocks until no request is waiting or in flight */
int fegpu_server_drain(fegpu_server *s);
/* hold = 1: no new launches (requests accumulate, e.g. during maintenance or
 * to admit a burst at once); hold = 0: resume */
int fegpu_server_hold(fegpu_server *s, int hold);
/* launches, request slices run, requests waiting */
int fegpu_server_stats(fegpu_server *s, int64_t *batches, int64_t *jobs, int64_t *pending);
/* free and total device memory */
int fegpu_server_memory(fegpu_server *s, int64_t *free_bytes, int64_t *total_bytes);

/* ---- generic assembler for element matrices formed on the host -----------
 * startassembly! / assemble! / makematrix! of SysmatAssemblerSparse(Symm)
 * (src/AssemblyModule.jl:209-329, 454-583) for FEMMs whose element matrices
 * are computed by the caller: triples are buffered on the host, then sorted
 * and reduced on the device into CSC (duplicates summed in input order).
 * kind: 0 SysmatAssemblerSparse, 1 SysmatAssemblerSparseSymm,
 * 2 SysmatAssemblerSparseDiag (element diagonals, src/AssemblyModule.jl:
 * 722-750), 3 SysmatAssemblerSparseHRZLumpingSymm (diagonals scaled by the
 * element total over the diagonal total, 1065-1095). */
#define FEGPU_ASM_SPARSE 0
#define FEGPU_ASM_SPARSE_SYMM 1
#define FEGPU_ASM_SPARSE_DIAG 2
#define FEGPU_ASM_HRZ_LUMPING_SYMM 3
int fegpu_assembler_create(fegpu_context *ctx, int kind, int64_t nrows,
                           int64_t ncols, fegpu_assembler **out);
int fegpu_assembler_destroy(fegpu_assembler *a);
int fegpu_assembler_assemble(fegpu_assembler *a, const double *mat_colmajor,
                             int nr, int nc, const int64_t *rows,
                             const int64_t *cols);
int fegpu_assembler_make(fegpu_assembler *a, int64_t *nnz);
int fegpu_assembler_copy_csc(fegpu_assembler *a, int64_t *colptr,
                             int64_t *rowval, double *nzval);

/* bilform_masslike (src/FEMMBaseModule.jl:1865-1917): the rectangular matrix
 * of nelem*ndn rows (rows (i-1)*ndn+1 .. i*ndn belong to element i, element
 * order) and nalldofs columns, M[(i-1)*ndn+p, dof(b,q)] = sum N_b Jac w c[p,q]
 * with Jac = Jacobianmdim(m).  The element blocks are formed on the device
 * and reduced into `a`, which must be a FEGPU_ASM_SPARSE assembler of size
 * nelem*ndn x nalldofs (the reference's default SysmatAssemblerSparse; its
 * startassembly! drops triples assembled before).  c: constant, per element
 * or per quadrature point (element order); a scalar or ndn x ndn row-major.
 * Afterwards the assembler holds the made matrix: *nnz entries, copied out
 * with fegpu_assembler_copy_csc. */
int fegpu_bilform_masslike(fegpu_dofmap *dm, const fegpu_coef *cf, int m,
                           fegpu_assembler *a, int64_t *nnz);

#ifdef __cplusplus
}
#endif
#endif
