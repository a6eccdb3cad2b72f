/*
 * fe_oracle.h -- CPU oracle for the FinEtools.jl assembly hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a serial, plain-C restatement of the
 * reference algorithm (FinEtools.jl v8.2.11), used to check the GPU library
 * and as the timed CPU baseline.  It is never linked into, loaded by or
 * called from the product library; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it.
 *
 * Parity pin: the oracle is checked against the reference's own known-answer
 * tests (assembler matrices in test/test_miscellaneous.jl:1939-2010 and
 * test/test_basics.jl:78-175, 1575-1610; patch/energy identities in
 * test/test_forms.jl:1-194, 301-535; colouring counts in
 * test/test_meshing.jl:7185-7244; node degrees in
 * test/test_miscellaneous.jl:931-949).  Julia is not available, so values are
 * not pinned bit-for-bit to the reference (which itself reorders arithmetic
 * through LoopVectorization @avx in src/MatrixUtilityModule.jl:486).
 *
 * Conventions: all node/DOF numbers that cross this interface are 1-based
 * (as in Julia); matrices are row-major unless stated otherwise.
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ORC_L2 (two-node line, src/FESetModule.jl:590-595) is an oracle-only type:
 * it runs the reference's one-dimensional known-answer tests. */
enum { ORC_Q4 = 0, ORC_H8 = 1, ORC_H20 = 2, ORC_T4 = 3, ORC_T10 = 4, ORC_L2 = 5 };
enum { ORC_DIFFUSION = 0, ORC_LIN_ELASTIC = 1, ORC_DOT = 2, ORC_DIV_GRAD = 3 };
enum { ORC_COEF_CONST = 0, ORC_COEF_PER_ELEMENT = 1, ORC_COEF_PER_QP = 2 };
/* SysmatAssemblerSparse, SysmatAssemblerSparseSymm, SysmatAssemblerSparseDiag,
 * SysmatAssemblerSparseHRZLumpingSymm (src/AssemblyModule.jl:88-329, 342-583,
 * 599-794, 943-1145) */
enum { ORC_ASM_SPARSE = 0, ORC_ASM_SPARSE_SYMM = 1, ORC_ASM_DIAG = 2, ORC_ASM_HRZ = 3 };

typedef struct {
  int etype;
  int64_t nelem;
  const int64_t *conn;    /* nelem x nne, row-major, 1-based node numbers   */
  int64_t nnodes;
  int sdim;
  const double *xyz;      /* nnodes x sdim, row-major                       */
  int ndn;
  const int64_t *dofnums; /* nnodes x ndn, row-major, 1-based DOF numbers   */
  int64_t nalldofs;
  int npts;
  const double *pc;       /* npts x mdim parametric coordinates, row-major  */
  const double *w;        /* npts weights                                   */
  double otherdim;        /* constant "other dimension" (thickness)         */
  const double *rm;       /* material frame: constant 3x3 rotation matrix,  */
                          /* row-major (CSys csmat), or NULL = identity     */
  int axisymmetric;       /* IntegDomain(..., axisymmetric = true)          */
  /* integrationdata() tables handed over by the caller (npts x nne and      */
  /* npts x nne x mdim, row-major), as the reference's forms take them from  */
  /* the FESet; NULL: computed here by bfun / bfundpar                       */
  const double *Ns;
  const double *dNs;
} orc_problem;

typedef struct {
  int kind;               /* ORC_COEF_*                                     */
  int ncomp;              /* values per (element | quadrature point)        */
  const double *data;
} orc_coef;

/* element-type facts */
int orc_nodesperelem(int etype);
int orc_manifdim(int etype);

/* integration rules (src/IntegRuleModule.jl:193-398, 470-516) */
int orc_gauss_rule(int dim, int order, double *pc, double *w);
int orc_tet_rule(int npts, double *pc, double *w);

/* basis functions (src/FESetModule.jl) */
void orc_bfun(int etype, const double *pc, double *N);
void orc_bfundpar(int etype, const double *pc, double *dN);

/* mesh generators (src/Mesh*Module.jl) */
void orc_linearspace(double start, double stop, int64_t n, double *out);
void orc_h8blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  const double *zs, int64_t nz, double *xyz, int64_t *conn);
void orc_t4blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  const double *zs, int64_t nz, double *xyz, int64_t *conn);
void orc_q4blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  double *xyz, int64_t *conn);
/* H8->H20 (etype_from=ORC_H8) or T4->T10 (ORC_T4).  Returns the new node
 * count; xyz_out must hold (nnodes + nelem*nedges) x 3 doubles and conn_out
 * nelem x nne_new. */
int64_t orc_quadratic_upgrade(int etype_from, int64_t nelem, const int64_t *conn,
                              int64_t nnodes, const double *xyz,
                              double *xyz_out, int64_t *conn_out);

/* node -> element map and greedy element colouring
 * (src/FENodeToFEMapModule.jl:44-74, src/MeshModificationModule.jl:1287-1365) */
int64_t orc_element_coloring(int64_t nelem, int nne, const int64_t *conn,
                             int64_t nnodes, int64_t *colors);

/* sparse matrix results (SparseMatrixCSC{Float64,Int64}, 1-based) */
typedef struct orc_matrix orc_matrix;
int64_t orc_matrix_nnz(const orc_matrix *m);
int64_t orc_matrix_nrows(const orc_matrix *m);
int64_t orc_matrix_ncols(const orc_matrix *m);
int64_t orc_matrix_zeros_dropped(const orc_matrix *m);
void orc_matrix_copy(const orc_matrix *m, int64_t *colptr, int64_t *rowval,
                     double *nzval);
void orc_matrix_free(orc_matrix *m);

/* generic assemblers (src/AssemblyModule.jl:88-583) */
typedef struct orc_assembler orc_assembler;
orc_assembler *orc_assembler_create(int kind, int64_t nrows, int64_t ncols);
int orc_assembler_assemble(orc_assembler *a, const double *mat_rowmajor,
                           int nr, int nc, const int64_t *rows,
                           const int64_t *cols);
orc_matrix *orc_assembler_make(orc_assembler *a);
void orc_assembler_free(orc_assembler *a);

/* the forms (src/FEMMBaseModule.jl:1207-1545, 1774-1824) */
orc_matrix *orc_bilform(const orc_problem *p, int form, const orc_coef *c,
                        int m, int asm_kind, double *phase_seconds);
int orc_linform_dot(const orc_problem *p, const orc_coef *f, int m, double *F);
orc_matrix *orc_bilform_convection(const orc_problem *p, const double *vel, int nsd);
/* bilform_masslike (src/FEMMBaseModule.jl:1865-1917): nelem*ndn x nalldofs */
orc_matrix *orc_bilform_masslike(const orc_problem *p, const orc_coef *c, int m);
const char *orc_last_error(void);

/* CSR node-adjacency degrees (connectionmatrix, src/FEMMBaseModule.jl:490-510) */
int64_t orc_connection_degrees(int64_t nelem, int nne, const int64_t *conn,
                               int64_t nnodes, int64_t *degree);

#ifdef __cplusplus
}
#endif
#endif
