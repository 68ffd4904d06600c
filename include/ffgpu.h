/*
 * ffgpu.h -- C ABI of the GB300-native FreeFEM assemble-and-solve library (libffgpu.so).
 *
 * Plain C types only: pointers, sizes and POD structs.  Every array argument may live in
 * host memory or in device memory of the context's GPU; host arrays are copied in (and
 * results copied out) inside the call, which is synchronous on return.  Every function
 * returns FFGPU_OK (0) or a negative FFGPU_E* code; ffgpu_last_error() gives the message.
 *
 * Each entry point names the FreeFEM interface it replaces (file:line in FreeFEM-sources).
 */
#ifndef FFGPU_H
#define FFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define FFGPU_OK 0
#define FFGPU_EINVAL (-1)    /* bad argument (sizes, layout, unsupported form)       */
#define FFGPU_ECUDA (-2)     /* CUDA runtime error                                   */
#define FFGPU_ENOCONV (-3)   /* Krylov solver hit its iteration cap (FreeFEM: ffassert) */
#define FFGPU_EMESH (-4)     /* mesh/space inconsistency found on the device          */
#define FFGPU_ENOMEM (-5)    /* device allocation failed                              */

/* finite elements: FreeFEM's P1, P2 and the vector space [P2,P2,P2] on tetrahedra */
#define FFGPU_FE_P1 1
#define FFGPU_FE_P2 2
#define FFGPU_FE_P2VEC3 3

/* bilinear forms (grad/div operators with P0 coefficients) */
#define FFGPU_FORM_DIFFUSION 0  /* int(c_stiff*kappa*grad(u).grad(v) + c_mass*u*v)      */
#define FFGPU_FORM_ELASTICITY 1 /* int(lambda*div(u)div(v) + 2mu*eps(u):eps(v)), [P2]^3 */

typedef struct ffgpu_ctx ffgpu_ctx;
typedef struct ffgpu_space ffgpu_space;
typedef struct ffgpu_matrix ffgpu_matrix;

/* One boundary term of a varf: int1d(Th, labels)(...) in 2D, int2d(Th, labels)(...) on the
 * boundary faces in 3D, on the space's boundary elements (ffgpu_space_set_boundary) whose label
 * is one of labels[0..nlabels) (nlabels = 0: every boundary element).  Each is integrated on the
 * edge/face of its adjacent element as FreeFEM's Element_Op / Element_rhs on a boundary edge or
 * face do (problem.cpp:6222-6262, 6516-6560, 8517-8580, 8612-8683): 3-point Gauss-Legendre on
 * an edge, the 7-point degree-5 rule on a face.
 *   robin: coefficient of u.v (of u_c v_c for every component c of [P2,P2,P2]), per boundary
 *          element (length nbe) or NULL, then robin_const (0 = no matrix term);
 *   g:     source of the linear term g.v per boundary element and component (nbe*ncomp) or
 *          NULL, then g_const[c].  Like f, it enters b = a(0,Vh) with a plus sign. */
typedef struct {
    int nlabels;
    const int32_t *labels;
    const double *robin;
    double robin_const;
    const double *g;
    double g_const[3];
} ffgpu_bterm;

/* ------------------------------------------------------------------ coefficient expressions
 * A coefficient or source of a varf term as an expression of the point, evaluated on the
 * device at every quadrature point, as FreeFEM's Element_Op / Element_rhs evaluate the term's
 * expression (optiexpK / the C_F0 of the term) at each point of the rule
 * (problem.cpp:6117-6132, 6391-6410, 7880-7900).  A postfix program over a stack of doubles
 * (depth <= 16):
 *   FFGPU_OP_CONST k     push consts[k]
 *   FFGPU_OP_X/Y/Z       push the point's coordinate (x = sum_i lambda_i X_i)
 *   FFGPU_OP_FE k        push FE function fe[k] at the point
 *   FFGPU_OP_DX/DY/DZ k  push a derivative of FE function fe[k] (P1, P2) at the point
 *   FFGPU_OP_ADD SUB MUL DIV POW MIN MAX     pop b, pop a, push a op b
 *   FFGPU_OP_NEG EXP LOG SQRT SIN COS TAN ABS TANH ATAN      pop a, push f(a)
 * The operand k follows its opcode in ops[].  Functions are CUDA's own (exp, log, ...). */
#define FFGPU_OP_CONST 1
#define FFGPU_OP_X 2
#define FFGPU_OP_Y 3
#define FFGPU_OP_Z 4
#define FFGPU_OP_FE 5
#define FFGPU_OP_DX 6
#define FFGPU_OP_DY 7
#define FFGPU_OP_DZ 8
#define FFGPU_OP_ADD 16
#define FFGPU_OP_SUB 17
#define FFGPU_OP_MUL 18
#define FFGPU_OP_DIV 19
#define FFGPU_OP_POW 20
#define FFGPU_OP_MIN 21
#define FFGPU_OP_MAX 22
#define FFGPU_OP_NEG 32
#define FFGPU_OP_EXP 33
#define FFGPU_OP_LOG 34
#define FFGPU_OP_SQRT 35
#define FFGPU_OP_SIN 36
#define FFGPU_OP_COS 37
#define FFGPU_OP_TAN 38
#define FFGPU_OP_ABS 39
#define FFGPU_OP_TANH 40
#define FFGPU_OP_ATAN 41

/* an FE function of the mesh by its DOF values (FreeFEM's u[] of a P0/P1/P2 fespace):
 *   kind 0 (P0): values[element];  FFGPU_FE_P1: values[vertex];
 *   FFGPU_FE_P2: values[dof[element*nloc + i]] with FreeFEM's local P2 order (vertices, then the
 *   edges: opposite vertex 0,1,2 in 2D; 01,02,03,12,13,23 in 3D); dof = NULL: the assembled
 *   space's own DOF table (the space must then be P2). */
#define FFGPU_FE_P0 0
typedef struct {
    int kind;
    const double *values;
    const int32_t *dof;
} ffgpu_fefunc;

typedef struct {
    int nops;
    const int32_t *ops;
    const double *consts;
    int nfe;
    const ffgpu_fefunc *fe;
} ffgpu_expr;

/* A volume term of a scalar (P1/P2) varf: int(Th)(coef * op_i(v) * op_j(u)), op 0 = value,
 * 1 = d/dx, 2 = d/dy, 3 = d/dz (FreeFEM's term tuple ((icomp,iop),(jcomp,jop)) of a
 * FormBilinear, problem.cpp:6123-6132, for the scalar component); coef = c * expr(x), expr
 * NULL meaning 1.  Integrated with the varf's rule (nqp points), added to the form's matrix. */
typedef struct {
    int iop, jop;
    double c;
    const ffgpu_expr *expr;
} ffgpu_term;

/* varf description.  kappa: P0 coefficient per element (length nt) or NULL (= 1);
 * the stiffness term is c_stiff*kappa_e, the mass term c_mass (0 = none).
 * Elasticity uses E and nu (mu = E/(2(1+nu)), lambda = E nu/((1+nu)(1-2nu))).
 * f: P0 source per element and component (nt*ncomp) or NULL, then f_const[c] applies.
 * bterms[0..nbterms): boundary terms, added after the volume terms and before on(...).
 * f_qp: a source of any form, given by its values at the points of a quadrature rule, as
 *   Element_rhs evaluates it (problem.cpp:7839-7911, 2D; 7917-7990, 3D): f_qp[(k*nqp + q)*ncomp
 *   + c] at the point of barycentric coordinates qp_lambda[q*(dim+1) .. +dim] of element k, the
 *   rule's weights qp_weight[q] relative to the element measure (nqp <= 64).  When non-NULL it
 *   replaces f and f_const: b_i += |K| sum_q qp_weight[q] f_q phi_i(lambda_q). */
typedef struct {
    int form;
    const double *kappa;
    double c_stiff, c_mass;
    double E, nu;
    const double *f;
    double f_const[3];
    int nbterms;
    const ffgpu_bterm *bterms;
    int nqp;
    const double *qp_lambda;
    const double *qp_weight;
    const double *f_qp;
    /* mass_qp: the coefficient of u*v (diffusion form) at the points of the same rule,
     * mass_qp[k*nqp + q]; when non-NULL it replaces c_mass: the element matrix gains
     * |K| sum_q qp_weight[q] c_q phi_i(lambda_q) phi_j(lambda_q) (Element_Op,
     * problem.cpp:6063-6160, 6337-6437). */
    const double *mass_qp;
    /* stiff_qp: the coefficient of grad u . grad v (diffusion form) at the points of the same
     * rule, stiff_qp[k*nqp + q]; when non-NULL it replaces kappa and c_stiff: the element matrix
     * gains |K| sum_q qp_weight[q] k_q grad phi_i(lambda_q) . grad phi_j(lambda_q). */
    const double *stiff_qp;
    /* lame: per-element Lame coefficients of the elasticity form, lame[2k] = lambda_k,
     * lame[2k+1] = mu_k (several materials), or NULL (then E and nu). */
    const double *lame;
    /* f_expr: the volume source as expressions evaluated on the device at the points of the
     * rule (nqp, qp_lambda, qp_weight), one per component (ncomp entries), or NULL.  When
     * non-NULL it replaces f, f_const and f_qp. */
    const ffgpu_expr *f_expr;
    /* terms[0..nterms): general volume terms of a scalar space (diffusion form), evaluated
     * with the same rule and added to the matrix after kappa/c_mass/mass_qp/stiff_qp. */
    int nterms;
    const ffgpu_term *terms;
} ffgpu_varf;

/* Dirichlet data of `on(labels, u=g)`.  Either onbc[dof] != 0 marks the DOFs directly, or
 * (onbc == NULL) the device marks them from the space's boundary elements
 * (ffgpu_space_set_boundary) whose label is one of labels[0..nlabels), for the components in
 * comp_mask (bit c = component c; 0 = all), as AssembleBC does (problem.cpp:9881-10034).
 * g[dof] is the value (NULL = 0).  tgv > 0 follows HashMatrix::SetBC: A_ii := tgv,
 * b_i := tgv*g_i. */
typedef struct {
    const uint8_t *onbc;
    const double *g;
    double tgv;
    int nlabels;
    const int32_t *labels;
    int comp_mask;
} ffgpu_bc;

/* Krylov parameters, named as in FreeFEM's Data_Sparse_Solver (VirtualSolver.hpp:30-96).
 * eps > 0 relative, eps < 0 absolute (CG.cpp:226); itmax <= 0 means n (VirtualSolverCG.hpp:135);
 * dim_krylov is GMRES's restart (NbSpace; <= 0: FreeFEM's default, 1000).  unroll: CG iterations
 * per CUDA-graph body (>=1).
 * spmv_mode (CG): 0 = SpMV in FP64 arithmetic; 1 = FP64 values and vectors with the products
 * formed exactly on the FP32 pipe and summed as double-float (about 2^-44 relative), every
 * other CG operation in FP64.
 * spmv_layout: 0 = the layout the tuner picks for the matrix's shape (timed once per shape and
 * context, then kept); otherwise a fixed layout code as ffgpu_matrix_spmv_layout reports it:
 * 64..71 SELL-32 variants, or block CSR with 1, 2, 4, 8 lanes per block row (FP64), 64..67 or
 * 4, 8, 16, 32 lanes (double-float).  The layout fixes the summation order of the SpMV and the
 * fused dot products, so a fixed code gives bit-identical results from run to run.  With 0, the
 * environment variable FFGPU_SPMV_LAYOUT, when set, fixes the FP64 layout the same way. */
typedef struct {
    double eps;
    int itmax;
    int dim_krylov;
    double tgv;
    int verb;
    int unroll;
    int spmv_mode;
    int spmv_layout;
} ffgpu_solver_params;

/* Solver report: iterations (FreeFEM's nbitermax / getnbiteration), final C-norm^2 of the
 * preconditioned residual and its threshold eps2, converged flag. */
typedef struct {
    int iterations;
    int converged;
    double gcg, eps2;
    double residual;        /* GMRES: relative residual; IR: final outer ratio */
    int outer_iterations;   /* IR only */
    double elapsed_ms;      /* device time of the solve */
} ffgpu_solver_stats;

/* ------------------------------------------------------------------ context */
/* One context per GPU and host thread; owns a CUDA stream and reduction scratch. */
int ffgpu_ctx_create(int device, ffgpu_ctx **out);
int ffgpu_ctx_destroy(ffgpu_ctx *ctx);
/* thread-local message of the last failing call */
const char *ffgpu_last_error(void);
/* number of kernel executions this library issued on the context since creation; kernels
 * run inside a CUDA graph count once per execution of their graph node */
int64_t ffgpu_ctx_kernel_launches(const ffgpu_ctx *ctx);
/* the cudaStream_t (as void*) every call of this context runs on, for timing with events;
 * library bookkeeping with no FreeFEM counterpart */
void *ffgpu_ctx_stream(const ffgpu_ctx *ctx);

/* ------------------------------------------------------------------ mesh + FE space
 * Replaces reading Mesh/Mesh3 and the FESpace numbering FreeFEM hands to the assembly loop
 * (src/fflib/problem.cpp:803-1111 / 1117-1411 read Th[k] and Vh(k,i)).
 * coords: nv*dim doubles; elems: nt*(dim+1) vertex indices (mesh order);
 * dof: nt*ndofK global DOF numbers, FreeFEM's Vh(k,i) (FESpacen.hpp:651-662), where for
 * FFGPU_FE_P2VEC3 local DOF c*10+i is component c of scalar node i (dof = 3*node + c).
 * dof may be NULL for FFGPU_FE_P1 with ndof == nv: the DOFs are then the vertices, FreeFEM's
 * P1 numbering without periodic conditions (FESpace.cpp:698-701, GenericMesh.hpp:1760-1764).
 * Builds the node->element incidence on the device. */
int ffgpu_space_create(ffgpu_ctx *ctx, int dim, int nv, const double *coords, int nt,
                       const int32_t *elems, int fe, int ndofK, const int32_t *dof, int ndof,
                       ffgpu_space **out);
int ffgpu_space_destroy(ffgpu_space *space);
/* Boundary elements of the mesh (Th.be(k): nbe x dim vertex indices and labels), kept on the
 * device for `on(...)` marking; builds the vertex -> boundary-element incidence once. */
int ffgpu_space_set_boundary(ffgpu_space *space, int nbe, const int32_t *belems, const int32_t *blabel);
/* The DOF mask of on(labels) (ndof bytes, host or device), as the assembly computes it. */
int ffgpu_space_bc_mask(ffgpu_space *space, int nlabels, const int32_t *labels, int comp_mask,
                        uint8_t *onbc);

/* FreeFEM's structured meshes on [0,1]^dim, built on the device into caller arrays (host or
 * device): square(nx, ny) (Carre_, src/fflib/lgmesh.cpp:1229-1384) for dim 2 and
 * cube(nx, ny, nz) (BuildCube, src/fflib/msh3.cpp:7879-8132, 6 tetrahedra per hexahedron) for
 * dim 3, with FreeFEM's vertex, element and boundary-element order and labels.
 * coords[nv*dim], elems[nt*(dim+1)], belems[nbe*dim], blabel[nbe]; sizes from ffgpu_mesh_sizes. */
int ffgpu_mesh_sizes(int dim, int nx, int ny, int nz, int *nv, int *nt, int *nbe);
int ffgpu_mesh_build(ffgpu_ctx *ctx, int dim, int nx, int ny, int nz, double *coords, int32_t *elems,
                     int32_t *belems, int32_t *blabel);
/* P2 node table of a tetrahedral mesh on the device (host or device arrays): FreeFEM's
 * first-encounter numbering over the element slots (4 vertices, then the edges
 * 01 02 03 12 13 23) of GenericMesh::BuildDFNumbering (src/femlib/GenericMesh.hpp:1878-1929).
 * nodes[nt*10]; *nnodes = the node count.  (2D P2: ffgpu_number_p2_2d.) */
int ffgpu_number_p2(ffgpu_ctx *ctx, int nv, int nt, const int32_t *elems, int32_t *nodes, int *nnodes);
/* P2 node table of a triangular mesh (host code, host arrays), FreeFEM's two steps:
 * ConstructDataFElement::Make (src/femlib/FESpace.cpp:623-877) -- node of vertex v = v, then
 * edge nodes nv, nv+1, ... by first encounter over (triangle, local edge j = the edge opposite
 * vertex j) -- and FESpace::renum (src/femlib/gibbs.cpp:1094-1166), the Gibbs profile
 * renumbering of the node graph, kept when the profile does not grow.
 * elems[nt*3]; nodes[nt*6] out (3 vertices, then the edges opposite vertices 0, 1, 2, as
 * FreeFEM's Vh(k,i) lists the DOFs of scalar P2); *nnodes = nv + number of edges. */
int ffgpu_number_p2_2d(int nv, int nt, const int32_t *elems, int32_t *nodes, int *nnodes);
/* The Gibbs renumbering alone (gibbsa_, src/femlib/gibbs.cpp:209-433) on a graph in 1-based
 * CSR form: vertex i (1..n) has the neighbours vois[ptvois[i-1]-1 .. ptvois[i]-2], 1-based,
 * ptvois[0] = 1 (the lists are sorted in place by degree).  r[i-1] = new 1-based number of
 * vertex i; *pfold, *pfnew = the profiles before and after (the new numbering is what FreeFEM
 * applies when *pfnew <= *pfold). */
int ffgpu_gibbs_renumber(int64_t n, const int64_t *ptvois, int64_t *vois, int64_t *r, int64_t *pfold,
                         int64_t *pfnew);

/* ------------------------------------------------------------------ assembly
 * matrix A = a(Vh,Vh, ...): replaces OpMatrixtoBilinearForm::Op::operator() /
 * AssembleBilinearForm / HashMatrix::operator+= / AssembleBC+SetBC
 * (src/fflib/problem.hpp:1611-1660, src/fflib/problem.cpp:803,1117,9881-10034,
 *  src/femlib/HashMatrix.cpp:1195-1238,1295-1332).
 * Pattern = every (i,j) two DOFs of one element couple, zeros kept, in FreeFEM's
 * row-then-column order; values summed in element order.  If rhs != NULL the linear form
 * of the same varf (a(0,Vh), problem.hpp:1351-1388) is assembled into it in the same pass. */
int ffgpu_matrix_assemble(ffgpu_space *space, const ffgpu_varf *varf, const ffgpu_bc *bc,
                          double *rhs, ffgpu_matrix **out);
/* re-run the numeric phase on an existing pattern (new coefficients, same mesh/space) */
int ffgpu_matrix_reassemble(ffgpu_matrix *A, const ffgpu_varf *varf, const ffgpu_bc *bc,
                            double *rhs);
/* real[int] b = a(0,Vh): replaces OpArraytoLinearForm / AssembleLinearForm / Element_rhs
 * (src/fflib/problem.hpp:1351-1388, src/fflib/problem.cpp:7839-7911,10555). */
int ffgpu_rhs_assemble(ffgpu_space *space, const ffgpu_varf *varf, const ffgpu_bc *bc,
                       double *rhs);
/* FreeFEM's sparse-matrix text forms, host only (no device, no context):
 * ffgpu_matrix_text_read replaces HashMatrix(istream&) (HashMatrix.cpp:137-214, `f >> A`):
 * reads the "(COO)" form FreeFEM prints by default and the "(Morse)" CSR form; entries are
 * assigned (a repeated (i, j) keeps its last value); returns the sorted CSR.  Call with
 * rowptr == NULL for n, m, nnz, half, then with rowptr[n+1], col[nnz], val[nnz].
 * ffgpu_matrix_text_write replaces operator<<(ostream&, HashMatrix) (HashMatrix.hpp:484-520,
 * `f << A` and solve(..., save=)) for a sorted CSR: FFGPU_TEXT_COO (0-based, as FreeFEM prints
 * a sorted matrix) or FFGPU_TEXT_MORSE (1-based), values at 20 significant digits. */
#define FFGPU_TEXT_COO 0
#define FFGPU_TEXT_MORSE 1
int ffgpu_matrix_text_read(const char *path, int *n, int *m, int64_t *nnz, int *half, int32_t *rowptr,
                           int32_t *col, double *val);
int ffgpu_matrix_text_write(const char *path, int format, int n, int m, int half, const int32_t *rowptr,
                            const int32_t *col, const double *val);
/* matrix from a sorted CSR (the addsolver path: HashMatrix::CSR, HashMatrix.cpp:859-867) */
int ffgpu_matrix_from_csr(ffgpu_ctx *ctx, int n, int64_t nnz, const int32_t *rowptr,
                          const int32_t *col, const double *val, ffgpu_matrix **out);
int ffgpu_matrix_destroy(ffgpu_matrix *A);
int ffgpu_matrix_info(const ffgpu_matrix *A, int *n, int64_t *nnz, int *block_size);
/* SpMV layout the solver's tuner chose for this matrix: mode 0 (FP64 CG), 1 (double-float CG)
 * or 2 (FP32 inner solve of ffgpu_solve_ir).  Returns 64 + a + 2u for the SELL-32 copy, with
 * a = 0 for contiguous per-warp chunk ranges or 1 for a rotated chunk stride, and the row loop
 * u = 0 unrolled, 1 unrolled deeper, 2 batched, 3 batched deeper (2 and 3: FP64 only); T in
 * {1,..,32} for block CSR with T lanes per block row; 0 before the first solve.  mode 3: 1 when the SELL copy stores 16-bit column differences;
 * mode 4: block entries the SELL copy stores, padding included (32 per slot; -1 past INT32_MAX).
 * mode 5: 1 when the last FP64 CG solve ran its whole iteration loop in one thread-block
 * cluster (opt-in with FFGPU_CLUSTER_CG=1: scalar systems of up to 8 x 9216 rows; a fixed
 * layout selects the regular path).
 * No FreeFEM counterpart. */
int ffgpu_matrix_spmv_layout(const ffgpu_matrix *A, int mode);
/* Average device time in ms of `nrep` back-to-back launches of the solver's SpMV kernel (K_a,
 * with its fused dot product) for mode 0 (FP64 CG), 1 (double-float CG) or 2 (FP32 inner solve
 * of ffgpu_solve_ir), in the layout the tuner chose, timed with CUDA events on the library
 * stream.  The matrix must have been solved in that mode first.  Reads the last solution, writes
 * only scratch vectors.  A measurement helper; no FreeFEM counterpart. */
int ffgpu_matrix_time_spmv(ffgpu_matrix *A, int mode, int nrep, float *ms);
/* [I,J,C] = A in sorted CSR form (HashMatrix::CSR / Sortij, HashMatrix.cpp:671-682,870-876) */
int ffgpu_matrix_csr(const ffgpu_matrix *A, int32_t *rowptr, int32_t *col, double *val);

/* y = A x (trans = 0) or A' x (trans = 1): HashMatrix::addMatMul (HashMatrix.cpp:1087-1154) */
int ffgpu_matrix_mult(ffgpu_matrix *A, const double *x, double *y, int trans);

/* ------------------------------------------------------------------ solvers
 * u[] = A^-1*b / A'^-1*b with solver=CG: replaces SolverCG::dosolver + HMatVirtPrecon +
 * ConjugueGradient (src/femlib/VirtualSolverCG.hpp:14-192, src/femlib/CG.cpp:196-265).
 * x holds the initial guess (RNM.hpp:568-571) and receives the solution; nrhs contiguous
 * right-hand sides of length n.  Returns FFGPU_ENOCONV if any RHS did not converge. */
int ffgpu_solve_cg(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                   const ffgpu_solver_params *prm, ffgpu_solver_stats *stats);
/* solver=GMRES: replaces SolverGMRES::dosolver + fgmres (VirtualSolverCG.hpp:195-257,
 * CG.cpp:348-517): right Jacobi preconditioning, modified Gram-Schmidt, Givens rotations. */
int ffgpu_solve_gmres(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                      const ffgpu_solver_params *prm, ffgpu_solver_stats *stats);

/* ------------------------------------------------------------------ direct solver
 * Sparse direct solves on the device, the direct solvers behind addsolver in the roles FreeFEM's
 * CHOLMOD / UMFPACK / MUMPS play (VirtualSolverSparseSuite.hpp:305, SparseLinearSolver.hpp:116,
 * plugin/seq/MUMPS_seq.cpp:260-300), driven as FreeFEM drives them (VirtualSolver::factorize:
 * symbolic once per pattern, numeric once per numeric state, then the solves,
 * VirtualSolver.hpp:226-239).
 * ffgpu_direct_method: FFGPU_DIRECT_AUTO (default: Cholesky when the matrix is symmetric,
 * else QR), FFGPU_DIRECT_CHOLESKY (symmetric positive definite: tgv > 0 and tgv = -2 rows keep
 * it so; FFGPU_EINVAL otherwise) or FFGPU_DIRECT_QR (any nonsingular matrix: rows scaled by
 * their largest entry, then sparse QR); a change drops the current factorisation.
 * ffgpu_direct_factor: fill-reducing ordering (nested dissection; approximate minimum degree as
 * the fallback), symbolic analysis, numeric factorisation (cuSOLVER's sparse Cholesky or QR);
 * a reassembly keeps the ordering and analysis and refactors at the next solve.  FFGPU_EINVAL
 * for a matrix the method cannot factor (not positive definite, singular), or when cuSOLVER is
 * not installed.
 * ffgpu_solve_direct: x = A^-1 b for nrhs right-hand sides, factoring first if needed.
 * ffgpu_solve_direct_trans: x = A^-1 b (trans 0) or A'^-1 b (trans 1), the direct side of
 * VirtualSolver::solve(x, b, N, trans) (VirtualSolver.hpp:235-239; UMFPACK solves A' x = b
 * with the factors of A, UMFPACK_At in VirtualSolverSparseSuite.hpp:169).  A symmetric matrix answers A' from
 * its Cholesky factors; a nonsymmetric one gets a second QR, of A' (same pattern, values read
 * transposed), at its first transpose solve, refactored with A after a reassembly.  FFGPU_EINVAL
 * when the pattern is not structurally symmetric. */
#define FFGPU_DIRECT_AUTO 0
#define FFGPU_DIRECT_CHOLESKY 1
#define FFGPU_DIRECT_QR 2
int ffgpu_direct_method(ffgpu_matrix *A, int method);
int ffgpu_direct_factor(ffgpu_matrix *A);
int ffgpu_solve_direct(ffgpu_matrix *A, const double *b, double *x, int nrhs, ffgpu_solver_stats *stats);
int ffgpu_solve_direct_trans(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                             ffgpu_solver_stats *stats);

/* ------------------------------------------------------------------ mixed precision
 * FP32 inner Jacobi-PCG (FP32 values, vectors, SpMV and dot products) inside an FP64
 * iterative-refinement loop (outer residual b - A x in FP64 on the FP64 matrix, FP64 update).
 * By default each refinement step replaces the inner iterated residual by the true one and
 * continues the conjugate-gradient recurrence (reliable updates); restart_inner = 1 starts a
 * fresh inner PCG instead.
 * Stops on FreeFEM's CG criterion applied to the true residual, (r, C r) < eps^2 (r0, C r0)
 * (CG.cpp:226,247), so it answers the same u[] = A^-1*b as ffgpu_solve_cg; no FreeFEM
 * counterpart of its own (FreeFEM's solvers are FP64). */
typedef struct {
    double eps;         /* outer tolerance, as ffgpu_solver_params.eps                       */
    double eps_inner;   /* residual drop of each FP32 inner segment (<=0: 1e-2; 1e-5 when
                           restart_inner)                                                     */
    int itmax_inner;    /* inner iteration cap per segment (<=0: n)                           */
    int max_outer;      /* refinement steps cap (<=0: 30)                                     */
    double tgv;
    int unroll;
    int restart_inner;  /* 0: replace the residual and keep the search direction (reliable
                           updates); 1: restart the inner PCG at every refinement step        */
} ffgpu_ir_params;

/* FP32 copy of the values used by the inner solves (built on first use, freed on reassembly) */
int ffgpu_matrix_to_f32(ffgpu_matrix *A);
int ffgpu_solve_ir(ffgpu_matrix *A, const double *b, double *x, const ffgpu_ir_params *prm,
                   ffgpu_solver_stats *stats);

/* ------------------------------------------------------------------ adjoint
 * Per-element sensitivities of A(kappa) u = b(f) for the P1 diffusion varf assembled by
 * ffgpu_matrix_assemble, given the state u and the adjoint lambda (A' lambda = dL/du, from
 * ffgpu_solve_cg with trans = 1, FreeFEM's A'^-1 path lgmat.cpp:3219 / HashMatrix.cpp:1094):
 *   grad_kappa[e] = -c_stiff |K| sum_ij lambda_i (grad phi_i . grad phi_j) u_j  (tgv diagonals excluded)
 *   grad_f[e]     =  sum_{i not tgv} lambda_i int_K phi_i
 * FreeFEM has no adjoint of its own; its scripts form the same gradient with a P0 test-function
 * varf int(-(grad lambda . grad u) w).  Either output may be NULL. */
int ffgpu_diffusion_sensitivity(ffgpu_matrix *A, const double *u, const double *lambda, double c_stiff,
                                double *grad_kappa, double *grad_f);

/* ------------------------------------------------------------------ batched problems
 * Many independent 2D P1 diffusion problems (int(kappa grad u.grad v) + int(f v) + on(...,u=0))
 * assembled in one pass and solved in one persistent, graph-captured launch with FP32 inner
 * Jacobi-PCG and FP64 refinement.  Each problem is what FreeFEM would assemble and solve alone
 * (pattern, values, stopping rule of SolverCG applied to the true residual); FreeFEM has no
 * batched path, it runs one script per problem.
 * create: nprob meshes, nv[p] vertices and nt[p] triangles each; coords (sum nv) x 2, elems
 *         (sum nt) x 3 with per-problem vertex numbers (host or device arrays).  A vertex
 *         number outside [0, nv[p]) gives FFGPU_EINVAL naming the first such problem.
 * assemble: kappa (sum nt) P0 values, constant source f, onbc (sum nv) Dirichlet mask, tgv.
 * solve: x (sum nv) receives all solutions; iterations[p] (may be NULL) the inner iterations.
 *        prm->eps is each problem's outer tolerance.  The first solve autotunes the CTA size
 *        and lanes per SpMV row by timing the candidates on the batch. */
typedef struct ffgpu_batch ffgpu_batch;
int ffgpu_batch_create(ffgpu_ctx *ctx, int nprob, const int32_t *nv, const int32_t *nt,
                       const double *coords, const int32_t *elems, ffgpu_batch **out);
int ffgpu_batch_assemble(ffgpu_batch *B, const double *kappa, double f, const uint8_t *onbc,
                         double tgv);
int ffgpu_batch_solve(ffgpu_batch *B, double *x, const ffgpu_ir_params *prm, int32_t *iterations,
                      ffgpu_solver_stats *stats);
/* right-hand sides of all problems (sum nv) as assembled */
int ffgpu_batch_rhs(const ffgpu_batch *B, double *b);
/* the block-diagonal matrix of the batch (owned by the batch) */
ffgpu_matrix *ffgpu_batch_matrix(const ffgpu_batch *B);
/* the autotuned launch shape: threads per CTA, lanes per SpMV row, its batch time */
int ffgpu_batch_info(const ffgpu_batch *B, int *cta_threads, int *lanes_per_row, float *tuned_ms);
int ffgpu_batch_destroy(ffgpu_batch *B);

/* ------------------------------------------------------------------ allocation-free CG
 * Jacobi-PCG on a caller's CSR matrix that allocates no memory: for callers that cannot
 * allocate device memory while they run (an application that hands the GPU's memory to its
 * own pool at start-up and calls the solver from its time loop).  No counterpart in FreeFEM;
 * the algorithm is ffgpu_solve_cg's.  Every array (rowptr, col, val, b, x) must be in device
 * memory; x holds the initial guess and receives the solution.  n <= 524288: the work vectors
 * live in a fixed ~17 MB device array that every GPU loading the library keeps until exit.
 * The first call on a device (made with that device current) looks the array up with
 * cudaGetSymbolAddress.  Every call synchronises `stream` (convergence is polled from the host
 * every 32 iterations), so it cannot be called while that stream is being captured into a
 * CUDA graph.  All calls share the array: calls that overlap on the GPU race, so serialise
 * them.  stream: cudaStream_t as void* (NULL = default stream).  iterations and
 * gcg_out[2] = {final gCg, eps2} may be NULL.  Arrays must be device memory of the current
 * device (or managed memory).
 * Returns FFGPU_EINVAL for n above the limit or non-device arrays, FFGPU_ENOCONV at itmax. */
int ffgpu_solve_cg_csr_noalloc(int n, int64_t nnz, const int32_t *rowptr, const int32_t *col,
                               const double *val, const double *b, double *x, double eps, int itmax,
                               double tgv, void *stream, int *iterations, double *gcg_out);

#ifdef __cplusplus
}
#endif
#endif /* FFGPU_H */
