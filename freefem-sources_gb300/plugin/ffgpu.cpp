// ffgpu.cpp -- FreeFEM plugin: `load "ffgpu"` registers the GB300 solvers.
//
// Build with FreeFEM's own plugin compiler (it adds ff++.hpp's include path and flags):
//     ff-c++ -auto ffgpu.cpp -I<repo>/include <repo>/freefem-sources_gb300/ffgpu/lib/libffgpu.so
// Scripts then select the device solvers by name, exactly like FreeFEM's own:
//     load "ffgpu"
//     matrix A = a(Vh, Vh, solver=GPUCG, eps=1e-10);      // or set(A, solver=GPUCG)
//     u[] = A^-1 * b;   u[] = A'^-1 * b;
//
// Solvers registered (addsolver, src/femlib/SparseLinearSolver.hpp:96-102):
//   GPUCG       Jacobi-PCG on the GPU      -- same algorithm and stopping rule as SolverCG
//                                             (src/femlib/VirtualSolverCG.hpp:113-192)
//   GPUGMRES    right-preconditioned FGMRES -- as SolverGMRES (VirtualSolverCG.hpp:195-257)
//   GPUCGMIXED  FP32 inner PCG + FP64 refinement, same stopping rule on the true residual
//   GPUCHOLESKY sparse Cholesky on the device, factored once per numeric state (the role of
//               FreeFEM's CHOLMOD / MUMPS plugins); symmetric positive definite matrices
//   GPUSPARSESOLVER  the direct solver of any nonsingular matrix (the role of UMFPACK, FreeFEM's
//               `sparsesolver`): Cholesky when the matrix is symmetric, else sparse QR
// The matrix FreeFEM assembled is uploaded once per numeric state (fac_numeric, in sorted CSR
// via HashMatrix::CSR, HashMatrix.cpp:859-867) and stays on the device with the solver object,
// which the matrix owns (VirtualMatrix.hpp:71-94).  Errors become ExecError / ffassert as in
// FreeFEM's own solvers; there is no CPU fallback.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <set>
#include <string>
#include <vector>

#include "ff++.hpp"
#include "ffgpu.h"

// label sets of an on(...) condition and of a domain of integration (defined in FreeFEM,
// lgfem.cpp:7792, 7809)
namespace Fem2D {
void Expandsetoflab(Stack stack, const BC_set &bc, set<long> &setoflab);
void Expandsetoflab(Stack stack, const CDomainOfIntegration &di, set<int> &setoflab, bool &all);
}

namespace {

ffgpu_ctx *g_ctx = nullptr;
// ffgpustrict (script variable; or the environment variable FFGPU_STRICT=1): a form the device
// does not assemble stops the script with ExecError instead of going to FreeFEM's own assembly
long g_strict = 0;

bool strict() {
    static const bool env = getenv("FFGPU_STRICT") && getenv("FFGPU_STRICT")[0] == '1';
    return env || g_strict != 0;
}

// A form the device does not take: reported at verbosity > 0, an error under ffgpustrict.
void not_on_device(const char *what, const std::string &why) {
    if (strict()) ExecError((std::string("ffgpu (ffgpustrict): ") + what + " not assembled on the device: " + why).c_str());
    if (verbosity > 0) std::cout << "  ffgpu: " << what << " assembled by FreeFEM on the CPU (" << why << ")" << std::endl;
}

ffgpu_ctx *context() {
    if (!g_ctx) {
        int r = ffgpu_ctx_create(0, &g_ctx);
        if (r != FFGPU_OK) {
            g_ctx = nullptr;
            ExecError((std::string("ffgpu: no usable CUDA device: ") + ffgpu_last_error()).c_str());
        }
    }
    return g_ctx;
}

enum Kind { kCG = 0, kGMRES = 1, kMixed = 2, kCholesky = 3, kSparse = 4 };

// FreeFEM's matrix in full sorted CSR: A.CSR (HashMatrix.cpp:859-867), the other triangle added
// when FreeFEM stores half of a symmetric matrix (HashMatrix::half)
static void full_csr(HashMatrix<int, double> &A, std::vector<int32_t> &rp, std::vector<int32_t> &col,
                     std::vector<double> &val) {
    int *IA = nullptr, *JA = nullptr;
    double *AA = nullptr;
    A.CSR(IA, JA, AA);
    const int n = A.n;
    if (!A.half) {
        rp.assign(IA, IA + n + 1);
        col.assign(JA, JA + IA[n]);
        val.assign(AA, AA + IA[n]);
        return;
    }
    std::vector<std::vector<std::pair<int, double> > > rows(n);
    for (int i = 0; i < n; ++i)
        for (int k = IA[i]; k < IA[i + 1]; ++k) {
            rows[i].push_back(std::make_pair(JA[k], AA[k]));
            if (JA[k] != i) rows[JA[k]].push_back(std::make_pair(i, AA[k]));
        }
    rp.assign(n + 1, 0);
    col.clear();
    val.clear();
    for (int i = 0; i < n; ++i) {
        std::sort(rows[i].begin(), rows[i].end());
        for (size_t k = 0; k < rows[i].size(); ++k) {
            col.push_back(rows[i][k].first);
            val.push_back(rows[i][k].second);
        }
        rp[i + 1] = (int32_t)col.size();
    }
}

template <int KIND>
class SolverGpu : public VirtualSolver<int, double> {
   public:
    // 1 unsym, 2 herm, 4 sym, 8 pos, 16 nopos, 32 seq (as SolverCG / SolverGMRES): full storage
    static const int orTypeSol;
    typedef HashMatrix<int, double> HMat;
    HMat &A;
    ffgpu_matrix *M;
    bool adopted;   // M is the device matrix of `matrix A = a(Vh,Vh)`, equal to A's values
    double eps, tgv;
    long itmax, verb, restart;
    double *veps;
    long *getnbiter;
    long cs, cn;

    SolverGpu(HMat &AA, const Data_Sparse_Solver &ds, Stack)
        : A(AA), M(nullptr), adopted(false), eps(ds.epsilon), tgv(ds.tgv), itmax(ds.itmax), verb(ds.verb),
          restart(ds.NbSpace), veps(ds.veps), getnbiter(ds.getnbiter), cs(0), cn(0) {
        if (ds.precon) ExecError("ffgpu: a script precon= function cannot run on the GPU");
        ffassert(A.n == A.m);
    }
    ~SolverGpu() {
        if (M) ffgpu_matrix_destroy(M);
    }
    // The device assembly hands over its matrix: the first factorisation uses it instead of
    // uploading FreeFEM's copy, unless the script changed A in between (HashMatrix's
    // re_do_numerics / re_do_symbolic flags, HashMatrix.hpp:278-279, read in UpdateState).
    void adopt(ffgpu_matrix *dm) {
        if (M) ffgpu_matrix_destroy(M);
        M = dm;
        adopted = true;
    }
    void UpdateState() {
        const bool num = A.GetReDoNumerics(), sym = A.GetReDoSymbolic();
        if (num) cn++;
        if (sym) cs++;
        if (num || sym) adopted = false;
        this->ChangeCodeState(A.n, cs, cn);
    }
    void fac_numeric() {
        if (M && adopted) {
            adopted = false;   // later factorisations follow FreeFEM's matrix
            if (verb > 1) std::cout << "  ffgpu: solver uses the device-assembled matrix" << std::endl;
            factor();
            return;
        }
        std::vector<int32_t> rp, col;
        std::vector<double> val;
        full_csr(A, rp, col, val);
        if (M) {
            ffgpu_matrix_destroy(M);
            M = nullptr;
        }
        int r = ffgpu_matrix_from_csr(context(), A.n, (int64_t)col.size(), rp.data(), col.data(), val.data(), &M);
        if (r != FFGPU_OK) ExecError((std::string("ffgpu upload: ") + ffgpu_last_error()).c_str());
        factor();
    }
    // the direct solver factors here, once per numeric state (VirtualSolver::factorize)
    void factor() {
        if (KIND != kCholesky && KIND != kSparse) return;
        int r = ffgpu_direct_method(M, KIND == kCholesky ? FFGPU_DIRECT_CHOLESKY : FFGPU_DIRECT_AUTO);
        if (r == FFGPU_OK) r = ffgpu_direct_factor(M);
        if (r != FFGPU_OK) ExecError((std::string("ffgpu direct solver: ") + ffgpu_last_error()).c_str());
    }
    void dosolver(double *x, double *b, int N, int trans) {
        ffgpu_solver_stats st;
        int r;
        if (KIND == kMixed) {
            ffgpu_ir_params p = {eps, 0.0, 0, 30, tgv, 8, 0};
            r = FFGPU_OK;
            for (int k = 0; k < N && r == FFGPU_OK; ++k)
                r = ffgpu_solve_ir(M, b + (size_t)k * A.n, x + (size_t)k * A.n, &p, &st);
        } else if (KIND == kCholesky || KIND == kSparse) {
            // Cholesky: A' = A; a nonsymmetric matrix solves A' x = b with a QR of A'
            r = ffgpu_solve_direct_trans(M, b, x, N, trans, &st);
        } else {
            ffgpu_solver_params p = {eps, (int)itmax, (int)restart, tgv, (int)verb, 8};
            r = KIND == kCG ? ffgpu_solve_cg(M, b, x, N, trans, &p, &st)
                            : ffgpu_solve_gmres(M, b, x, N, trans, &p, &st);
        }
        if (r == FFGPU_ENOCONV) {
            std::cerr << "Error: ffgpu Krylov solver did not converge: " << ffgpu_last_error() << std::endl;
            ffassert(0);
        }
        if (r != FFGPU_OK) ExecError((std::string("ffgpu solve: ") + ffgpu_last_error()).c_str());
        if (getnbiter) *getnbiter = st.iterations;
        if (veps) *veps = KIND == kGMRES ? eps : std::sqrt(st.eps2);
        if (verb > 1) std::cout << "  ffgpu: " << st.iterations << " iterations, " << st.elapsed_ms << " ms" << std::endl;
    }
};

template <> const int SolverGpu<kCG>::orTypeSol = 1 | 2 | 4 | 8 | 32;
template <> const int SolverGpu<kGMRES>::orTypeSol = 1 | 2 | 4 | 8 | 16 | 32;
template <> const int SolverGpu<kMixed>::orTypeSol = 1 | 2 | 4 | 8 | 32;
template <> const int SolverGpu<kCholesky>::orTypeSol = 1 | 2 | 4 | 8 | 32;
template <> const int SolverGpu<kSparse>::orTypeSol = 1 | 2 | 4 | 8 | 16 | 32;

// ------------------------------------------------------------------ device assembly
// `matrix A = a(Vh, Vh, ...)` is routed here (an OpMatrixtoBilinearForm with a higher
// overload preference, problem.hpp:1611, AFunction2.cpp:87-100).  A form the device assembles
// is recognised from its terms; anything else -- other elements, coefficients that are not
// piecewise constant, quadratures that are not exact for the form, symmetric storage, other
// terms -- is assembled by FreeFEM's own operator, unchanged.
//   scalar P1 / P2 (2D, 3D):  int(Th)(k*(grad u . grad v) [+ m*u*v]) + on(labels, u = ...)
//     with k piecewise constant (a P0 function, a constant, any expression constant per
//     element) -- for P1 any expression, as its quadrature-rule average per element -- and m
//     constant;
//   3D [P2,P2,P2]:            int3d(Th)(lambda*div(u)*div(v) + 2*mu*(eps(u):eps(v)))
//     + on(labels, ...) with constant lambda, mu (any way of writing it whose terms add up
//     to the isotropic tensor);
//   both with boundary terms int1d(Th, labels)(c*u*v) in 2D / int2d(Th, labels)(c*u*v) on a
//     3D mesh (c*(u1*v1+u2*v2+u3*v3) for [P2,P2,P2]), c constant on every boundary element,
//     and, in the linear form, int1d / int2d(Th, labels)(g*v) with g constant on every
//     boundary element (boundary quadrature exact for the term).
// The device matrix is built by ffgpu_matrix_assemble (pattern, values and tgv rows) and
// handed to FreeFEM as its HashMatrix (sorted CSR, HashMatrix::set).

template <class MMesh> struct Dim;
template <> struct Dim<Mesh> { static const int d = 2; typedef R2 Rd; };
template <> struct Dim<Mesh3> { static const int d = 3; typedef R3 Rd; };

// One boundary term of the device's kind: labels (empty: the whole boundary) and, per boundary
// element, the coefficient of u.v (Robin) or of v_c (source) -- constant on every boundary element.
struct BoundaryRec {
    std::vector<int32_t> labels;
    std::vector<double> robin;   // nbe, empty: none
    std::vector<double> g;       // nbe * ncomp, empty: none
};

// the volume rule of `di`: size, point q (reference coordinates) and its weight
static int rule_size(Stack s, const CDomainOfIntegration &di, const Mesh *) { return di.FIT(s).n; }
static int rule_size(Stack s, const CDomainOfIntegration &di, const Mesh3 *) { return di.FIV(s).n; }
static void rule_point(Stack s, const CDomainOfIntegration &di, int q, R2 &P, double &w) {
    const QuadratureFormular &FI = di.FIT(s);
    P = R2(FI[q].x, FI[q].y);
    w = FI[q].a;
}
static void rule_point(Stack s, const CDomainOfIntegration &di, int q, R3 &P, double &w) {
    const GQuadratureFormular<R3> &FI = di.FIV(s);
    P = R3(FI[q].x, FI[q].y, FI[q].z);
    w = FI[q].a;
}
static void barycentric(const R2 &P, double *l) { l[0] = 1. - P.x - P.y; l[1] = P.x; l[2] = P.y; }
static void barycentric(const R3 &P, double *l) { l[0] = 1. - P.x - P.y - P.z; l[1] = P.x; l[2] = P.y; l[3] = P.z; }

struct Recognised {
    int fe = 0, form = FFGPU_FORM_DIFFUSION;
    std::vector<double> kappa;
    double c_mass = 0, lam = 0, mu = 0, tgv = 1e30;
    // a mass coefficient that depends on the point: its values at the points of the rule
    int nqp = 0;
    std::vector<double> lam_q, w_q;   // nqp x (dim+1) barycentric coordinates, weights
    std::vector<double> mqp;          // nt x nqp
    std::vector<double> kqp[3];       // per derivative d: nt x nqp (grad u . grad v at the points)
    int comp_mask = -1;   // components constrained by on(...) (-1: no on)
    std::vector<int32_t> labels;
    std::vector<BoundaryRec> bterms;   // Robin terms, in varf order
    std::string why;
};

// a term's coefficient at the points of its rule, per element, added into `out` (Element_Op
// takes it so, problem.cpp:6063-6160, 6337-6437); every such term must use one rule
template <class MMesh, class FES>
static bool coef_at_points(Stack stack, const C_F0 &coef, const MMesh &Th, const FES &Uh,
                           const CDomainOfIntegration &di, Recognised &r, std::vector<double> &out) {
    typedef typename Dim<MMesh>::Rd Rd;
    const int d = Dim<MMesh>::d, nt = Th.nt;
    const int nq = rule_size(stack, di, &Th);
    std::vector<Rd> P(nq);
    std::vector<double> lam((size_t)nq * (d + 1)), w(nq);
    for (int q = 0; q < nq; ++q) {
        rule_point(stack, di, q, P[q], w[q]);
        barycentric(P[q], &lam[(size_t)q * (d + 1)]);
    }
    if (r.nqp == 0) {
        if (nq < 1 || nq > 64) { r.why = "quadrature rule size"; return false; }
        r.nqp = nq;
        r.lam_q = lam;
        r.w_q = w;
    } else if (lam != r.lam_q || w != r.w_q) {
        r.why = "terms at quadrature points with different rules";
        return false;
    }
    if (out.empty()) out.assign((size_t)nt * nq, 0.0);
    for (int k = 0; k < nt; ++k) {
        typename FES::FElement FK = Uh[k];
        for (int q = 0; q < nq; ++q) {
            MeshPointStack(stack)->set(Th[k](P[q]), P[q], FK);
            out[(size_t)k * nq + q] += GetAny<double>(coef.eval(stack));
        }
    }
    return true;
}

// element type of a space: FFGPU_FE_* or 0
static int fe_kind(const FESpace &Uh) {
    if (Uh.N != 1) return 0;
    if (Uh.TFE[0] == &P1Lagrange) return FFGPU_FE_P1;
    if (Uh.TFE[0] == &P2Lagrange) return FFGPU_FE_P2;
    return 0;
}
static int fe_kind(const FESpace3 &Uh) {
    if (Uh.TFE[0] == &DataFE<Mesh3>::P1) return FFGPU_FE_P1;
    if (Uh.TFE[0] == &DataFE<Mesh3>::P2) return FFGPU_FE_P2;
    const GTypeOfFESum<Mesh3> *s = dynamic_cast<const GTypeOfFESum<Mesh3> *>(Uh.TFE[0]);
    if (s && s->k == 3 && s->teb[0] == &DataFE<Mesh3>::P2 && s->teb[1] == &DataFE<Mesh3>::P2 &&
        s->teb[2] == &DataFE<Mesh3>::P2)
        return FFGPU_FE_P2VEC3;
    return 0;
}

// position of a FreeFEM operator code among (id, dx, dy[, dz]), -1 for anything else
static int op_index(int op, int d) {
    op %= last_operatortype;
    if (op == op_id) return 0;
    if (op == op_dx) return 1;
    if (op == op_dy) return 2;
    if (op == op_dz && d == 3) return 3;
    return -1;
}

// two interior reference points of a simplex (barycentre and an off-centre point)
static void ref_points(R2 &a, R2 &b) { a = R2(1. / 3., 1. / 3.); b = R2(0.2, 0.3); }
static void ref_points(R3 &a, R3 &b) { a = R3(0.25, 0.25, 0.25); b = R3(0.1, 0.2, 0.3); }

// the element average of a coefficient by the domain's own quadrature rule,
// sum_q a_q c(x_q) (weights relative to the element measure, problem.cpp:6096-6100): for a P1
// stiffness term, whose gradients are constant, int_K c grad(phi_i).grad(phi_j) as FreeFEM
// forms it is |K| (sum_q a_q c_q) grad(phi_i).grad(phi_j)
template <class FElement>
static double rule_average(Stack stack, const C_F0 &coef, const Mesh::Element &K, FElement &FK,
                           const CDomainOfIntegration &di) {
    const QuadratureFormular &FI = di.FIT(stack);
    double s = 0;
    for (int q = 0; q < FI.n; ++q) {
        const R2 P(FI[q].x, FI[q].y);
        MeshPointStack(stack)->set(K(P), P, FK);
        s += FI[q].a * GetAny<double>(coef.eval(stack));
    }
    return s;
}
template <class FElement>
static double rule_average(Stack stack, const C_F0 &coef, const Mesh3::Element &K, FElement &FK,
                           const CDomainOfIntegration &di) {
    const GQuadratureFormular<R3> &FI = di.FIV(stack);
    double s = 0;
    for (int q = 0; q < FI.n; ++q) {
        const R3 P(FI[q].x, FI[q].y, FI[q].z);
        MeshPointStack(stack)->set(K(P), P, FK);
        s += FI[q].a * GetAny<double>(coef.eval(stack));
    }
    return s;
}

// quadrature exactness of a domain of integration (volume, boundary)
static int exactness(Stack s, const CDomainOfIntegration &di, const Mesh *) { return di.FIT(s).exact; }
static int exactness(Stack s, const CDomainOfIntegration &di, const Mesh3 *) { return di.FIV(s).exact; }
static int bexactness(Stack s, const CDomainOfIntegration &di, const Mesh *) { return di.FIE(s).exact; }
static int bexactness(Stack s, const CDomainOfIntegration &di, const Mesh3 *) { return di.FIT(s).exact; }

// int2d(Th) in 2D / int3d(Th) in 3D over the whole mesh; int1d(Th, labels) in 2D / int2d(Th,
// labels) on a 3D mesh: its boundary (CDomainOfIntegration kinds, problem.hpp:313)
static bool volume_domain(const CDomainOfIntegration &di, int d) {
    return di.kind == (d == 2 ? CDomainOfIntegration::int2d : CDomainOfIntegration::int3d) && di.d == d &&
           di.dHat == d && di.what.empty() && !di.islevelset() && !di.withmap();
}
static bool boundary_domain(const CDomainOfIntegration &di, int d) {
    return di.kind == (d == 2 ? CDomainOfIntegration::int1d : CDomainOfIntegration::int2d) && di.d == d &&
           di.dHat == d && !di.islevelset() && !di.withmap();
}

// boundary elements in FreeFEM's order, their labels, adjacent element and local edge/face
static int nb_boundary(const Mesh &Th) { return Th.neb; }
static int nb_boundary(const Mesh3 &Th) { return Th.nbe; }
static int boundary_label(const Mesh &Th, int e) { return Th.bedges[e].lab; }
static int boundary_label(const Mesh3 &Th, int e) { return Th.be(e).lab; }
// two points of edge/face ie in reference coordinates and the outward unit normal, as
// Element_rhs places its quadrature points there (problem.cpp:8645-8652, 8543-8548)
static void boundary_points(const Mesh::Element &T, int ie, R2 *P, R2 &N) {
    const R2 PA(TriangleHat[VerticesOfTriangularEdge[ie][0]]), PB(TriangleHat[VerticesOfTriangularEdge[ie][1]]);
    P[0] = PA * 0.5 + PB * 0.5;
    P[1] = PA * 0.3 + PB * 0.7;
    const R2 E = T.Edge(ie);
    N = R2(E.y, -E.x) / sqrt((E, E));
}
static void boundary_points(const Mesh3::Element &T, int ie, R3 *P, R3 &N) {
    P[0] = T.PBord(ie, R2(1. / 3., 1. / 3.));
    P[1] = T.PBord(ie, R2(0.2, 0.3));
    N = T.N(ie);
    N /= N.norme();
}

// Values of `coef` on the boundary elements of `di` (others 0); false when it is not constant
// on one of them.
template <class MMesh, class FES>
static bool boundary_values(Stack stack, const MMesh &Th, const FES &Uh, const std::set<int> &labs, bool all,
                            const C_F0 &coef, std::vector<double> &out, int stride, int comp) {
    typedef typename Dim<MMesh>::Rd Rd;
    const bool constant = coef.LeftValue()->MeshIndependent();
    const int nbe = nb_boundary(Th);
    for (int e = 0; e < nbe; ++e) {
        const int lab = boundary_label(Th, e);
        if (!all && !labs.count(lab)) continue;
        int ie;
        const int k = Th.BoundaryElement(e, ie);
        typename FES::FElement FK = Uh[k];
        Rd P[2], N;
        boundary_points(Th[k], ie, P, N);
        MeshPointStack(stack)->set(Th[k](P[0]), P[0], FK, lab, N, ie);
        const double ca = GetAny<double>(coef.eval(stack));
        if (!constant) {
            MeshPointStack(stack)->set(Th[k](P[1]), P[1], FK, lab, N, ie);
            const double cb = GetAny<double>(coef.eval(stack));
            if (!(std::fabs(ca - cb) <= 1e-14 * std::max(std::fabs(ca), std::fabs(cb)))) return false;
        }
        out[(size_t)e * stride + comp] += ca;
    }
    return true;
}

// Label set and quadrature check of a boundary domain, shared by the two readers below.
template <class MMesh>
static bool boundary_domain_labels(Stack stack, const MMesh &Th, const CDomainOfIntegration &di, int degree,
                                   std::set<int> &labs, bool &all, BoundaryRec &r, std::string &why) {
    if (GetAny<const MMesh *>((*di.Th)(stack)) != &Th) { why = "integration mesh"; return false; }
    if (bexactness(stack, di, &Th) < degree) { why = "boundary quadrature not exact"; return false; }
    all = true;
    Fem2D::Expandsetoflab(stack, di, labs, all);
    if (!all) r.labels.assign(labs.begin(), labs.end());
    return true;
}

// A boundary FormBilinear: Robin sum over the components of c u_j v_j, the same c for every
// component; r.robin per boundary element.
template <class MMesh, class FES>
static bool read_boundary_bilinear(Stack stack, const MMesh &Th, const FES &Uh, const CDomainOfIntegration &di,
                                   const BilinearOperator &op, int fe, BoundaryRec &r, std::string &why) {
    const int d = Dim<MMesh>::d, nc = fe == FFGPU_FE_P2VEC3 ? 3 : 1, order = fe == FFGPU_FE_P1 ? 1 : 2;
    std::set<int> labs;
    bool all;
    if (!boundary_domain_labels(stack, Th, di, 2 * order, labs, all, r, why)) return false;
    const int nbe = nb_boundary(Th);
    std::vector<double> per((size_t)nbe * nc, 0.0);
    for (BilinearOperator::const_iterator l = op.v.begin(); l != op.v.end(); ++l) {
        const int ju = l->first.first.first, jv = l->first.second.first;
        if (ju != jv || ju >= nc || op_index(l->first.first.second, d) != 0 || op_index(l->first.second.second, d) != 0) {
            why = "boundary term other than c*u*v"; return false;
        }
        if (!boundary_values(stack, Th, Uh, labs, all, l->second, per, nc, ju)) {
            why = "boundary coefficient not constant on boundary elements"; return false;
        }
    }
    r.robin.assign(nbe, 0.0);
    for (int e = 0; e < nbe; ++e) {
        for (int c = 1; c < nc; ++c)
            if (per[(size_t)e * nc + c] != per[(size_t)e * nc]) { why = "Robin coefficients differ between components"; return false; }
        r.robin[e] = per[(size_t)e * nc];
    }
    return true;
}

// A boundary FormLinear: sources g_j v_j; r.g per boundary element and component.
template <class MMesh, class FES>
static bool read_boundary_linear(Stack stack, const MMesh &Th, const FES &Uh, const CDomainOfIntegration &di,
                                 const Ftest &ft, int fe, BoundaryRec &r, std::string &why) {
    const int d = Dim<MMesh>::d, nc = fe == FFGPU_FE_P2VEC3 ? 3 : 1, order = fe == FFGPU_FE_P1 ? 1 : 2;
    std::set<int> labs;
    bool all;
    if (!boundary_domain_labels(stack, Th, di, order, labs, all, r, why)) return false;
    r.g.assign((size_t)nb_boundary(Th) * nc, 0.0);
    for (Ftest::const_iterator l = ft.v.begin(); l != ft.v.end(); ++l) {
        const int jv = l->first.first;
        if (jv >= nc || op_index(l->first.second, d) != 0) { why = "boundary term other than g*v"; return false; }
        if (!boundary_values(stack, Th, Uh, labs, all, l->second, r.g, nc, jv)) {
            why = "boundary source not constant on boundary elements"; return false;
        }
    }
    return true;
}

// the C ABI's view of the recognised boundary terms
static std::vector<ffgpu_bterm> c_bterms(const std::vector<BoundaryRec> &bt) {
    std::vector<ffgpu_bterm> out(bt.size());
    for (size_t t = 0; t < bt.size(); ++t) {
        memset(&out[t], 0, sizeof(ffgpu_bterm));
        out[t].nlabels = (int)bt[t].labels.size();
        out[t].labels = bt[t].labels.empty() ? nullptr : bt[t].labels.data();
        out[t].robin = bt[t].robin.empty() ? nullptr : bt[t].robin.data();
        out[t].g = bt[t].g.empty() ? nullptr : bt[t].g.data();
    }
    return out;
}

// Reads the form's terms.  Returns true when the device can assemble it; r.why otherwise.
template <class MMesh, class FES>
static bool recognise(Stack stack, const list<C_F0> &largs, const MMesh &Th, const FES &Uh, Recognised &r) {
    typedef typename Dim<MMesh>::Rd Rd;
    const int d = Dim<MMesh>::d;
    r.fe = fe_kind(Uh);
    if (!r.fe) { r.why = "element type"; return false; }
    const int nc = r.fe == FFGPU_FE_P2VEC3 ? 3 : 1;
    r.form = nc == 3 ? FFGPU_FORM_ELASTICITY : FFGPU_FORM_DIFFUSION;
    const int nt = Th.nt;
    // coefficient of (u_j, op_p) (v_i, op_q), ops 0 id, 1..d derivatives: per element (scalar)
    // or constant (vector space), accumulated over all terms
    const int NO = 1 + d, NT = nc * NO;
    std::vector<double> tab((size_t)NT * NT, 0.0);
    std::vector<double> kx(r.fe == FFGPU_FE_P2VEC3 ? 0 : (size_t)nt * (d + 1), 0.0);   // k_dd per element, mass
    std::set<long> on;
    FreeFempp::TypeVarForm<double> *tvf = FreeFempp::TypeVarForm<double>::Global;
    MeshPoint mp = *MeshPointStack(stack);
    Rd pa, pb;
    ref_points(pa, pb);
    bool ok = true;
    for (list<C_F0>::const_iterator ii = largs.begin(); ok && ii != largs.end(); ++ii) {
        aType t = ii->left();
        Expression e = ii->LeftValue();
        if (t == tvf->tBC) {
            const BC_set *bc = dynamic_cast<const BC_set *>(e);
            if (!bc) { r.why = "boundary condition"; ok = false; break; }
            // constrained components: one set for all on(...) of the form
            int mask = 0;
            for (size_t i = 0; i < bc->bc.size(); ++i) mask |= 1 << bc->bc[i].first;
            if (r.comp_mask >= 0 && r.comp_mask != mask) { r.why = "on() with different components"; ok = false; break; }
            r.comp_mask = mask;
            Fem2D::Expandsetoflab(stack, *bc, on);
            continue;
        }
        if (t == tvf->tFL) continue;   // linear terms: not part of the matrix
        if (t != tvf->tFB) { r.why = "term kind"; ok = false; break; }
        const FormBilinear *bf = dynamic_cast<const FormBilinear *>(e);
        const CDomainOfIntegration &di = *bf->di;
        if (boundary_domain(di, d)) {
            BoundaryRec br;
            if (!read_boundary_bilinear(stack, Th, Uh, di, *bf->b, r.fe, br, r.why)) { ok = false; break; }
            r.bterms.push_back(br);
            continue;
        }
        if (!volume_domain(di, d)) { r.why = "domain of integration"; ok = false; break; }
        if (GetAny<const MMesh *>((*di.Th)(stack)) != &Th) { r.why = "integration mesh"; ok = false; break; }
        const int ex = exactness(stack, di, &Th);
        const BilinearOperator &op = *bf->b;
        for (BilinearOperator::const_iterator l = op.v.begin(); ok && l != op.v.end(); ++l) {
            const int ju = l->first.first.first, jv = l->first.second.first;
            const int pu = op_index(l->first.first.second, d), pv = op_index(l->first.second.second, d);
            if (ju >= nc || jv >= nc || pu < 0 || pv < 0) { r.why = "operator"; ok = false; break; }
            // degree of the integrand for these two operators (coefficient constant on elements)
            const int order = r.fe == FFGPU_FE_P1 ? 1 : 2;
            const int deg = (pu ? order - 1 : order) + (pv ? order - 1 : order);
            const bool constant = l->second.LeftValue()->MeshIndependent();
            if (nc == 1 && pu == 0 && pv == 0 && ju == 0 && jv == 0 && (!constant || ex < deg)) {
                // a mass coefficient that depends on the point, or a rule that does not integrate
                // the mass exactly: the coefficient at the rule's points
                if (!coef_at_points(stack, l->second, Th, Uh, di, r, r.mqp)) { ok = false; break; }
                continue;
            }
            if (ex < deg) { r.why = "quadrature not exact for the form"; ok = false; break; }
            if (nc == 3) {
                // elasticity: coefficients independent of the mesh point
                if (!constant) { r.why = "coefficient not constant"; ok = false; break; }
                typename FES::FElement FK = Uh[0];
                MeshPointStack(stack)->set(Th[0](pa), pa, FK);
                tab[(size_t)(ju * NO + pu) * NT + (jv * NO + pv)] += GetAny<double>(l->second.eval(stack));
                continue;
            }
            if (constant) {
                typename FES::FElement FK = Uh[0];
                MeshPointStack(stack)->set(Th[0](pa), pa, FK);
                const double c = GetAny<double>(l->second.eval(stack));
                if (pu == pv && pu > 0) for (int k = 0; k < nt; ++k) kx[(size_t)k * (d + 1) + pu - 1] += c;
                else if (pu == 0 && pv == 0) for (int k = 0; k < nt; ++k) kx[(size_t)k * (d + 1) + d] += c;
                else if (c != 0.0) { r.why = "mixed derivative term"; ok = false; }
                continue;
            }
            // coefficient depending on the point.  A P1 stiffness term takes any coefficient,
            // as its average by the form's own quadrature rule (the gradients are constant on
            // the element); other terms need it constant on every element (P0)
            const bool p1_stiff = r.fe == FFGPU_FE_P1 && pu == pv && pu > 0;
            std::vector<double> cterm(nt);   // the term's value per element, added once all pass
            bool at_points = false;
            for (int k = 0; k < nt; ++k) {
                typename FES::FElement FK = Uh[k];
                MeshPointStack(stack)->set(Th[k](pa), pa, FK);
                double ca = GetAny<double>(l->second.eval(stack));
                MeshPointStack(stack)->set(Th[k](pb), pb, FK);
                const double cb = GetAny<double>(l->second.eval(stack));
                if (!(std::fabs(ca - cb) <= 1e-14 * std::max(std::fabs(ca), std::fabs(cb)))) {
                    if (!p1_stiff) {
                        // a P2 stiffness term dx_d(u) dx_d(v): its coefficient at the rule's points
                        if (pu == pv && pu > 0 && ju == 0 && jv == 0) { at_points = true; break; }
                        r.why = "coefficient not constant on elements (a P1 stiffness term takes any)"; ok = false; break;
                    }
                    ca = rule_average(stack, l->second, Th[k], FK, di);
                }
                if (!(pu == pv && pu > 0) && !(pu == 0 && pv == 0) && ca != 0.0) {
                    r.why = "mixed derivative term"; ok = false; break;
                }
                cterm[k] = ca;
            }
            if (!ok) break;
            if (at_points) {
                if (!coef_at_points(stack, l->second, Th, Uh, di, r, r.kqp[pu - 1])) { ok = false; break; }
                continue;
            }
            for (int k = 0; k < nt; ++k) {
                if (pu == pv && pu > 0) kx[(size_t)k * (d + 1) + pu - 1] += cterm[k];
                else if (pu == 0 && pv == 0) kx[(size_t)k * (d + 1) + d] += cterm[k];
            }
        }
    }
    *MeshPointStack(stack) = mp;
    if (!ok) return false;
    r.labels.assign(on.begin(), on.end());
    if (nc == 1) {
        r.kappa.resize(nt);
        const double m0 = kx[d];
        for (int k = 0; k < nt; ++k) {
            const double *c = &kx[(size_t)k * (d + 1)];
            for (int a = 1; a < d; ++a)
                if (c[a] != c[0]) { r.why = "anisotropic diffusion"; return false; }
            if (!r.mqp.empty())   // constant mass terms join the values at the points
                for (int q = 0; q < r.nqp; ++q) r.mqp[(size_t)k * r.nqp + q] += c[d];
            else if (c[d] != m0) { r.why = "mass coefficient not constant"; return false; }
            r.kappa[k] = c[0];
        }
        r.c_mass = r.mqp.empty() ? m0 : 0.0;
        bool at = false;
        for (int a = 0; a < d; ++a) at |= !r.kqp[a].empty();
        if (at) {
            // stiffness at the points: the constant / P0 parts join, every derivative alike
            for (int a = 0; a < d; ++a) {
                if (r.kqp[a].empty()) r.kqp[a].assign((size_t)nt * r.nqp, 0.0);
                for (int k = 0; k < nt; ++k)
                    for (int q = 0; q < r.nqp; ++q) r.kqp[a][(size_t)k * r.nqp + q] += kx[(size_t)k * (d + 1) + a];
            }
            for (int a = 1; a < d; ++a)
                if (r.kqp[a] != r.kqp[0]) { r.why = "anisotropic diffusion"; return false; }
            for (int k = 0; k < nt; ++k) r.kappa[k] = 1.0;
        }
        return true;
    }
    // isotropic elasticity: T[(j,p),(i,q)] = lambda d_jp d_iq + mu (d_ij d_pq + d_jq d_ip)
    const double lam = tab[(size_t)(0 * NO + 1) * NT + (1 * NO + 2)];
    const double mu = tab[(size_t)(0 * NO + 2) * NT + (0 * NO + 2)];
    for (int j = 0; j < 3; ++j)
        for (int p = 0; p <= 3; ++p)
            for (int i = 0; i < 3; ++i)
                for (int q = 0; q <= 3; ++q) {
                    double want = 0;
                    if (p > 0 && q > 0) {
                        const int pp = p - 1, qq = q - 1;
                        want = lam * (j == pp) * (i == qq) + mu * ((i == j) * (pp == qq) + (j == qq) * (i == pp));
                    }
                    const double got = tab[(size_t)(j * NO + p) * NT + (i * NO + q)];
                    if (std::fabs(got - want) > 1e-13 * (std::fabs(lam) + std::fabs(mu)))
                        { r.why = "not isotropic elasticity"; return false; }
                }
    r.lam = lam;
    r.mu = mu;
    return true;
}

// mesh arrays in the C ABI's layout
static void mesh_arrays(const Mesh &Th, std::vector<double> &X, std::vector<int32_t> &E, std::vector<int32_t> &BE,
                        std::vector<int32_t> &BL) {
    X.resize(2 * (size_t)Th.nv);
    for (int i = 0; i < Th.nv; ++i) { X[2 * i] = Th(i).x; X[2 * i + 1] = Th(i).y; }
    E.resize(3 * (size_t)Th.nt);
    for (int k = 0; k < Th.nt; ++k)
        for (int j = 0; j < 3; ++j) E[3 * (size_t)k + j] = Th(Th[k][j]);
    BE.resize(2 * (size_t)Th.neb);
    BL.resize(Th.neb);
    for (int i = 0; i < Th.neb; ++i) {
        for (int j = 0; j < 2; ++j) BE[2 * (size_t)i + j] = Th(Th.bedges[i][j]);
        BL[i] = Th.bedges[i].lab;
    }
}
static void mesh_arrays(const Mesh3 &Th, std::vector<double> &X, std::vector<int32_t> &E, std::vector<int32_t> &BE,
                        std::vector<int32_t> &BL) {
    X.resize(3 * (size_t)Th.nv);
    for (int i = 0; i < Th.nv; ++i) { X[3 * i] = Th(i).x; X[3 * i + 1] = Th(i).y; X[3 * i + 2] = Th(i).z; }
    E.resize(4 * (size_t)Th.nt);
    for (int k = 0; k < Th.nt; ++k)
        for (int j = 0; j < 4; ++j) E[4 * (size_t)k + j] = Th(Th[k][j]);
    BE.resize(3 * (size_t)Th.nbe);
    BL.resize(Th.nbe);
    for (int i = 0; i < Th.nbe; ++i) {
        for (int j = 0; j < 3; ++j) BE[3 * (size_t)i + j] = Th(Th.be(i)[j]);
        BL[i] = Th.be(i).lab;
    }
}

static void dump(const std::string &path, const void *p, size_t n) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) ExecError(("ffgpu: cannot write " + path).c_str());
    if (n) fwrite(p, 1, n, f);
    fclose(f);
}

static const char *fe_name(int fe) { return fe == FFGPU_FE_P1 ? "P1" : (fe == FFGPU_FE_P2 ? "P2" : "[P2,P2,P2]"); }

// The device assembly of a recognised form into FreeFEM's matrix object; false: not ours.
template <class MMesh, class FES>
static bool device_matrix(Stack stack, const list<C_F0> &largs, const FES &Uh, const Data_Sparse_Solver &ds,
                          Matrice_Creuse<double> &A, ffgpu_matrix **keep) {
    const MMesh &Th = Uh.Th;
    const int d = Dim<MMesh>::d;
    Recognised r;
    if (ds.sym) r.why = "symmetric storage requested";
    else if (!recognise(stack, largs, Th, Uh, r)) {}
    if (!r.why.empty()) {
        not_on_device("form", r.why);
        return false;
    }
    double ksum = 0;
    for (size_t k = 0; k < r.kappa.size(); ++k) ksum += r.kappa[k] * (double)(k % 7 + 1);
    if (verbosity > 1) {
        std::cout << "  ffgpu: device assembly " << fe_name(r.fe) << " dim " << d << " nt " << Th.nt
                  << " ndof " << Uh.NbOfDF;
        if (r.form == FFGPU_FORM_ELASTICITY) std::cout << " lambda " << r.lam << " mu " << r.mu;
        else std::cout << " kappa-check " << std::setprecision(17) << ksum << " mass " << r.c_mass;
        if (!r.mqp.empty()) {
            double ms = 0;
            for (size_t k = 0; k < r.mqp.size(); ++k) ms += r.mqp[k] * (double)(k % 7 + 1);
            std::cout << " | mass at " << r.nqp << " points, mq-check " << std::setprecision(17) << ms;
        }
        if (!r.kqp[0].empty()) {
            double ks = 0;
            for (size_t k = 0; k < r.kqp[0].size(); ++k) ks += r.kqp[0][k] * (double)(k % 7 + 1);
            std::cout << " | stiffness at " << r.nqp << " points, kq-check " << std::setprecision(17) << ks;
        }
        std::cout << " tgv " << ds.tgv << " components " << r.comp_mask << " labels";
        for (size_t i = 0; i < r.labels.size(); ++i) std::cout << " " << r.labels[i];
        for (size_t t = 0; t < r.bterms.size(); ++t) {
            double rs = 0;
            for (size_t e = 0; e < r.bterms[t].robin.size(); ++e) rs += r.bterms[t].robin[e] * (double)(e % 7 + 1);
            std::cout << " | robin-check " << std::setprecision(17) << rs << " on";
            if (r.bterms[t].labels.empty()) std::cout << " all";
            for (size_t i = 0; i < r.bterms[t].labels.size(); ++i) std::cout << " " << r.bterms[t].labels[i];
        }
        std::cout << std::setprecision(6) << std::endl;
    }
    std::vector<double> X;
    std::vector<int32_t> E, BE, BL;
    mesh_arrays(Th, X, E, BE, BL);
    const int ndofK = Uh[0].NbDoF();
    std::vector<int32_t> dof((size_t)Th.nt * ndofK);
    for (int k = 0; k < Th.nt; ++k) {
        typename FES::FElement K = Uh[k];
        if (K.NbDoF() != ndofK) ExecError("ffgpu: elements with different numbers of DOFs");
        for (int i = 0; i < ndofK; ++i) dof[(size_t)k * ndofK + i] = K(i);
    }
    if (const char *dir = getenv("FFGPU_PLUGIN_DUMP")) {
        // the arrays handed to the C ABI, for checking the extraction against other builders
        const std::string p(dir);
        dump(p + "/coords.bin", X.data(), X.size() * sizeof(double));
        dump(p + "/elems.bin", E.data(), E.size() * sizeof(int32_t));
        dump(p + "/dof.bin", dof.data(), dof.size() * sizeof(int32_t));
        dump(p + "/belems.bin", BE.data(), BE.size() * sizeof(int32_t));
        dump(p + "/blabel.bin", BL.data(), BL.size() * sizeof(int32_t));
        dump(p + "/kappa.bin", r.kappa.data(), r.kappa.size() * sizeof(double));
        dump(p + "/mass_qp.bin", r.mqp.data(), r.mqp.size() * sizeof(double));
        dump(p + "/stiff_qp.bin", r.kqp[0].data(), r.kqp[0].size() * sizeof(double));
        for (size_t t = 0; t < r.bterms.size(); ++t)
            dump(p + "/robin" + std::to_string(t) + ".bin", r.bterms[t].robin.data(), r.bterms[t].robin.size() * sizeof(double));
    }
    ffgpu_ctx *ctx = context();
    ffgpu_space *S = nullptr;
    ffgpu_matrix *M = nullptr;
    int rc = ffgpu_space_create(ctx, d, Th.nv, X.data(), Th.nt, E.data(), r.fe, ndofK, dof.data(), Uh.NbOfDF, &S);
    if (!rc && !BL.empty()) rc = ffgpu_space_set_boundary(S, (int)BL.size(), BE.data(), BL.data());
    if (!rc) {
        ffgpu_varf v;
        memset(&v, 0, sizeof(v));
        v.form = r.form;
        v.c_stiff = 1.0;
        if (r.form == FFGPU_FORM_ELASTICITY) {
            v.E = r.mu * (3 * r.lam + 2 * r.mu) / (r.lam + r.mu);
            v.nu = r.lam / (2 * (r.lam + r.mu));
        } else {
            v.kappa = r.kappa.data();
            v.c_mass = r.c_mass;
            if (r.nqp) {
                v.nqp = r.nqp;
                v.qp_lambda = r.lam_q.data();
                v.qp_weight = r.w_q.data();
                v.mass_qp = r.mqp.empty() ? nullptr : r.mqp.data();
                v.stiff_qp = r.kqp[0].empty() ? nullptr : r.kqp[0].data();
            }
        }
        const std::vector<ffgpu_bterm> bt = c_bterms(r.bterms);
        v.nbterms = (int)bt.size();
        v.bterms = bt.empty() ? nullptr : bt.data();
        ffgpu_bc bc;
        memset(&bc, 0, sizeof(bc));
        bc.tgv = ds.tgv;
        bc.nlabels = (int)r.labels.size();
        bc.labels = r.labels.data();
        bc.comp_mask = r.fe == FFGPU_FE_P2VEC3 && r.comp_mask != 7 ? r.comp_mask : 0;
        rc = ffgpu_matrix_assemble(S, &v, r.labels.empty() ? nullptr : &bc, nullptr, &M);
    }
    int n = 0, bs = 0;
    int64_t nnz = 0;
    std::vector<int32_t> rp, col;
    std::vector<double> val;
    if (!rc) rc = ffgpu_matrix_info(M, &n, &nnz, &bs);
    if (!rc) {
        rp.resize(n + 1);
        col.resize(nnz);
        val.resize(nnz);
        rc = ffgpu_matrix_csr(M, rp.data(), col.data(), val.data());
    }
    // the matrix stays on the device for a GPU solver of A; the space's arrays it needs for
    // reassembly are not kept (a reassembly comes through this path again)
    if (rc && M) { ffgpu_matrix_destroy(M); M = nullptr; }
    if (S) ffgpu_space_destroy(S);
    if (rc) ExecError((std::string("ffgpu assembly: ") + ffgpu_last_error()).c_str());
    // FreeFEM's matrix object, as creationBlockOfMatrixToBilinearForm leaves it (problem.hpp:1663-1714)
    A.A = 0;
    A.Uh = Uh;
    A.Vh = Uh;
    HashMatrix<int, double> *H = new HashMatrix<int, double>(n, n, 0, 0);
    H->set(n, n, 0, (size_t)nnz, rp.data(), col.data(), val.data(), 0, 1);
    // H now holds the device matrix's values: clear its change flags, so that a solver can tell
    // whether the script modified A before the first solve
    H->GetReDoNumerics();
    H->GetReDoSymbolic();
    A.A.master(H);
    *keep = M;
    return true;
}

// the device matrix to the GPU solver of A, if A has one of ours; otherwise it is freed
static void hand_over(VirtualMatrix<int, double> &VA, ffgpu_matrix *M) {
    if (!M) return;
    VirtualSolver<int, double> *vs = dynamic_cast<VirtualSolver<int, double> *>(VA.vsolver);
    if (SolverGpu<kCG> *s = dynamic_cast<SolverGpu<kCG> *>(vs)) return s->adopt(M);
    if (SolverGpu<kGMRES> *s = dynamic_cast<SolverGpu<kGMRES> *>(vs)) return s->adopt(M);
    if (SolverGpu<kMixed> *s = dynamic_cast<SolverGpu<kMixed> *>(vs)) return s->adopt(M);
    if (SolverGpu<kCholesky> *s = dynamic_cast<SolverGpu<kCholesky> *>(vs)) return s->adopt(M);
    if (SolverGpu<kSparse> *s = dynamic_cast<SolverGpu<kSparse> *>(vs)) return s->adopt(M);
    ffgpu_matrix_destroy(M);
}

template <class MMesh, class v_fes>
struct GpuBilinear : public OpMatrixtoBilinearForm<double, MMesh, v_fes, v_fes> {
    typedef OpMatrixtoBilinearForm<double, MMesh, v_fes, v_fes> Base;
    typedef typename v_fes::pfes pfes;
    typedef typename v_fes::FESpace FES;
    class GOp : public Base::Op {
       public:
        GOp(Expression aa, Expression bb, int initt) : Base::Op(aa, bb, initt) {}
        AnyType operator()(Stack stack) const {
            const Call_FormBilinear<v_fes, v_fes> *b = this->b;
            pfes *pUh = GetAny<pfes *>((*b->euh)(stack));
            pfes *pVh = GetAny<pfes *>((*b->evh)(stack));
            const FES *PUh = (FES *)**pUh, *PVh = (FES *)**pVh;
            if (!PUh || PUh != PVh || isVF(b->largs)) {
                not_on_device("form", !PUh ? "no space" : (PUh != PVh ? "different test and trial spaces" : "a VF form"));
                return Base::Op::operator()(stack);
            }
            Data_Sparse_Solver ds;
            ds.factorize = 0;
            ds.initmat = true;
            const int np = OpCall_FormBilinear_np::n_name_param - NB_NAME_PARM_HMAT;
            SetEnd_Data_Sparse_Solver<double>(stack, ds, b->nargs, np);
            Matrice_Creuse<double> &A(*GetAny<Matrice_Creuse<double> *>((*this->a)(stack)));
            if (this->init) A.init();
            ffgpu_matrix *M = nullptr;
            if (!device_matrix<MMesh, FES>(stack, b->largs, *PUh, ds, A, &M)) return Base::Op::operator()(stack);
            A.pHM()->half = ds.sym;
            SetSolver(stack, false, *A.A, ds);
            hand_over(*A.A, M);
            return SetAny<Matrice_Creuse<double> *>(&A);
        }
    };
    E_F0 *code(const basicAC_F0 &args) const {
        return new GOp(to<Matrice_Creuse<double> *>(args[0]), args[1], this->init);
    }
    GpuBilinear(int initt) : Base(initt) { this->pref = 10; }
};

// ------------------------------------------------------------------ device linear form
// `b = a(0, Vh)` for a recognised space: int(Th)(f*v) terms with f constant on elements (per
// component for [P2,P2,P2]), exact quadrature, on(labels, u = constants).  Bilinear terms do not
// contribute to b.  Anything else, and `b += a(0,Vh)`, is FreeFEM's own operator.
struct RecognisedRhs {
    int fe = 0;
    std::vector<double> f;        // nt x ncomp
    // sources that are not constant on elements: values at the points of the rule
    int nqp = 0;
    std::vector<double> lam, w;   // nqp x (dim+1) barycentric coordinates, weights
    std::vector<double> fqp;      // (nt x nqp) x ncomp
    std::vector<int32_t> labels;
    std::vector<BoundaryRec> bterms;   // boundary sources, in varf order
    double g[3] = {0, 0, 0};      // on(...) values per component
    int comp_mask = -1;
    std::string why;
};

// Every volume source term taken at the points of its rule, as Element_rhs takes it
// (problem.cpp:7839-7911, 7917-7990), summed per (element, point, component); the terms must
// share one rule.  The device integrates the values with the rule's weights.
template <class MMesh, class FES>
static bool rhs_at_points(Stack stack, const list<C_F0> &largs, const MMesh &Th, const FES &Uh, RecognisedRhs &r) {
    typedef typename Dim<MMesh>::Rd Rd;
    const int d = Dim<MMesh>::d, nc = r.fe == FFGPU_FE_P2VEC3 ? 3 : 1, nt = Th.nt;
    FreeFempp::TypeVarForm<double> *tvf = FreeFempp::TypeVarForm<double>::Global;
    r.nqp = 0;
    for (list<C_F0>::const_iterator ii = largs.begin(); ii != largs.end(); ++ii) {
        if (ii->left() != tvf->tFL) continue;
        const FormLinear *lf = dynamic_cast<const FormLinear *>(ii->LeftValue());
        const CDomainOfIntegration &di = *lf->di;
        if (!volume_domain(di, d)) continue;   // boundary sources: per boundary element
        const int nq = rule_size(stack, di, &Th);
        std::vector<Rd> P(nq);
        std::vector<double> lam((size_t)nq * (d + 1)), w(nq);
        for (int q = 0; q < nq; ++q) {
            rule_point(stack, di, q, P[q], w[q]);
            barycentric(P[q], &lam[(size_t)q * (d + 1)]);
        }
        if (r.nqp == 0) {
            if (nq < 1 || nq > 64) { r.why = "quadrature rule size"; return false; }
            r.nqp = nq;
            r.lam = lam;
            r.w = w;
            r.fqp.assign((size_t)nt * nq * nc, 0.0);
        } else if (lam != r.lam || w != r.w) {
            r.why = "volume sources with different quadrature rules";
            return false;
        }
        const Ftest &ft = *lf->l;
        for (Ftest::const_iterator l = ft.v.begin(); l != ft.v.end(); ++l) {
            const int jv = l->first.first;
            for (int k = 0; k < nt; ++k) {
                typename FES::FElement FK = Uh[k];
                for (int q = 0; q < nq; ++q) {
                    MeshPointStack(stack)->set(Th[k](P[q]), P[q], FK);
                    r.fqp[((size_t)k * nq + q) * nc + jv] += GetAny<double>(l->second.eval(stack));
                }
            }
        }
    }
    r.f.assign(r.f.size(), 0.0);
    return true;
}

template <class MMesh, class FES>
static bool recognise_rhs(Stack stack, const list<C_F0> &largs, const MMesh &Th, const FES &Uh, RecognisedRhs &r) {
    typedef typename Dim<MMesh>::Rd Rd;
    const int d = Dim<MMesh>::d;
    r.fe = fe_kind(Uh);
    if (!r.fe) { r.why = "element type"; return false; }
    const int nc = r.fe == FFGPU_FE_P2VEC3 ? 3 : 1, nt = Th.nt;
    r.f.assign((size_t)nt * nc, 0.0);
    std::set<long> on;
    FreeFempp::TypeVarForm<double> *tvf = FreeFempp::TypeVarForm<double>::Global;
    MeshPoint mp = *MeshPointStack(stack);
    Rd pa, pb;
    ref_points(pa, pb);
    bool ok = true, at_points = false;
    for (list<C_F0>::const_iterator ii = largs.begin(); ok && ii != largs.end(); ++ii) {
        aType t = ii->left();
        Expression e = ii->LeftValue();
        if (t == tvf->tFB) continue;   // bilinear terms: not part of b
        if (t == tvf->tBC) {
            const BC_set *bc = dynamic_cast<const BC_set *>(e);
            int mask = 0;
            for (size_t i = 0; ok && i < bc->bc.size(); ++i) {
                const int c = bc->bc[i].first;
                mask |= 1 << c;
                if (!bc->bc[i].second->MeshIndependent()) { r.why = "on() value not constant"; ok = false; break; }
                const double gv = GetAny<double>((*bc->bc[i].second)(stack));
                if (r.comp_mask >= 0 && (r.comp_mask >> c & 1) && r.g[c] != gv) { r.why = "on() values differ"; ok = false; }
                r.g[c] = gv;
            }
            if (r.comp_mask >= 0 && r.comp_mask != mask) { r.why = "on() with different components"; ok = false; }
            r.comp_mask = mask;
            Fem2D::Expandsetoflab(stack, *bc, on);
            continue;
        }
        if (t != tvf->tFL) { r.why = "term kind"; ok = false; break; }
        const FormLinear *lf = dynamic_cast<const FormLinear *>(e);
        const CDomainOfIntegration &di = *lf->di;
        if (boundary_domain(di, d)) {
            BoundaryRec br;
            if (!read_boundary_linear(stack, Th, Uh, di, *lf->l, r.fe, br, r.why)) { ok = false; break; }
            r.bterms.push_back(br);
            continue;
        }
        if (!volume_domain(di, d)) { r.why = "domain of integration"; ok = false; break; }
        if (GetAny<const MMesh *>((*di.Th)(stack)) != &Th) { r.why = "integration mesh"; ok = false; break; }
        // a rule that does not integrate the basis exactly: the values at its points
        if (exactness(stack, di, &Th) < (r.fe == FFGPU_FE_P1 ? 1 : 2)) at_points = true;
        const Ftest &ft = *lf->l;
        for (Ftest::const_iterator l = ft.v.begin(); ok && l != ft.v.end(); ++l) {
            const int jv = l->first.first, pv = op_index(l->first.second, d);
            if (jv >= nc || pv != 0) { r.why = "operator"; ok = false; break; }
            const bool constant = l->second.LeftValue()->MeshIndependent();
            for (int k = 0; !at_points && k < nt; ++k) {
                typename FES::FElement FK = Uh[k];
                MeshPointStack(stack)->set(Th[k](pa), pa, FK);
                const double ca = GetAny<double>(l->second.eval(stack));
                if (!constant) {
                    MeshPointStack(stack)->set(Th[k](pb), pb, FK);
                    const double cb = GetAny<double>(l->second.eval(stack));
                    if (!(std::fabs(ca - cb) <= 1e-14 * std::max(std::fabs(ca), std::fabs(cb)))) {
                        at_points = true;   // a function of the point: the rule's points
                        break;
                    }
                }
                r.f[(size_t)k * nc + jv] += ca;
                if (constant && k == 0) {   // the same value everywhere
                    for (int kk = 1; kk < nt; ++kk) r.f[(size_t)kk * nc + jv] += ca;
                    break;
                }
            }
        }
    }
    if (ok && at_points) ok = rhs_at_points(stack, largs, Th, Uh, r);
    *MeshPointStack(stack) = mp;
    if (!ok) return false;
    r.labels.assign(on.begin(), on.end());
    return true;
}

template <class MMesh, class FES>
static bool device_rhs(Stack stack, const list<C_F0> &largs, const FES &Uh, double tgv, KN_<double> &out) {
    const MMesh &Th = Uh.Th;
    const int d = Dim<MMesh>::d;
    RecognisedRhs r;
    if (!recognise_rhs(stack, largs, Th, Uh, r)) {
        not_on_device("linear form", r.why);
        return false;
    }
    if (verbosity > 1) {
        double fs = 0;
        for (size_t k = 0; k < r.f.size(); ++k) fs += r.f[k] * (double)(k % 7 + 1);
        std::cout << "  ffgpu: device linear form " << fe_name(r.fe) << " dim " << d << " f-check " << std::setprecision(17)
                  << fs << " g " << r.g[0] << std::setprecision(6) << " tgv " << tgv;
        if (r.nqp) {
            double qs = 0;
            for (size_t k = 0; k < r.fqp.size(); ++k) qs += r.fqp[k] * (double)(k % 7 + 1);
            std::cout << " | at " << r.nqp << " points, fq-check " << std::setprecision(17) << qs << std::setprecision(6);
        }
        for (size_t t = 0; t < r.bterms.size(); ++t) {
            double gs = 0;
            for (size_t e = 0; e < r.bterms[t].g.size(); ++e) gs += r.bterms[t].g[e] * (double)(e % 7 + 1);
            std::cout << " | g-check " << std::setprecision(17) << gs << std::setprecision(6) << " on";
            if (r.bterms[t].labels.empty()) std::cout << " all";
            for (size_t i = 0; i < r.bterms[t].labels.size(); ++i) std::cout << " " << r.bterms[t].labels[i];
        }
        std::cout << std::endl;
    }
    std::vector<double> X;
    std::vector<int32_t> E, BE, BL;
    mesh_arrays(Th, X, E, BE, BL);
    const int ndofK = Uh[0].NbDoF(), nc = r.fe == FFGPU_FE_P2VEC3 ? 3 : 1;
    if (const char *dir = getenv("FFGPU_PLUGIN_DUMP")) {
        const std::string p(dir);
        dump(p + "/rhs_coords.bin", X.data(), X.size() * sizeof(double));
        dump(p + "/rhs_elems.bin", E.data(), E.size() * sizeof(int32_t));
        dump(p + "/rhs_fqp.bin", r.fqp.data(), r.fqp.size() * sizeof(double));
        dump(p + "/rhs_lambda.bin", r.lam.data(), r.lam.size() * sizeof(double));
        dump(p + "/rhs_weight.bin", r.w.data(), r.w.size() * sizeof(double));
    }
    std::vector<int32_t> dof((size_t)Th.nt * ndofK);
    for (int k = 0; k < Th.nt; ++k) {
        typename FES::FElement K = Uh[k];
        for (int i = 0; i < ndofK; ++i) dof[(size_t)k * ndofK + i] = K(i);
    }
    ffgpu_ctx *ctx = context();
    ffgpu_space *S = nullptr;
    int rc = ffgpu_space_create(ctx, d, Th.nv, X.data(), Th.nt, E.data(), r.fe, ndofK, dof.data(), Uh.NbOfDF, &S);
    if (!rc && !BL.empty()) rc = ffgpu_space_set_boundary(S, (int)BL.size(), BE.data(), BL.data());
    std::vector<double> g;
    if (!rc) {
        ffgpu_varf v;
        memset(&v, 0, sizeof(v));
        v.form = nc == 3 ? FFGPU_FORM_ELASTICITY : FFGPU_FORM_DIFFUSION;
        v.c_stiff = 1.0;
        v.E = 1.0;
        v.f = r.f.data();
        if (r.nqp) {
            v.nqp = r.nqp;
            v.qp_lambda = r.lam.data();
            v.qp_weight = r.w.data();
            v.f_qp = r.fqp.data();
        }
        const std::vector<ffgpu_bterm> bt = c_bterms(r.bterms);
        v.nbterms = (int)bt.size();
        v.bterms = bt.empty() ? nullptr : bt.data();
        ffgpu_bc bc;
        memset(&bc, 0, sizeof(bc));
        bc.tgv = tgv;
        bc.nlabels = (int)r.labels.size();
        bc.labels = r.labels.data();
        bc.comp_mask = nc == 3 && r.comp_mask != 7 ? r.comp_mask : 0;
        if (r.g[0] != 0 || r.g[1] != 0 || r.g[2] != 0) {
            g.resize(Uh.NbOfDF);
            for (int i = 0; i < Uh.NbOfDF; ++i) g[i] = r.g[i % nc];
            bc.g = g.data();
        }
        rc = ffgpu_rhs_assemble(S, &v, r.labels.empty() ? nullptr : &bc, (double *)out);
    }
    if (S) ffgpu_space_destroy(S);
    if (rc) ExecError((std::string("ffgpu linear form: ") + ffgpu_last_error()).c_str());
    return true;
}

template <class MMesh, class v_fes>
struct GpuLinear : public OpArraytoLinearForm<double, MMesh, v_fes> {
    typedef OpArraytoLinearForm<double, MMesh, v_fes> Base;
    typedef typename v_fes::FESpace FES;
    class GOp : public Base::Op {
       public:
        GOp(Expression xx, Expression ll, bool isptr, bool init, bool zero) : Base::Op(xx, ll, isptr, init, zero) {}
        AnyType operator()(Stack stack) const {
            if (!this->zero) return Base::Op::operator()(stack);   // b += a(0,Vh)
            v_fes *&pp = *GetAny<v_fes **>((*this->l->ppfes)(stack));
            FES *pVh = *pp;
            if (!pVh) return Base::Op::operator()(stack);
            double tgv = ff_tgv;
            if (this->l->nargs[0]) tgv = GetAny<double>((*this->l->nargs[0])(stack));
            const long n = pVh->NbOfDF;
            KN<double> *px = nullptr;
            if (this->isptr) {
                px = GetAny<KN<double> *>((*this->x)(stack));
                if (this->init) px->init(n);
                if (px->N() != n) px->resize(n);
            }
            KN_<double> xx(px ? *(KN_<double> *)px : GetAny<KN_<double> >((*this->x)(stack)));
            if (xx.N() != n || xx.step != 1 || !device_rhs<MMesh, FES>(stack, this->l->largs, *pVh, tgv, xx))
                return Base::Op::operator()(stack);
            return SetAny<KN_<double> >(xx);
        }
    };
    E_F0 *code(const basicAC_F0 &args) const {
        if (this->isptr) return new GOp(to<KN<double> *>(args[0]), args[1], this->isptr, this->init, this->zero);
        return new GOp(to<KN_<double> >(args[0]), args[1], this->isptr, this->init, this->zero);
    }
    GpuLinear(const basicForEachType *tt, bool isptrr, bool initt, bool zzero = 1) : Base(tt, isptrr, initt, zzero) {
        this->pref = 10;
    }
};

}  // namespace

static void Load_Init() {
    addsolver<SolverGpu<kCG> >("GPUCG", 20);
    addsolver<SolverGpu<kGMRES> >("GPUGMRES", 20);
    addsolver<SolverGpu<kMixed> >("GPUCGMIXED", 20);
    addsolver<SolverGpu<kCholesky> >("GPUCHOLESKY", 20);
    addsolver<SolverGpu<kSparse> >("GPUSPARSESOLVER", 20);
    // script constants, as lgfem.cpp:6380-6395 declares CG, GMRES, ...: solver=GPUCG
    static std::string gpucg = "GPUCG", gpugmres = "GPUGMRES", gpumixed = "GPUCGMIXED", gpuchol = "GPUCHOLESKY",
                       gpusparse = "GPUSPARSESOLVER";
    Global.New("GPUCG", CConstant<std::string *>(&gpucg));
    Global.New("GPUGMRES", CConstant<std::string *>(&gpugmres));
    Global.New("GPUCGMIXED", CConstant<std::string *>(&gpumixed));
    Global.New("GPUCHOLESKY", CConstant<std::string *>(&gpuchol));
    Global.New("GPUSPARSESOLVER", CConstant<std::string *>(&gpusparse));
    // `ffgpustrict = 1;` in a script: forms the device does not assemble are errors
    Global.New("ffgpustrict", CPValue<long>(g_strict));
    // device assembly behind `matrix A = a(Vh,Vh)` (lgfem.cpp:6669-6673, :6823-6826)
    TheOperators->Add("=", new GpuBilinear<Mesh, v_fes>(0), new GpuBilinear<Mesh3, v_fes3>(0));
    TheOperators->Add("<-", new GpuBilinear<Mesh, v_fes>(1));
    TheOperators->Add("<-", new GpuBilinear<Mesh3, v_fes3>(1));
    // and the linear form `b = a(0,Vh)` (lgfem.cpp:6668-6688)
    TheOperators->Add("=", new GpuLinear<Mesh, v_fes>(atype<KN_<double> >(), false, false),
                      new GpuLinear<Mesh3, v_fes3>(atype<KN_<double> >(), false, false));
    TheOperators->Add("<-", new GpuLinear<Mesh, v_fes>(atype<KN<double> *>(), true, true),
                      new GpuLinear<Mesh3, v_fes3>(atype<KN<double> *>(), true, true));
    if (verbosity > 1)
        std::cout << " load: ffgpu (GPUCG, GPUGMRES, GPUCGMIXED, GPUCHOLESKY, GPUSPARSESOLVER)" << std::endl;
}

LOADFUNC(Load_Init)
