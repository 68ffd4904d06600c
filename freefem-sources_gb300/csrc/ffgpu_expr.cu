// ffgpu_expr.cu -- coefficient and source expressions evaluated on the device at the points of
// a quadrature rule, and the general volume terms int(coef * op_i(v) * op_j(u)) of a scalar
// (P1/P2) space.
//
// FreeFEM evaluates the expression of every varf term at each quadrature point of each element
// inside Element_Op (problem.cpp:6117-6132 in 2D, 6391-6410 in 3D) and Element_rhs
// (problem.cpp:7880-7900), then adds coef * w_q * |K| * op_i(phi_i) * op_j(phi_j) term by term.
// Here an expression is a postfix program (ffgpu_expr); the element kernels run it per point:
//   * terms_kernel: one thread per (element, test function i), the row i of the element matrix
//     of all terms (nn doubles in registers), point by point and term by term as Element_Op;
//   * source_expr_kernel: one thread per element, the element vector of the source.
// The element matrices / vectors then enter the row kernels of the assembly like the other
// per-element contributions (ffgpu_assembly.cu).
#include <math.h>
#include <string.h>

#include <memory>
#include <vector>

#include "ffgpu_internal.cuh"

namespace ffgpu {

constexpr int kMaxTerms = 16;
constexpr int kMaxExprs = 16;     // expressions per launch (terms, or source components)
constexpr int kExprStack = 16;
constexpr int kExprThreads = 128;

struct FeDev {
    int kind;
    const double *values;
    const int32_t *dof;     // element -> DOF table (P2), nn entries per element
};

struct ExprDev {
    int nops;
    const int32_t *ops;
    const double *consts;
    const FeDev *fe;
};

// P2 edges in FreeFEM's local order: 2D edge k opposite vertex k; 3D 01 02 03 12 13 23
template <int DIM>
__device__ __forceinline__ void p2_edge(int k, int &a, int &b) {
    if (DIM == 2) {
        a = k == 0 ? 1 : (k == 1 ? 2 : 0);
        b = k == 0 ? 2 : (k == 1 ? 0 : 1);
    } else {
        a = k < 3 ? 0 : (k < 5 ? 1 : 2);
        b = k < 3 ? k + 1 : (k == 3 ? 2 : 3);
    }
}

// value and gradient of local basis function i of P1 (NN = DIM+1) or P2 at barycentric l
template <int DIM, int NN>
__device__ __forceinline__ double basis_val(int i, const double *l) {
    constexpr int NV = DIM + 1;
    if (NN == NV || i < NV) return NN == NV ? l[i] : l[i] * (2. * l[i] - 1.);
    int a, b;
    p2_edge<DIM>(i - NV, a, b);
    return 4. * l[a] * l[b];
}
template <int DIM, int NN>
__device__ __forceinline__ double basis_der(int i, int d, const double *l, const double *G) {
    constexpr int NV = DIM + 1;
    if (NN == NV) return G[3 * i + d];
    if (i < NV) return (4. * l[i] - 1.) * G[3 * i + d];
    int a, b;
    p2_edge<DIM>(i - NV, a, b);
    return 4. * (l[a] * G[3 * b + d] + l[b] * G[3 * a + d]);
}

// FE function at the point (op 0: value, 1..3: derivative d = op-1)
template <int DIM>
__device__ double fe_at(const FeDev &f, int op, int64_t e, const int32_t *vert, const double *l, const double *G,
                        const int32_t *snodes, int snn) {
    constexpr int NV = DIM + 1;
    if (f.kind == FFGPU_FE_P0) return op == 0 ? __ldg(f.values + e) : 0.0;
    double s = 0;
    if (f.kind == FFGPU_FE_P1) {
        for (int i = 0; i < NV; ++i) {
            const double u = __ldg(f.values + vert[i]);
            s = fma(op == 0 ? l[i] : G[3 * i + op - 1], u, s);
        }
        return s;
    }
    constexpr int N2 = DIM == 2 ? 6 : 10;
    const int32_t *nd = f.dof ? f.dof + e * N2 : snodes + e * snn;
    for (int i = 0; i < N2; ++i) {
        const double u = __ldg(f.values + __ldg(nd + i));
        s = fma(op == 0 ? basis_val<DIM, N2>(i, l) : basis_der<DIM, N2>(i, op - 1, l, G), u, s);
    }
    return s;
}

// Runs the program at the point of barycentric coordinates l in element e.
template <int DIM>
__device__ double expr_eval(const ExprDev &E, int64_t e, const int32_t *vert, const double *X, const double *l,
                            const double *G, const int32_t *snodes, int snn) {
    constexpr int NV = DIM + 1;
    double st[kExprStack];
    int sp = 0;
    for (int pc = 0; pc < E.nops; ++pc) {
        const int op = __ldg(E.ops + pc);
        if (op == FFGPU_OP_CONST) {
            st[sp++] = __ldg(E.consts + __ldg(E.ops + ++pc));
        } else if (op >= FFGPU_OP_X && op <= FFGPU_OP_Z) {
            const int d = op - FFGPU_OP_X;
            double x = 0;
            if (d < DIM)
                for (int i = 0; i < NV; ++i) x = fma(l[i], X[3 * i + d], x);
            st[sp++] = x;
        } else if (op >= FFGPU_OP_FE && op <= FFGPU_OP_DZ) {
            const int k = __ldg(E.ops + ++pc);
            st[sp++] = fe_at<DIM>(E.fe[k], op - FFGPU_OP_FE, e, vert, l, G, snodes, snn);
        } else if (op >= FFGPU_OP_ADD && op <= FFGPU_OP_MAX) {
            const double b = st[--sp], a = st[sp - 1];
            double r;
            switch (op) {
                case FFGPU_OP_ADD: r = a + b; break;
                case FFGPU_OP_SUB: r = a - b; break;
                case FFGPU_OP_MUL: r = a * b; break;
                case FFGPU_OP_DIV: r = a / b; break;
                case FFGPU_OP_POW: r = pow(a, b); break;
                case FFGPU_OP_MIN: r = fmin(a, b); break;
                default: r = fmax(a, b); break;
            }
            st[sp - 1] = r;
        } else {
            const double a = st[sp - 1];
            double r;
            switch (op) {
                case FFGPU_OP_NEG: r = -a; break;
                case FFGPU_OP_EXP: r = exp(a); break;
                case FFGPU_OP_LOG: r = log(a); break;
                case FFGPU_OP_SQRT: r = sqrt(a); break;
                case FFGPU_OP_SIN: r = sin(a); break;
                case FFGPU_OP_COS: r = cos(a); break;
                case FFGPU_OP_TAN: r = tan(a); break;
                case FFGPU_OP_ABS: r = fabs(a); break;
                case FFGPU_OP_TANH: r = tanh(a); break;
                default: r = atan(a); break;
            }
            st[sp - 1] = r;
        }
    }
    return st[0];
}

struct TermDev {
    int iop, jop;
    double c;
    int expr;     // index into the launch's expressions, -1: none
};

struct TermArgs {
    int64_t nt;
    int nqp, nterms;
    const double *lam, *w, *geo, *coords;
    const int32_t *elems, *snodes;
    int snn;
    TermDev t[kMaxTerms];
    ExprDev ex[kMaxExprs];
    double *out;
};

// element vertex coordinates (padded to 3 per vertex) and the barycentric gradients
template <int DIM>
__device__ __forceinline__ void element_frame(const TermArgs &A, int64_t e, int32_t *vert, double *X, double *G) {
    constexpr int NV = DIM + 1;
    const double *ge = A.geo + e * kGeoStride;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        vert[i] = __ldg(A.elems + e * NV + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            X[3 * i + d] = d < DIM ? __ldg(A.coords + (int64_t)vert[i] * DIM + d) : 0.0;
            G[3 * i + d] = d < DIM ? __ldg(ge + 4 + 3 * i + d) : 0.0;
        }
    }
}

// One thread per (element, test function i): row i of the element matrix of all terms,
// |K| sum_q w_q sum_t c_t(x_q) op_i(phi_i) op_j(phi_j)
template <int DIM, int NN>
__global__ void __launch_bounds__(kExprThreads) terms_kernel(TermArgs A) {
    constexpr int NV = DIM + 1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= A.nt * NN) return;
    const int64_t e = t / NN;
    const int i = (int)(t - e * NN);
    int32_t vert[NV];
    double X[3 * NV], G[3 * NV];
    element_frame<DIM>(A, e, vert, X, G);
    double acc[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) acc[j] = 0.0;
    for (int q = 0; q < A.nqp; ++q) {
        double l[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) l[k] = __ldg(A.lam + q * NV + k);
        const double wq = __ldg(A.w + q);
        for (int k = 0; k < A.nterms; ++k) {
            const TermDev &T = A.t[k];
            double c = T.c;
            if (T.expr >= 0) c *= expr_eval<DIM>(A.ex[T.expr], e, vert, X, l, G, A.snodes, A.snn);
            const double vi = T.iop == 0 ? basis_val<DIM, NN>(i, l) : basis_der<DIM, NN>(i, T.iop - 1, l, G);
            const double cv = c * wq * vi;
#pragma unroll
            for (int j = 0; j < NN; ++j) {
                const double uj = T.jop == 0 ? basis_val<DIM, NN>(j, l) : basis_der<DIM, NN>(j, T.jop - 1, l, G);
                acc[j] = fma(cv, uj, acc[j]);
            }
        }
    }
    const double meas = __ldg(A.geo + e * kGeoStride);
#pragma unroll
    for (int j = 0; j < NN; ++j) A.out[(e * NN + i) * NN + j] = meas * acc[j];
}

// One thread per element: |K| sum_q w_q f_c(x_q) phi_i(lambda_q), component c = expression c
template <int DIM, int NN, int BS>
__global__ void __launch_bounds__(kExprThreads) source_expr_kernel(TermArgs A) {
    constexpr int NV = DIM + 1;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= A.nt) return;
    int32_t vert[NV];
    double X[3 * NV], G[3 * NV];
    element_frame<DIM>(A, e, vert, X, G);
    double s[NN * BS];
#pragma unroll
    for (int k = 0; k < NN * BS; ++k) s[k] = 0.0;
    for (int q = 0; q < A.nqp; ++q) {
        double l[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) l[k] = __ldg(A.lam + q * NV + k);
        const double wq = __ldg(A.w + q);
#pragma unroll
        for (int c = 0; c < BS; ++c) {
            const double wf = wq * expr_eval<DIM>(A.ex[c], e, vert, X, l, G, A.snodes, A.snn);
#pragma unroll
            for (int i = 0; i < NN; ++i) s[i * BS + c] = fma(wf, basis_val<DIM, NN>(i, l), s[i * BS + c]);
        }
    }
    const double meas = __ldg(A.geo + e * kGeoStride);
#pragma unroll
    for (int k = 0; k < NN * BS; ++k) A.out[e * NN * BS + k] = meas * s[k];
}

// ------------------------------------------------------------------ host side
// Device copies of the expressions of one call (programs, constants, FE functions).
struct ExprUpload {
    ffgpu_ctx *ctx;
    std::vector<std::unique_ptr<DevIn<int32_t>>> iarr;
    std::vector<std::unique_ptr<DevIn<double>>> darr;
    std::vector<FeDev *> fe_dev;
    int err = FFGPU_OK;
    explicit ExprUpload(ffgpu_ctx *c) : ctx(c) {}
    ~ExprUpload() {
        for (FeDev *p : fe_dev) dfree(ctx, p);
    }
    template <typename T>
    const T *in(std::vector<std::unique_ptr<DevIn<T>>> &vec, const T *p, size_t n) {
        vec.emplace_back(new DevIn<T>(p, n, ctx));
        if (vec.back()->err) err = vec.back()->err;
        return vec.back()->d;
    }
    int add(const ffgpu_expr *x, ffgpu_space *S, ExprDev &out) {
        FFGPU_CHECK(x && x->nops > 0 && x->ops, FFGPU_EINVAL, "expression: empty program");
        FFGPU_CHECK(x->nfe >= 0 && x->nfe <= 64 && (x->nfe == 0 || x->fe), FFGPU_EINVAL, "expression: bad FE list");
        // validate on the host: operands in range, stack depth within bounds, one result
        int depth = 0, nconst = 0;
        std::vector<int32_t> ops(x->nops);
        if (is_device_ptr(x->ops)) {
            FFGPU_CUDA(cudaMemcpy(ops.data(), x->ops, sizeof(int32_t) * x->nops, cudaMemcpyDeviceToHost));
        } else {
            memcpy(ops.data(), x->ops, sizeof(int32_t) * x->nops);
        }
        for (int pc = 0; pc < x->nops; ++pc) {
            const int op = ops[pc];
            if (op == FFGPU_OP_CONST || (op >= FFGPU_OP_FE && op <= FFGPU_OP_DZ)) {
                FFGPU_CHECK(pc + 1 < x->nops, FFGPU_EINVAL, "expression: opcode %d without its operand", op);
                const int k = ops[++pc];
                if (op == FFGPU_OP_CONST) {
                    FFGPU_CHECK(k >= 0 && k < 1 << 20, FFGPU_EINVAL, "expression: constant index %d", k);
                    nconst = k + 1 > nconst ? k + 1 : nconst;
                } else {
                    FFGPU_CHECK(k >= 0 && k < x->nfe, FFGPU_EINVAL, "expression: FE function %d of %d", k, x->nfe);
                }
                ++depth;
            } else if (op >= FFGPU_OP_X && op <= FFGPU_OP_Z) {
                ++depth;
            } else if (op >= FFGPU_OP_ADD && op <= FFGPU_OP_MAX) {
                FFGPU_CHECK(depth >= 2, FFGPU_EINVAL, "expression: binary opcode %d on a stack of %d", op, depth);
                --depth;
            } else {
                FFGPU_CHECK(op >= FFGPU_OP_NEG && op <= FFGPU_OP_ATAN, FFGPU_EINVAL, "expression: unknown opcode %d", op);
                FFGPU_CHECK(depth >= 1, FFGPU_EINVAL, "expression: unary opcode %d on an empty stack", op);
            }
            FFGPU_CHECK(depth <= kExprStack, FFGPU_EINVAL, "expression: stack deeper than %d", kExprStack);
        }
        FFGPU_CHECK(depth == 1, FFGPU_EINVAL, "expression: the program leaves %d values", depth);
        FFGPU_CHECK(nconst == 0 || x->consts, FFGPU_EINVAL, "expression: constants missing");
        out.nops = x->nops;
        out.ops = in<int32_t>(iarr, x->ops, x->nops);
        out.consts = nconst ? in<double>(darr, x->consts, nconst) : nullptr;
        out.fe = nullptr;
        if (x->nfe) {
            std::vector<FeDev> h(x->nfe);
            for (int k = 0; k < x->nfe; ++k) {
                const ffgpu_fefunc &f = x->fe[k];
                h[k].kind = f.kind;
                h[k].dof = nullptr;
                size_t nval = 0;
                if (f.kind == FFGPU_FE_P0) nval = S->nt;
                else if (f.kind == FFGPU_FE_P1) nval = S->nv;
                else {
                    FFGPU_CHECK(f.kind == FFGPU_FE_P2, FFGPU_EINVAL, "expression: FE function kind %d", f.kind);
                    const int n2 = S->dim == 2 ? 6 : 10;
                    if (f.dof) {
                        h[k].dof = in<int32_t>(iarr, f.dof, (size_t)S->nt * n2);
                        FFGPU_TRY(err);
                        // the number of values is the largest DOF + 1
                        int mx = 0;
                        FFGPU_TRY(device_max_i32(ctx, h[k].dof, S->nt * n2, &mx));
                        nval = (size_t)mx + 1;
                    } else {
                        FFGPU_CHECK(S->fe == FFGPU_FE_P2, FFGPU_EINVAL,
                                    "expression: a P2 function without its DOF table needs a P2 space");
                        nval = S->ndof;
                    }
                }
                FFGPU_CHECK(f.values, FFGPU_EINVAL, "expression: FE function %d has no values", k);
                h[k].values = in<double>(darr, f.values, nval);
            }
            FeDev *d = nullptr;
            FFGPU_CUDA(dalloc(ctx, (void **)&d, sizeof(FeDev) * x->nfe));
            fe_dev.push_back(d);
            // pageable source: the call returns once h has been staged
            FFGPU_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(FeDev) * x->nfe, cudaMemcpyHostToDevice, ctx->stream));
            out.fe = d;
        }
        return err;
    }
};

static int frame_args(ffgpu_space *S, const ffgpu_varf *v, const double *geo, ExprUpload &U, TermArgs &A,
                      const char *what) {
    FFGPU_CHECK(v->nqp > 0 && v->nqp <= 64 && v->qp_lambda && v->qp_weight, FFGPU_EINVAL,
                "%s: the rule (1..64 points with coordinates and weights) is needed (nqp %d)", what, v->nqp);
    memset(&A, 0, sizeof(A));
    A.nt = S->nt;
    A.nqp = v->nqp;
    A.lam = U.in<double>(U.darr, v->qp_lambda, (size_t)v->nqp * (S->dim + 1));
    A.w = U.in<double>(U.darr, v->qp_weight, v->nqp);
    A.geo = geo;
    A.coords = S->coords;
    A.elems = S->elems;
    A.snodes = S->nodes;
    A.snn = S->nn;
    return U.err;
}

int terms_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **tloc) {
    *tloc = nullptr;
    if (!v || v->nterms <= 0) return FFGPU_OK;
    FFGPU_CHECK(v->terms && v->nterms <= kMaxTerms, FFGPU_EINVAL, "varf terms: 1..%d terms expected", kMaxTerms);
    FFGPU_CHECK(v->form == FFGPU_FORM_DIFFUSION && S->bs == 1, FFGPU_EINVAL,
                "varf terms: scalar spaces (diffusion form) only");
    ffgpu_ctx *ctx = S->ctx;
    ExprUpload U(ctx);
    TermArgs A;
    FFGPU_TRY(frame_args(S, v, geo, U, A, "varf terms"));
    A.nterms = v->nterms;
    int nex = 0;
    for (int k = 0; k < v->nterms; ++k) {
        const ffgpu_term &t = v->terms[k];
        FFGPU_CHECK(t.iop >= 0 && t.iop <= S->dim && t.jop >= 0 && t.jop <= S->dim, FFGPU_EINVAL,
                    "varf term %d: operators (%d, %d) not in 0..%d", k, t.iop, t.jop, S->dim);
        A.t[k].iop = t.iop;
        A.t[k].jop = t.jop;
        A.t[k].c = t.c;
        A.t[k].expr = -1;
        if (t.expr) {
            FFGPU_TRY(U.add(t.expr, S, A.ex[nex]));
            A.t[k].expr = nex++;
        }
    }
    FFGPU_CUDA(dalloc(ctx, (void **)tloc, sizeof(double) * (size_t)S->nt * S->nn * S->nn));
    A.out = *tloc;
    void (*k)(TermArgs) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = terms_kernel<2, 3>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = terms_kernel<3, 4>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = terms_kernel<2, 6>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = terms_kernel<3, 10>;
    if (!k) { dfree(ctx, *tloc); *tloc = nullptr; }
    FFGPU_CHECK(k, FFGPU_EINVAL, "varf terms: unsupported element");
    const int64_t nthr = (int64_t)S->nt * S->nn;
    k<<<(int)((nthr + kExprThreads - 1) / kExprThreads), kExprThreads, 0, ctx->stream>>>(A);
    // the uploads are freed in stream order after the kernel (DevIn, cudaFreeAsync)
    const int rc = launch_check(ctx, "terms");
    if (rc) { dfree(ctx, *tloc); *tloc = nullptr; }
    return rc;
}

int source_expr_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **fint) {
    *fint = nullptr;
    if (!v || !v->f_expr) return FFGPU_OK;
    ffgpu_ctx *ctx = S->ctx;
    ExprUpload U(ctx);
    TermArgs A;
    FFGPU_TRY(frame_args(S, v, geo, U, A, "source expression"));
    for (int c = 0; c < S->bs; ++c) FFGPU_TRY(U.add(&v->f_expr[c], S, A.ex[c]));
    FFGPU_CUDA(dalloc(ctx, (void **)fint, sizeof(double) * (size_t)S->nt * S->nn * S->bs));
    A.out = *fint;
    void (*k)(TermArgs) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = source_expr_kernel<2, 3, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = source_expr_kernel<3, 4, 1>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = source_expr_kernel<2, 6, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = source_expr_kernel<3, 10, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2VEC3) k = source_expr_kernel<3, 10, 3>;
    if (!k) { dfree(ctx, *fint); *fint = nullptr; }
    FFGPU_CHECK(k, FFGPU_EINVAL, "source expression: unsupported element");
    k<<<(int)((S->nt + kExprThreads - 1) / kExprThreads), kExprThreads, 0, ctx->stream>>>(A);
    const int rc = launch_check(ctx, "source_expr");
    if (rc) { dfree(ctx, *fint); *fint = nullptr; }
    return rc;
}

}  // namespace ffgpu
