// ffgpu_direct.cu -- sparse direct solvers on the device behind addsolver: Cholesky
// factorisation of a symmetric positive definite matrix (tgv rows included) and QR of any
// nonsingular one (the UMFPACK role), factored once per numeric state and reused by every
// solve, as FreeFEM's direct solvers are driven
// (VirtualSolver::factorize: fac_symbolic / fac_numeric, then dosolver, VirtualSolver.hpp:226-239;
// the CHOLMOD / MUMPS plugins, VirtualSolverSparseSuite.hpp:305, plugin/seq/MUMPS_seq.cpp:260-300).
//
//   symbolic (once per pattern): FreeFEM's sorted CSR to the host, a fill-reducing ordering
//     (nested dissection, METIS through cuSOLVER; approximate minimum degree if that fails),
//     P A P' built on the host, cuSOLVER's symbolic Cholesky analysis on the device;
//   numeric (once per numeric state): the permuted values gathered on the device, the numeric
//     factorisation, a zero-pivot check (not positive definite / singular: an error, as CHOLMOD
//     and UMFPACK report);
//   solve: b permuted on the device, the two triangular solves (QR: Q' b, then R), x unpermuted;
//   a transpose solve A' x = b (UMFPACK_At) uses the Cholesky factors of a symmetric matrix, and
//   for a nonsymmetric one a second QR, of P A' P' (same pattern, values gathered transposed),
//   built at the first transpose solve and refactored with A.
// QR is not invariant under row scaling: a tgv row (1e30 on its diagonal) would dominate the
// Householder reflections, so every row of P A P' is divided by its largest magnitude first
// (D P A P', with D P b on the right-hand side).
// The factorisation itself is cuSOLVER's (a library routine, like a GEMM from cuBLAS); the
// ordering, permutation and the plumbing around it are this file's.  cuSOLVER's sparse routines
// are opened when the direct solver is first used: a machine without them still loads
// libffgpu.so, and the direct solver then reports itself unavailable.
#include <cusolverSp.h>
#include <cusolverSp_LOWLEVEL_PREVIEW.h>
#include <cusparse.h>
#include <dlfcn.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include "ffgpu_internal.cuh"

#pragma nv_diag_suppress 1215
#pragma GCC diagnostic ignored "-Wdeprecated-declarations"

namespace ffgpu {

struct SolverLib {
    bool ok = false;
    std::string why;
    decltype(&cusolverSpCreate) Create;
    decltype(&cusolverSpDestroy) Destroy;
    decltype(&cusolverSpSetStream) SetStream;
    decltype(&cusolverSpXcsrmetisndHost) MetisNd;
    decltype(&cusolverSpXcsrsymamdHost) SymAmd;
    decltype(&cusolverSpCreateCsrcholInfo) CreateInfo;
    decltype(&cusolverSpDestroyCsrcholInfo) DestroyInfo;
    decltype(&cusolverSpXcsrcholAnalysis) Analysis;
    decltype(&cusolverSpDcsrcholBufferInfo) BufferInfo;
    decltype(&cusolverSpDcsrcholFactor) Factor;
    decltype(&cusolverSpDcsrcholZeroPivot) ZeroPivot;
    decltype(&cusolverSpDcsrcholSolve) Solve;
    // sparse QR (the nonsymmetric case); optional: without it only Cholesky is offered
    bool qr_ok = false;
    decltype(&cusolverSpCreateCsrqrInfo) QrCreateInfo;
    decltype(&cusolverSpDestroyCsrqrInfo) QrDestroyInfo;
    decltype(&cusolverSpXcsrqrAnalysis) QrAnalysis;
    decltype(&cusolverSpDcsrqrBufferInfo) QrBufferInfo;
    decltype(&cusolverSpDcsrqrSetup) QrSetup;
    decltype(&cusolverSpDcsrqrFactor) QrFactor;
    decltype(&cusolverSpDcsrqrZeroPivot) QrZeroPivot;
    decltype(&cusolverSpDcsrqrSolve) QrSolve;
    decltype(&cusparseCreateMatDescr) CreateDescr;
    decltype(&cusparseDestroyMatDescr) DestroyDescr;
    decltype(&cusparseSetMatType) SetType;
    decltype(&cusparseSetMatIndexBase) SetBase;
};

static void *open_first(const char *const *names) {
    for (int i = 0; names[i]; ++i)
        if (void *h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL)) return h;
    return nullptr;
}

static const SolverLib &solver_lib() {
    static SolverLib L;
    static std::once_flag once;
    std::call_once(once, [] {
        static const char *const sol[] = {"libcusolver.so.12", "libcusolver.so.11", "libcusolver.so", nullptr};
        static const char *const sp[] = {"libcusparse.so.12", "libcusparse.so.11", "libcusparse.so", nullptr};
        void *hs = open_first(sol), *hp = open_first(sp);
        if (!hs || !hp) { L.why = "cuSOLVER / cuSPARSE shared libraries not found"; return; }
        bool ok = true;
        auto get = [&](void *h, const char *name, auto &fn) {
            void *p = dlsym(h, name);
            if (!p) { ok = false; L.why = std::string("missing symbol ") + name; }
            fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(p);
        };
        get(hs, "cusolverSpCreate", L.Create);
        get(hs, "cusolverSpDestroy", L.Destroy);
        get(hs, "cusolverSpSetStream", L.SetStream);
        get(hs, "cusolverSpXcsrmetisndHost", L.MetisNd);
        get(hs, "cusolverSpXcsrsymamdHost", L.SymAmd);
        get(hs, "cusolverSpCreateCsrcholInfo", L.CreateInfo);
        get(hs, "cusolverSpDestroyCsrcholInfo", L.DestroyInfo);
        get(hs, "cusolverSpXcsrcholAnalysis", L.Analysis);
        get(hs, "cusolverSpDcsrcholBufferInfo", L.BufferInfo);
        get(hs, "cusolverSpDcsrcholFactor", L.Factor);
        get(hs, "cusolverSpDcsrcholZeroPivot", L.ZeroPivot);
        get(hs, "cusolverSpDcsrcholSolve", L.Solve);
        get(hp, "cusparseCreateMatDescr", L.CreateDescr);
        get(hp, "cusparseDestroyMatDescr", L.DestroyDescr);
        get(hp, "cusparseSetMatType", L.SetType);
        get(hp, "cusparseSetMatIndexBase", L.SetBase);
        L.ok = ok;
        const std::string why = L.why;
        get(hs, "cusolverSpCreateCsrqrInfo", L.QrCreateInfo);
        get(hs, "cusolverSpDestroyCsrqrInfo", L.QrDestroyInfo);
        get(hs, "cusolverSpXcsrqrAnalysis", L.QrAnalysis);
        get(hs, "cusolverSpDcsrqrBufferInfo", L.QrBufferInfo);
        get(hs, "cusolverSpDcsrqrSetup", L.QrSetup);
        get(hs, "cusolverSpDcsrqrFactor", L.QrFactor);
        get(hs, "cusolverSpDcsrqrZeroPivot", L.QrZeroPivot);
        get(hs, "cusolverSpDcsrqrSolve", L.QrSolve);
        L.qr_ok = L.ok && ok;
        if (L.ok) L.why = L.qr_ok ? why : "sparse QR symbols missing: " + L.why;
    });
    return L;
}

struct DirectState {
    int method = FFGPU_DIRECT_CHOLESKY;      // the factorisation in use (Cholesky or QR)
    cusolverSpHandle_t h = nullptr;
    cusparseMatDescr_t descr = nullptr;
    csrcholInfo_t info = nullptr;
    csrqrInfo_t qinfo = nullptr;
    double *rscale = nullptr;                // QR: 1 / largest magnitude of each row of P A P' (device)
    bool qr_factored = false;                // qinfo holds a factorisation (a refactor re-analyses)
    int n = 0;
    int64_t nnz = 0;
    int32_t *rp = nullptr, *col = nullptr;   // P A P' pattern (device)
    int32_t *src = nullptr;                  // value k of P A P' = exported value src[k] (device)
    int32_t *perm = nullptr;                 // new row k = old row perm[k] (device)
    double *val = nullptr, *exported = nullptr, *t1 = nullptr, *t2 = nullptr;
    void *buf = nullptr;
    bool factored = false;
    bool trans = false;                      // this state factors A' (its values gathered transposed)
    DirectState *tr = nullptr;               // QR of A' for transpose solves, built on demand
};

#define FFGPU_SOLVER(call)                                                                          \
    do {                                                                                             \
        cusolverStatus_t s_ = (call);                                                                \
        if (s_ != CUSOLVER_STATUS_SUCCESS) {                                                         \
            set_error("%s:%d %s: cuSOLVER status %d", __FILE__, __LINE__, #call, (int)s_);           \
            return FFGPU_ECUDA;                                                                      \
        }                                                                                            \
    } while (0)

__global__ void gather_kernel(int64_t n, const int32_t *__restrict__ idx, const double *__restrict__ src,
                              double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}
__global__ void scatter_kernel(int64_t n, const int32_t *__restrict__ idx, const double *__restrict__ src,
                               double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[idx[i]] = src[i];
}
// asymmetry of the stored values, one block row per thread: |a_rc - a_cr| above 1e-12 of
// sqrt(|a_rr a_cc|) anywhere -> flag.  Scaled by the diagonal, not by the entry: element
// integrals leave couplings that vanish in exact arithmetic (P2 vertex-vertex on right
// triangles) at rounding level, and those differ from their transposes by more than their size.
__global__ void symmetry_kernel(int nb, int bs, const int32_t *__restrict__ browptr,
                                const int32_t *__restrict__ bcol, const int32_t *__restrict__ diagpos,
                                const double *__restrict__ v, const double *__restrict__ vt, int *flag) {
    const int R = blockIdx.x * blockDim.x + threadIdx.x;
    if (R >= nb) return;
    const int b2 = bs * bs;
    const double *dR = v + (int64_t)diagpos[R] * b2;
    for (int32_t k = browptr[R]; k < browptr[R + 1]; ++k) {
        const int Cb = bcol[k];
        const double *dC = v + (int64_t)diagpos[Cb] * b2;
        for (int p = 0; p < bs; ++p)
            for (int q = 0; q < bs; ++q) {
                const int64_t i = (int64_t)k * b2 + p * bs + q;
                const double scale = sqrt(fabs(dR[p * bs + p]) * fabs(dC[q * bs + q]));
                if (fabs(v[i] - vt[i]) > 1e-12 * scale) atomicExch(flag, 1);
            }
    }
}

// QR's row equilibration: rs[k] = 1 / max_j |a_kj| of the permuted matrix, then a_kj *= rs[k]
__global__ void row_scale_kernel(int n, const int32_t *__restrict__ rp, double *__restrict__ val,
                                 double *__restrict__ rs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double m = 0.0;
    for (int j = rp[k]; j < rp[k + 1]; ++j) m = fmax(m, fabs(val[j]));
    const double r = m > 0.0 ? 1.0 / m : 1.0;
    rs[k] = r;
    for (int j = rp[k]; j < rp[k + 1]; ++j) val[j] *= r;
}
__global__ void scale_kernel(int64_t n, const double *__restrict__ rs, double *__restrict__ v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] *= rs[i];
}

static int grid_of(int64_t n) { return (int)((n + 255) / 256); }

void direct_invalidate(ffgpu_matrix *A) {
    if (DirectState *d = static_cast<DirectState *>(A->direct)) {
        d->factored = false;
        if (d->tr) d->tr->factored = false;
    }
}

static void free_state(ffgpu_ctx *ctx, DirectState *d) {
    if (!d) return;
    free_state(ctx, d->tr);
    const SolverLib &L = solver_lib();
    if (d->info) L.DestroyInfo(d->info);
    if (d->qinfo) L.QrDestroyInfo(d->qinfo);
    if (d->descr) L.DestroyDescr(d->descr);
    if (d->h) L.Destroy(d->h);
    dfree(ctx, d->rp); dfree(ctx, d->col); dfree(ctx, d->src); dfree(ctx, d->perm);
    dfree(ctx, d->val); dfree(ctx, d->exported); dfree(ctx, d->t1); dfree(ctx, d->t2);
    dfree(ctx, d->rscale);
    if (d->buf) cudaFree(d->buf);
    delete d;
}

void direct_release(ffgpu_matrix *A) {
    DirectState *d = static_cast<DirectState *>(A->direct);
    if (!d) return;
    cudaStreamSynchronize(A->ctx->stream);
    free_state(A->ctx, d);
    A->direct = nullptr;
}

// position of the transposed entry of each exported entry: entry j at (r, c) -> the entry at
// (c, r); false when the pattern is not structurally symmetric
static bool transpose_map(int n, const std::vector<int32_t> &rp, const std::vector<int32_t> &col,
                          std::vector<int32_t> &tmap) {
    tmap.resize(col.size());
    for (int r = 0; r < n; ++r)
        for (int j = rp[r]; j < rp[r + 1]; ++j) {
            const int c = col[j];
            const int32_t *b = col.data() + rp[c], *e = col.data() + rp[c + 1];
            const int32_t *f = std::lower_bound(b, e, r);
            if (f == e || *f != r) return false;
            tmap[j] = (int32_t)(f - col.data());
        }
    return true;
}

// symbolic phase: ordering, permuted pattern, cuSOLVER analysis
static int direct_symbolic(ffgpu_matrix *A, DirectState *d) {
    const SolverLib &L = solver_lib();
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    const int n = A->n;
    const int64_t nnz = A->nnz;
    FFGPU_CHECK(nnz < INT32_MAX, FFGPU_EINVAL, "direct solver: %lld nonzeros exceed 32-bit indices", (long long)nnz);
    d->n = n;
    d->nnz = nnz;
    std::vector<int32_t> rp(n + 1), col(nnz);
    std::vector<double> val(nnz);
    FFGPU_TRY(ffgpu_matrix_csr(A, rp.data(), col.data(), val.data()));
    FFGPU_SOLVER(L.Create(&d->h));
    FFGPU_SOLVER(L.SetStream(d->h, s));
    if (L.CreateDescr(&d->descr) != CUSPARSE_STATUS_SUCCESS) {
        set_error("direct solver: cusparseCreateMatDescr failed");
        return FFGPU_ECUDA;
    }
    L.SetType(d->descr, CUSPARSE_MATRIX_TYPE_GENERAL);
    L.SetBase(d->descr, CUSPARSE_INDEX_BASE_ZERO);
    // fill-reducing ordering: new row k = old row p[k]
    std::vector<int32_t> p(n);
    if (L.MetisNd(d->h, n, (int)nnz, d->descr, rp.data(), col.data(), nullptr, p.data()) != CUSOLVER_STATUS_SUCCESS)
        FFGPU_SOLVER(L.SymAmd(d->h, n, (int)nnz, d->descr, rp.data(), col.data(), p.data()));
    std::vector<int32_t> inv(n);
    for (int k = 0; k < n; ++k) inv[p[k]] = k;
    // A' has A's pattern (FreeFEM's patterns are structurally symmetric): the same permuted
    // pattern, each value taken from the transposed position
    std::vector<int32_t> tmap;
    FFGPU_CHECK(!d->trans || transpose_map(n, rp, col, tmap), FFGPU_EINVAL,
                "direct solver: a transpose solve needs a structurally symmetric pattern");
    // P A P': row k is old row p[k] with its columns renamed and sorted; src maps to the export
    std::vector<int32_t> brp(n + 1), bcol(nnz), src(nnz);
    brp[0] = 0;
    std::vector<std::pair<int32_t, int32_t>> row;
    for (int k = 0; k < n; ++k) {
        const int r = p[k];
        row.clear();
        for (int j = rp[r]; j < rp[r + 1]; ++j) row.emplace_back(inv[col[j]], d->trans ? tmap[j] : j);
        std::sort(row.begin(), row.end());
        int64_t o = brp[k];
        for (const auto &e : row) { bcol[o] = e.first; src[o] = e.second; ++o; }
        brp[k + 1] = (int32_t)o;
    }
    FFGPU_CUDA(dalloc(ctx, (void **)&d->rp, sizeof(int32_t) * (n + 1)));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->col, sizeof(int32_t) * nnz));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->src, sizeof(int32_t) * nnz));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->perm, sizeof(int32_t) * n));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->val, sizeof(double) * nnz));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->exported, sizeof(double) * nnz));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->t1, sizeof(double) * n));
    FFGPU_CUDA(dalloc(ctx, (void **)&d->t2, sizeof(double) * n));
    FFGPU_CUDA(cudaMemcpyAsync(d->rp, brp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s));
    FFGPU_CUDA(cudaMemcpyAsync(d->col, bcol.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s));
    FFGPU_CUDA(cudaMemcpyAsync(d->src, src.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s));
    FFGPU_CUDA(cudaMemcpyAsync(d->perm, p.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));   // the host vectors die here
    if (d->method == FFGPU_DIRECT_QR) {
        FFGPU_CUDA(dalloc(ctx, (void **)&d->rscale, sizeof(double) * n));
        FFGPU_SOLVER(L.QrCreateInfo(&d->qinfo));
        FFGPU_SOLVER(L.QrAnalysis(d->h, n, n, (int)nnz, d->descr, d->rp, d->col, d->qinfo));
        return FFGPU_OK;
    }
    FFGPU_SOLVER(L.CreateInfo(&d->info));
    FFGPU_SOLVER(L.Analysis(d->h, n, (int)nnz, d->descr, d->rp, d->col, d->info));
    return FFGPU_OK;
}

// numeric phase: the permuted values, the factorisation, the pivot check
static int direct_numeric(ffgpu_matrix *A, DirectState *d) {
    const SolverLib &L = solver_lib();
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    const int n = d->n;
    const int64_t nnz = d->nnz;
    // the exported CSR values (FreeFEM's sorted order) on the device, then P A P'
    std::vector<int32_t> rp(n + 1), col(nnz);
    FFGPU_TRY(ffgpu_matrix_csr(A, rp.data(), col.data(), d->exported));
    gather_kernel<<<grid_of(nnz), 256, 0, s>>>(nnz, d->src, d->exported, d->val);
    FFGPU_TRY(launch_check(ctx, "direct gather"));
    size_t internal = 0, work = 0;
    if (d->method == FFGPU_DIRECT_QR) {
        if (d->qr_factored) {
            // a factored csrqr info takes no second setup: a new numeric state starts from a new
            // analysis of the same pattern
            L.QrDestroyInfo(d->qinfo);
            d->qinfo = nullptr;
            FFGPU_SOLVER(L.QrCreateInfo(&d->qinfo));
            FFGPU_SOLVER(L.QrAnalysis(d->h, n, n, (int)nnz, d->descr, d->rp, d->col, d->qinfo));
        }
        row_scale_kernel<<<grid_of(n), 256, 0, s>>>(n, d->rp, d->val, d->rscale);
        FFGPU_TRY(launch_check(ctx, "direct row scale"));
        FFGPU_SOLVER(L.QrBufferInfo(d->h, n, n, (int)nnz, d->descr, d->val, d->rp, d->col, d->qinfo, &internal,
                                    &work));
        if (d->buf) { cudaFree(d->buf); d->buf = nullptr; }
        FFGPU_CUDA(cudaMalloc(&d->buf, std::max<size_t>(work, 256)));
        FFGPU_SOLVER(L.QrSetup(d->h, n, n, (int)nnz, d->descr, d->val, d->rp, d->col, 0.0, d->qinfo));
        // the factorisation also solves one system: a zero right-hand side on the scratch vectors
        FFGPU_CUDA(cudaMemsetAsync(d->t1, 0, sizeof(double) * n, s));
        FFGPU_SOLVER(L.QrFactor(d->h, n, n, (int)nnz, d->t1, d->t2, d->qinfo, d->buf));
        int pos = -1;
        FFGPU_SOLVER(L.QrZeroPivot(d->h, d->qinfo, 0.0, &pos));
        d->qr_factored = true;
        FFGPU_CHECK(pos < 0, FFGPU_EINVAL, "direct solver: the matrix is singular (zero pivot of R at column %d)",
                    pos);
        d->factored = true;
        return FFGPU_OK;
    }
    FFGPU_SOLVER(L.BufferInfo(d->h, n, (int)nnz, d->descr, d->val, d->rp, d->col, d->info, &internal, &work));
    if (d->buf) { cudaFree(d->buf); d->buf = nullptr; }
    FFGPU_CUDA(cudaMalloc(&d->buf, std::max<size_t>(work, 256)));
    FFGPU_SOLVER(L.Factor(d->h, n, (int)nnz, d->descr, d->val, d->rp, d->col, d->info, d->buf));
    int pivot = -1;
    FFGPU_SOLVER(L.ZeroPivot(d->h, d->info, 0.0, &pivot));
    FFGPU_CHECK(pivot < 0, FFGPU_EINVAL,
                "direct solver: the matrix is not positive definite (zero pivot at permuted row %d)", pivot);
    d->factored = true;
    return FFGPU_OK;
}

// the factorisation of A itself: the method is chosen at the first call (a symmetry test for
// AUTO), the symbolic phase runs once per pattern, the numeric phase once per numeric state
static int direct_prepare_own(ffgpu_matrix *A) {
    DirectState *d = static_cast<DirectState *>(A->direct);
    ffgpu_ctx *ctx = A->ctx;
    if (!d) {
        // Cholesky needs a symmetric matrix (tgv > 0 and tgv = -2 keep it so; -1 and -3 do not)
        int method = A->direct_method;
        if (method != FFGPU_DIRECT_QR) {
            FFGPU_TRY(matrix_prepare_transpose(A));
            int *flag = ctx->d_iscratch + 8;
            FFGPU_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
            symmetry_kernel<<<grid_of(A->nb), 256, 0, ctx->stream>>>(A->nb, A->bs, A->browptr, A->bcol,
                                                                    A->diagpos, A->val, A->val_t, flag);
            FFGPU_TRY(launch_check(ctx, "symmetry"));
            int hf = 0;
            FFGPU_CUDA(cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            FFGPU_CUDA(cudaStreamSynchronize(ctx->stream));
            FFGPU_CHECK(!hf || method == FFGPU_DIRECT_AUTO, FFGPU_EINVAL,
                        "direct solver: Cholesky needs a symmetric matrix");
            method = hf ? FFGPU_DIRECT_QR : FFGPU_DIRECT_CHOLESKY;
        }
        FFGPU_CHECK(method != FFGPU_DIRECT_QR || solver_lib().qr_ok, FFGPU_EINVAL,
                    "direct solver: sparse QR unavailable: %s", solver_lib().why.c_str());
        d = new DirectState();
        d->method = method;
        A->direct = d;
        const int rc = direct_symbolic(A, d);
        if (rc) { direct_release(A); return rc; }
    }
    const int rc = direct_numeric(A, d);
    if (rc) direct_release(A);
    return rc;
}

// the factorisation of A (trans 0) or A' (trans 1) behind the next solve; a symmetric matrix
// (Cholesky) answers both
static int direct_prepare(ffgpu_matrix *A, int trans, DirectState **out) {
    FFGPU_CHECK(solver_lib().ok, FFGPU_EINVAL, "direct solver unavailable: %s", solver_lib().why.c_str());
    DirectState *d = static_cast<DirectState *>(A->direct);
    if (!d || !d->factored) FFGPU_TRY(direct_prepare_own(A));
    d = static_cast<DirectState *>(A->direct);
    *out = d;
    if (!trans || d->method == FFGPU_DIRECT_CHOLESKY) return FFGPU_OK;
    DirectState *t = d->tr;
    if (t && t->factored) {
        *out = t;
        return FFGPU_OK;
    }
    if (!t) {
        t = new DirectState();
        t->method = FFGPU_DIRECT_QR;
        t->trans = true;
        d->tr = t;
        const int rc = direct_symbolic(A, t);
        if (rc) {
            d->tr = nullptr;
            cudaStreamSynchronize(A->ctx->stream);
            free_state(A->ctx, t);
            return rc;
        }
    }
    const int rc = direct_numeric(A, t);
    if (rc) {
        d->tr = nullptr;
        cudaStreamSynchronize(A->ctx->stream);
        free_state(A->ctx, t);
        return rc;
    }
    *out = t;
    return FFGPU_OK;
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_direct_method(ffgpu_matrix *A, int method) {
    FFGPU_CHECK(A, FFGPU_EINVAL, "ffgpu_direct_method: NULL matrix");
    FFGPU_CHECK(method == FFGPU_DIRECT_AUTO || method == FFGPU_DIRECT_CHOLESKY || method == FFGPU_DIRECT_QR,
                FFGPU_EINVAL, "ffgpu_direct_method: unknown method %d", method);
    if (A->direct_method != method) {
        FFGPU_CUDA(cudaSetDevice(A->ctx->device));
        direct_release(A);
        A->direct_method = method;
    }
    return FFGPU_OK;
}

int ffgpu_direct_factor(ffgpu_matrix *A) {
    FFGPU_CHECK(A, FFGPU_EINVAL, "ffgpu_direct_factor: NULL matrix");
    FFGPU_CUDA(cudaSetDevice(A->ctx->device));
    DirectState *d = nullptr;
    return direct_prepare(A, 0, &d);
}

int ffgpu_solve_direct_trans(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                             ffgpu_solver_stats *stats) {
    FFGPU_CHECK(A && b && x && nrhs >= 1, FFGPU_EINVAL, "ffgpu_solve_direct: bad argument");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DirectState *d = nullptr;
    FFGPU_TRY(direct_prepare(A, trans ? 1 : 0, &d));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    const SolverLib &L = solver_lib();
    const int64_t n = A->n;
    DevIn<double> bd(b, (size_t)n * nrhs, ctx);
    DevOut<double> xd(x, (size_t)n * nrhs, ctx, false);
    FFGPU_TRY(bd.err);
    FFGPU_TRY(xd.err);
    for (int k = 0; k < nrhs; ++k) {
        gather_kernel<<<grid_of(n), 256, 0, s>>>(n, d->perm, bd.d + k * n, d->t1);
        FFGPU_TRY(launch_check(ctx, "direct permute"));
        if (d->method == FFGPU_DIRECT_QR) {
            scale_kernel<<<grid_of(n), 256, 0, s>>>(n, d->rscale, d->t1);
            FFGPU_TRY(launch_check(ctx, "direct scale"));
            FFGPU_SOLVER(L.QrSolve(d->h, (int)n, (int)n, d->t1, d->t2, d->qinfo, d->buf));
        } else {
            FFGPU_SOLVER(L.Solve(d->h, (int)n, d->t1, d->t2, d->info, d->buf));
        }
        scatter_kernel<<<grid_of(n), 256, 0, s>>>(n, d->perm, d->t2, xd.d + k * n);
        FFGPU_TRY(launch_check(ctx, "direct unpermute"));
    }
    cudaEventRecord(e1, s);
    FFGPU_TRY(xd.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->converged = 1;
        stats->elapsed_ms = ms;
    }
    return FFGPU_OK;
}

int ffgpu_solve_direct(ffgpu_matrix *A, const double *b, double *x, int nrhs, ffgpu_solver_stats *stats) {
    return ffgpu_solve_direct_trans(A, b, x, nrhs, 0, stats);
}

}  // extern "C"
