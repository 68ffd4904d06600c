// ffgpu_internal.cuh -- shared types and helpers of libffgpu (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>

#include "ffgpu.h"

namespace ffgpu {

constexpr int kWarp = 32;
constexpr int kNumSM = 152;          // GB300: 2 dies x 76 SMs
constexpr int kCandMax = 512;        // candidate neighbour nodes gathered per matrix row
constexpr int kRedBlocks = 4 * kNumSM;  // reduction partials of the fused vector kernels

void set_error(const char *fmt, ...);

#define FFGPU_CUDA(call)                                                               \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ffgpu::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                \
                             cudaGetErrorString(e_));                                  \
            return FFGPU_ECUDA;                                                        \
        }                                                                              \
    } while (0)

#define FFGPU_CHECK(cond, code, ...)                                                   \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            ffgpu::set_error(__VA_ARGS__);                                             \
            return (code);                                                             \
        }                                                                              \
    } while (0)

#define FFGPU_TRY(expr)                                                                \
    do {                                                                               \
        int r_ = (expr);                                                               \
        if (r_ != FFGPU_OK) return r_;                                                 \
    } while (0)

// Device-side status word: kernels record the first failure here instead of trapping.
enum DevStatus : int {
    kDevOk = 0,
    kDevCandOverflow = 1,   // more candidate neighbours than kCandMax
    kDevDegOverflow = 2,    // row degree above the smem capacity the launch was sized for
    kDevBadDofLayout = 3,   // [P2]^3 DOF table not of the form 3*node+c
    kDevBadIndex = 4,       // index out of range in an input table
    kDevNotFound = 5,       // column missing from a row (pattern inconsistency)
    kDevTimeout = 6,        // a bounded wait in a kernel ran out (tensor-core element kernel)
};

// Scalars of a running Krylov solve, kept in device memory so the iteration loop runs
// inside one CUDA graph without host round trips.
struct KrylovScalars {
    double gcg, gcgp, eps2, rho, gamma, s_gh, s_hq;
    double gcg0;
    int iter, itmax, done, converged;
    unsigned int ticket;   // last-block counter of the fused reductions
    int pad;
    // the two-kernel iteration's (G, C G) and iteration count, one slot per parity of its K_ca
    // launches: a launch reads the other slot and its block 0 writes its own
    struct FusedSlot {
        double gcg;
        int iter, first;
    } fs[2];
};

struct ffgpu_ctx_impl;
}  // namespace ffgpu

struct ffgpu_ctx {
    int device;
    cudaStream_t stream;
    cudaMemPool_t pool;         // the context's buffers: stream-ordered, kept mapped between objects
    int64_t launches;
    double *d_part;             // reduction partials [kRedBlocks * 4]
    int *d_status;              // DevStatus word
    unsigned int *d_ticket;     // last-block counters
    int *d_iscratch;            // small integer scratch (max reductions)
    // SpMV layout chosen by timing, per matrix shape (nb, nnzb, bs) and mode, kept for the
    // context's lifetime: every later matrix of a shape gets the same layout, however many
    // shapes the context has seen
    struct Tuned { int64_t nb, nnzb; int bs, lanes, mode; };
    std::vector<Tuned> tuned;
    // batched solver launch shape chosen by timing, per batch shape (problems, DOFs, nnz)
    struct BatchTuned { int64_t nprob, n, nnz; int cand; };
    std::vector<BatchTuned> btuned;
};

struct ffgpu_space {
    ffgpu_ctx *ctx;
    int dim, nvk, nv, nt, fe, nn, bs, ndofK, ndof, nnodes;
    double *coords;      // nv*dim
    int32_t *elems;      // nt*nvk
    int32_t *nodes;      // nt*nn  (scalar node of each local basis function)
    int32_t *inc_ptr;    // nnodes+1
    int32_t *inc_elem;   // node -> incident elements, ascending
    uint8_t *inc_loc;    // local index of the node in that element
    int max_inc;
    // boundary elements (for on(labels)): nbe x dim vertices, labels, vertex -> element CSR
    int nbe;
    int32_t *belems, *blabel, *bv_ptr, *bv_elem;
    uint8_t *vmark;       // scratch: vertex on a selected boundary element (nv)
    // adjacent element and its local edge/face of each boundary element (boundary terms)
    int32_t *bel_elem, *bel_face;
};

struct ffgpu_matrix {
    ffgpu_ctx *ctx;
    ffgpu_space *space;   // NULL for matrices uploaded from CSR
    int n, bs, nb;        // DOFs, block size, block rows
    int64_t nnzb, nnz;
    int max_deg;
    int32_t *browptr;     // nb+1
    int32_t *bcol;        // nnzb
    int32_t *diagpos;     // nb: index of the diagonal block of each block row
    int32_t *rowperm;     // nb: block rows by decreasing degree (stable), the SpMV's row order
    double *val;          // nnzb*bs*bs, each block row-major
    double *geo;          // per-element geometry cache (16 doubles per element)
    uint8_t *bcmask;      // on(labels) DOF mask computed on the device (ndof)
    // solver state (lazily allocated)
    double *diag_inv;     // Jacobi 1/A_ii (1 if tiny)
    uint8_t *wcl;         // tgv rows found by gettgv
    int ntgv;
    double tgv_found;
    double *vec;          // work vectors (8*n)
    double *val_t;        // transpose values (same pattern), built on demand
    float *val32;         // FP32 copy for the mixed-precision inner solve
    float2 *valx, *valx_t;  // exact hi/lo FP32 splits of val (and of val_t) for the double-float SpMV
    float2 *hx;           // split copy of the CG search vector
    ffgpu::KrylovScalars *ks;
    // cached CG graph
    cudaGraphExec_t cg_exec;
    int cg_unroll, cg_trans, cg_mode;
    int cg_kernels_init, cg_kernels_body;
    // tuning
    int csr_lanes;        // lanes per block row of the FP64 SpMV (tuned)
    int csr_lanes_x;      // lanes per block row of the double-float SpMV (tuned)
    int layout_pinned;    // the caller fixed the SpMV layout of the current solve
    int last_cluster;     // the last FP64 CG solve ran in one thread-block cluster
    void *direct;         // factorisation state of the direct solver (ffgpu_direct.cu), or NULL
    int direct_method;    // FFGPU_DIRECT_AUTO / _CHOLESKY / _QR
    // SELL-32 copy for the Krylov SpMVs: block rows sliced into chunks of 32 (one row per
    // lane), rows sorted by decreasing degree inside windows of 1024 rows, each chunk padded
    // to its longest row and stored slot-major so that a warp reads 32 consecutive entries.
    int nchunk;           // ceil(nb/32)
    int64_t nslot;        // slot rows (sum of the chunk lengths)
    int32_t *sperm;       // nchunk*32: block row of each lane (-1: padding lane)
    int32_t *slen;        // nchunk: slots of each chunk
    int32_t *soff;        // nchunk+1: first slot row of each chunk
    int32_t *scol;        // nslot*32 block columns (NULL when scol16 is used)
    int16_t *scol16;      // nslot*32 column - row, when bs == 1 and every |column - row| < 2^15
    double *sval, *sval_t;      // FP64 values of A and A^T, (slot row, entry, lane) order
    float2 *svalx, *svalx_t;    // double-float splits of the same
    float *sval32;              // FP32 values for the mixed-precision inner solve
    // per-grid partitions of the chunks over warps, balanced by slot count (nw+1 starts)
    int spart_nw[4];
    int32_t *spart[4];
    int sell32_kind;      // chunk assignment of the FP32 SELL SpMV (tuned): 64 ranges, 65 rotated
};

namespace ffgpu {

// -------------------------------------------------------------------- host helpers
bool is_device_ptr(const void *p);

// Buffers of spaces, matrices and solver state come from the context's memory pool in the order of
// its stream: rebuilding a matrix of the same size reuses mapped memory, with no device-wide
// synchronisation of cudaMalloc/cudaFree.  Every user of these buffers runs on ctx->stream.
inline cudaError_t dalloc(ffgpu_ctx *ctx, void **p, size_t bytes) {
    return cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream);
}
inline void dfree(ffgpu_ctx *ctx, void *p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

// A view of a caller array on the device: copies host data in on construction when needed.
template <typename T>
struct DevIn {
    const T *d = nullptr;
    T *owned = nullptr;
    int err = FFGPU_OK;
    ffgpu_ctx *ctx;
    DevIn(const T *p, size_t n, ffgpu_ctx *c) : ctx(c) {
        if (!p || n == 0) { d = nullptr; return; }
        if (is_device_ptr(p)) { d = p; return; }
        if (dalloc(ctx, (void **)&owned, n * sizeof(T)) != cudaSuccess) {
            set_error("device allocation of %zu bytes failed", n * sizeof(T));
            err = FFGPU_ENOMEM; owned = nullptr; return;
        }
        if (cudaMemcpyAsync(owned, p, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
            set_error("host to device copy failed"); err = FFGPU_ECUDA; return;
        }
        d = owned;
    }
    ~DevIn() { dfree(ctx, owned); }
};

// A device buffer standing in for a caller output array; copied back by finish().
template <typename T>
struct DevOut {
    T *user = nullptr, *d = nullptr;
    bool owned = false;
    size_t n = 0;
    int err = FFGPU_OK;
    ffgpu_ctx *ctx;
    DevOut(T *p, size_t nn, ffgpu_ctx *c, bool copy_in) : user(p), n(nn), ctx(c) {
        if (!p || n == 0) return;
        if (is_device_ptr(p)) { d = p; return; }
        owned = true;
        if (dalloc(ctx, (void **)&d, n * sizeof(T)) != cudaSuccess) {
            set_error("device allocation of %zu bytes failed", n * sizeof(T));
            err = FFGPU_ENOMEM; d = nullptr; return;
        }
        if (copy_in &&
            cudaMemcpyAsync(d, p, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
            set_error("host to device copy failed"); err = FFGPU_ECUDA;
        }
    }
    int finish() {
        if (owned && d) {
            if (cudaMemcpyAsync(user, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess) {
                set_error("device to host copy failed"); return FFGPU_ECUDA;
            }
            if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
                set_error("stream sync failed"); return FFGPU_ECUDA;
            }
        }
        return FFGPU_OK;
    }
    ~DevOut() { if (owned) dfree(ctx, d); }
};

int check_device_status(ffgpu_ctx *ctx, const char *where);
int launch_check(ffgpu_ctx *ctx, const char *what);
int device_scan_i32(ffgpu_ctx *ctx, const int32_t *in, int32_t *out, int n);  // exclusive, out[n]=total
// status kBadIndex when an element lists a vertex outside [0, nv) (ffgpu_assembly.cu)
__global__ void check_elems_kernel(const int32_t *elems, int64_t m, int nv, int *status);
int device_max_i32(ffgpu_ctx *ctx, const int32_t *in, int n, int *host_max);
// order[0..n): indices sorted by decreasing key (0 <= key <= maxkey), ties by increasing index
int device_order_by_key_desc(ffgpu_ctx *ctx, const int32_t *key, int n, int maxkey, int32_t *order);
// Boundary terms of a varf prepared for one assembly call (ffgpu_boundary.cu): for every node
// the (boundary element, local node) codes b*nn + il touching it, ascending, and per boundary
// element its element vector (nn*bs, component-major) and Robin element matrix (nn*nn).
constexpr int kGeoStride = 16;   // element geometry: doubles per element: meas, kappa, -, -, G[4][3]

struct BoundaryTerms {
    const int32_t *ptr = nullptr;    // nnodes + 1
    const int32_t *list = nullptr;
    const double *rhs = nullptr;     // NULL: no linear boundary term
    const double *mat = nullptr;     // NULL: no Robin term
    const int32_t *bel_elem = nullptr;
};
int boundary_prepare(ffgpu_space *S, const ffgpu_varf *v, bool want_rhs, bool want_mat, BoundaryTerms &bt);
void boundary_release(ffgpu_space *S, BoundaryTerms &bt);
// Element vectors of a source given at quadrature points (ffgpu_varf.f_qp), for the linear
// form: *fint = nt * nn * bs values |K| sum_q w_q f_q phi_i(lambda_q) ((e*nn + i)*bs + c), or
// NULL when the varf has none.  geo: the element geometry (measure first).
int source_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **fint);
// Element mass matrices of a coefficient given at quadrature points (ffgpu_varf.mass_qp):
// *mloc = nt * nn * nn values |K| sum_q w_q c_q phi_i phi_j ((e*nn + i)*nn + j), or NULL.
int mass_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **mloc);
// Element stiffness matrices of a coefficient given at quadrature points (ffgpu_varf.stiff_qp):
// *kloc = nt * nn * nn values |K| sum_q w_q k_q grad phi_i . grad phi_j, or NULL.
int stiff_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **kloc);
// General volume terms of a scalar varf (ffgpu_varf.terms, ffgpu_expr.cu): *tloc = nt * nn * nn
// element matrices |K| sum_q w_q sum_t c_t(x_q) op_i(phi_i) op_j(phi_j), or NULL when none.
int terms_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **tloc);
// Element vectors of a source given as expressions (ffgpu_varf.f_expr), as source_prepare.
int source_expr_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **fint);
// on(labels) DOF mask on the device (onbc: ndof bytes, device)
int space_bc_mask_device(ffgpu_space *S, int nlabels, const int32_t *labels, int comp_mask, uint8_t *onbc);

// SpMV layout cache of the context (0: shape not tuned yet)
int tuned_layout(const ffgpu_ctx *ctx, const ffgpu_matrix *A, int mode);
void tuned_store(ffgpu_ctx *ctx, const ffgpu_matrix *A, int mode, int code);
// Tuner rule: the first candidate (in the tuner's fixed order) whose time is within
// kTuneMargin of the fastest.  Candidates closer than the margin are treated as equal, so
// timing noise between runs rarely changes the choice (and with it the summation order).
constexpr float kTuneMargin = 0.03f;
int tuned_pick(const float *ms, int n);

// Work-vector slot stride: slots start on 512-byte boundaries (16-byte vector accesses).
inline int64_t vstride(int64_t n) { return (n + 63) & ~(int64_t)63; }

// SELL-32 layout of a matrix (see ffgpu_matrix): kinds of value arrays
enum SellKind { kSell64 = 0, kSell64T = 1, kSellX = 2, kSellXT = 3, kSell32 = 4 };
struct SellArgs {
    int nchunk;
    const int32_t *perm, *len, *off, *col;
    const int16_t *col16;
    const int32_t *part;   // chunks [part[w], part[w+1]) belong to warp w of the launch
};
int sell_prepare(ffgpu_matrix *A);               // structure (once per pattern)
// chunk ranges of the nw warps of a launch, equal slot counts (built once per nw)
int sell_partition(ffgpu_matrix *A, int nw, const int32_t **part);
int sell_values(ffgpu_matrix *A, int kind);      // value array of one kind (once per numeric state)
void sell_release_values(ffgpu_matrix *A);       // drop the value arrays (new numeric state)
// mean time of nrep launches of the FP32 K_a of the mixed solve (after a mixed solve)
int ir_time_ka(ffgpu_matrix *A, int nrep, float *ms);
void sell_release(ffgpu_matrix *A);              // drop everything (matrix destruction)
inline SellArgs sell_args(const ffgpu_matrix *A) {
    return SellArgs{A->nchunk, A->sperm, A->slen, A->soff, A->scol, A->scol16, nullptr};
}
// Persistent grid of a kernel: resident blocks per SM (occupancy calculator) x SMs
int resident_grid(const void *kernel, int threads, size_t smem = 0);
// the resident grid capped to `need` blocks: small problems get fewer, fuller blocks and a
// shorter cross-block reduction
int sized_grid(const void *kernel, int threads, int64_t need, size_t smem = 0);

// matrix-level operations shared by the solvers
int matrix_prepare_solver(ffgpu_matrix *A);
int matrix_prepare_transpose(ffgpu_matrix *A);
int matrix_prepare_split(ffgpu_matrix *A, int trans);
int spmv(ffgpu_matrix *A, const double *x, double *y, int trans, cudaStream_t s);
// The CG iteration loop of a small scalar system in one thread-block cluster (ffgpu_cluster.cu):
// whether it takes the matrix (a rule on sizes and the device, never on timings), and the run
// from the state cg_init leaves (x, g, h, Krylov scalars; x receives the solution).
bool cluster_cg_fits(ffgpu_matrix *A, int trans);
constexpr int kClusterRefused = 1;   // cluster_cg_run: the launch was refused, nothing ran
int cluster_cg_run(ffgpu_matrix *A, int trans, double *x, const double *g, const double *h, cudaStream_t s);
// the direct solver's factorisation: stale after a numeric change (the ordering and the
// symbolic analysis stay), freed with the matrix (ffgpu_direct.cu)
// P2 element matrices on the tensor cores (ffgpu_elemtc.cu): NULL *out when not applicable
int elem_tc_prepare(ffgpu_space *S, const double *geo, double lam, double mu, const double *lame, double **out);
void direct_invalidate(ffgpu_matrix *A);
void direct_release(ffgpu_matrix *A);
// solver=GMRES for one right-hand side (ffgpu_gmres.cu); b, x device pointers
int gmres_one(ffgpu_matrix *A, const double *b, double *x, int trans, const ffgpu_solver_params *prm,
              ffgpu_solver_stats *st);

// -------------------------------------------------------------------- device helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Programmatic dependent launch: wait until the grids this one depends on have completed and
// their writes are visible.  A no-op for a kernel launched without the programmatic attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic dependent launch allowed (pdl): the kernel may be scheduled while
// the previous kernel on the stream drains, and waits in griddep_wait() for its results; every
// kernel launched this way calls griddep_wait() before it reads anything.
static inline cudaError_t launch_ex(const void *fn, int grid, int block, void **args, size_t smem,
                                    cudaStream_t s, bool pdl) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// programmatic dependent launch between the Krylov loop kernels (FFGPU_PDL=0 turns it off)
static inline bool pdl_default() {
    const char *e = getenv("FFGPU_PDL");
    return !(e && e[0] == '0');
}

__device__ __forceinline__ void dev_fail(int *status, int code) {
    atomicCAS(status, 0, code);
}

}  // namespace ffgpu
