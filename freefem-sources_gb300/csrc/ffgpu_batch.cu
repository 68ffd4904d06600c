// ffgpu_batch.cu -- many independent small problems solved in one persistent launch.
//
// A batch is the disjoint union of nprob meshes: one FE space and one assembly pass give a
// block-diagonal matrix whose blocks are each problem's own FreeFEM matrix (problem p's DOFs
// are offset by voff[p]; its pattern and values are those of a lone assembly).  The solve is
// one persistent kernel: every CTA takes problems from a queue (largest first) and runs the
// whole mixed-precision solve of a problem -- FP64 outer refinement r = b - A x, FP32 inner
// Jacobi-PCG on A d = r -- with CTA barriers only (no grid-wide waits).  An inner iteration
// is two passes over the problem's rows and two CTA reductions: the SpMV forms the direction
// h = gamma h_old - C g where it reads it (two direction buffers alternate), and the update
// pass sums (g, Cg) and (g, h), from which (g, h_next) = gamma (g, h) - (g, Cg) follows.
// The launch sequence
// (FP32 values, Jacobi, queue reset, persistent solve) is captured in a CUDA graph.  The CTA
// size and lanes per SpMV row are picked by timing the candidates on the batch (autotune).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "ffgpu_internal.cuh"

#include <new>

extern "C" int ffgpu_matrix_to_f32(ffgpu_matrix *A);

namespace ffgpu {

struct BatchArgs {
    int nprob;
    const int32_t *order;      // problems sorted by decreasing size
    const int32_t *voff;       // nprob+1 DOF offsets
    const int32_t *rp, *col;   // CSR of the union (global column numbers)
    const uint16_t *col16;     // the same columns numbered within their problem (every problem
                               // below 65 536 DOFs): 2 bytes per entry instead of 4
    const double *val;
    const float *val32;
    const double *dinv;
    const float *dinv32;
    const uint8_t *wcl;
    const double *b;
    double *x;
    float *g, *h, *q, *d;      // FP32 work vectors (union length)
    float *h2;                 // second direction buffer (directions alternate between h and h2)
    double *r;                 // FP64 residual
    int *queue;
    int *iters, *outers, *conv;
    double *resid;
    double eps, tgv;
    float eps_in;
    int itmax_in, max_outer;
};

template <int NT>
__device__ __forceinline__ double cta_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (w == 0) {
        t = lane < NT / 32 ? sh[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

template <int NT>
__device__ __forceinline__ float cta_sum_f(float v, float *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    float t = 0;
    if (w == 0) {
        t = lane < NT / 32 ? sh[lane] : 0.0f;
        t = warp_sum(t);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

// column of entry k of a row of the problem starting at DOF r0
template <bool C16>
__device__ __forceinline__ int batch_col(const BatchArgs &B, int r0, int k) {
    return C16 ? r0 + (int)B.col16[k] : B.col[k];
}

// two CTA-wide sums with the barriers of one (each summed as cta_sum_f sums it)
template <int NT>
__device__ __forceinline__ float2 cta_sum2_f(float a, float b, float *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    __syncthreads();
    if (lane == 0) { sh[w] = a; sh[32 + w] = b; }
    __syncthreads();
    if (w == 0) {
        float ta = lane < NT / 32 ? sh[lane] : 0.0f, tb = lane < NT / 32 ? sh[32 + lane] : 0.0f;
        ta = warp_sum(ta);
        tb = warp_sum(tb);
        if (lane == 0) { sh[64] = ta; sh[65] = tb; }
    }
    __syncthreads();
    return make_float2(sh[64], sh[65]);
}

// rows [r0, r1) with T lanes per row: y = A x in FP64
template <int NT, int T, bool C16>
__device__ __forceinline__ void cta_spmv64(const BatchArgs &B, int r0, int r1, const double *x, double *y) {
    const int sub = threadIdx.x % T;
    for (int base = r0; base < r1; base += NT / T) {
        int i = base + threadIdx.x / T;
        int ii = i < r1 ? i : r0;
        int kb = B.rp[ii], ke = B.rp[ii + 1];
        double s = 0;
        for (int k = kb + sub; k < ke; k += T) s = fma(B.val[k], x[batch_col<C16>(B, r0, k)], s);
#pragma unroll
        for (int o = T / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (i < r1 && sub == 0) y[i] = s;
    }
}

// The direction of this iteration, h = gamma h_old - C g, formed where it is read (the
// previous iteration's direction update folded into this SpMV); every reader rounds it the same
// way.
__device__ __forceinline__ float batch_dir(const BatchArgs &B, const float *hold, float gamma, int j) {
    return fmaf(gamma, hold[j], -(B.dinv32[j] * B.g[j]));
}

// FP32 q = A h and (h, q) over the problem's rows [r0, r1), T lanes per row, with h formed from
// h_old, g and C at every gather (batch_dir) and written to hnew by each row's first lane.  A
// lane group takes four rows at a time (rows base + u G, G = NT / T) and issues their row
// bounds, columns, values and gathers together.
template <int NT, int T, bool C16>
__device__ __forceinline__ float cta_spmv32_dot(const BatchArgs &B, int r0, int r1, const float *hold,
                                                float gamma, float *hnew, float *y) {
    constexpr int G = NT / T;
    constexpr int U = 4;
    const int sub = threadIdx.x % T;
    float dot = 0;
    for (int base = r0; base < r1; base += G * U) {
        int kb[U], ke[U];
        float sacc[U];
        int len = 0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * G + threadIdx.x / T;
            const int ii = i < r1 ? i : r0;
            kb[u] = B.rp[ii];
            ke[u] = i < r1 ? B.rp[ii + 1] : kb[u];
            sacc[u] = 0.f;
            len = max(len, ke[u] - kb[u]);
        }
        for (int t = sub; t < len; t += T) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int k = kb[u] + t;
                if (k < ke[u]) sacc[u] = fmaf(B.val32[k], batch_dir(B, hold, gamma, batch_col<C16>(B, r0, k)), sacc[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            float sv = sacc[u];
#pragma unroll
            for (int o = T / 2; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
            const int i = base + u * G + threadIdx.x / T;
            if (i < r1 && sub == 0) {
                const float hi = batch_dir(B, hold, gamma, i);
                hnew[i] = hi;
                y[i] = sv;
                dot = fmaf(hi, sv, dot);
            }
        }
    }
    return dot;
}

// elements per thread whose loads the vector passes issue together
constexpr int kVb = 4;

template <int NT, int T, bool C16>
__global__ void __launch_bounds__(NT) batch_ir_kernel(BatchArgs B) {
    __shared__ double sh[33];
    __shared__ float shf[66];
    __shared__ int s_p;
    for (;;) {
        if (threadIdx.x == 0) s_p = atomicAdd(B.queue, 1);
        __syncthreads();
        const int slot = s_p;
        __syncthreads();
        if (slot >= B.nprob) return;
        const int p = B.order[slot];
        const int r0 = B.voff[p], r1 = B.voff[p + 1];
        // x0 = b / tgv on tgv rows (SolverCG::dosolver), x = 0 elsewhere
        for (int i = r0 + threadIdx.x; i < r1; i += NT) B.x[i] = B.wcl[i] ? B.b[i] / B.tgv : 0.0;
        __syncthreads();
        double eps2 = 0, gcg = 0, gcg0 = 0;
        int outer = 0, inner = 0, conv = 0;
        for (outer = 0; outer <= B.max_outer; ++outer) {
            cta_spmv64<NT, T, C16>(B, r0, r1, B.x, B.r);
            __syncthreads();
            double s64 = 0;
            float sa = 0;
            for (int i = r0 + threadIdx.x; i < r1; i += NT) {
                double ri = B.b[i] - B.r[i];
                s64 = fma(ri, B.dinv[i] * ri, s64);
                float gi = -(float)ri, zi = B.dinv32[i] * gi;
                B.g[i] = gi; B.h[i] = 0.0f; B.d[i] = 0.0f;   // first direction -C g: gamma 0
                sa = fmaf(gi, zi, sa);
            }
            gcg = cta_sum<NT>(s64, sh);
            if (outer == 0) {
                gcg0 = gcg;
                eps2 = B.eps > 0 ? B.eps * B.eps * gcg : B.eps * B.eps;
                if (gcg < 1e-30) { conv = 1; break; }
            }
            if (gcg < eps2) { conv = 1; break; }
            if (outer == B.max_outer) break;
            float ig = cta_sum_f<NT>(sa, shf);
            float s_gh = -ig, gamma = 0.0f;
            float *hold = B.h, *hnew = B.h2;
            const float ieps2 = B.eps_in * B.eps_in * ig;
            for (int it = 0; it < B.itmax_in && ig >= 1e-30f && ig >= ieps2; ++it) {
                float hq = cta_spmv32_dot<NT, T, C16>(B, r0, r1, hold, gamma, hnew, B.q);
                hq = cta_sum_f<NT>(hq, shf);
                const float rho = -s_gh / hq;
                // a thread's elements i, i + NT, ... are taken kVb at a time, their loads issued
                // before the first store (the stores could alias the next loads otherwise); the
                // sums keep the element order
                float sg = 0, sgh = 0;
                for (int i0 = r0 + threadIdx.x; i0 < r1; i0 += kVb * NT) {
                    float hv[kVb], qv[kVb], dv[kVb], gv[kVb], cv[kVb];
#pragma unroll
                    for (int u = 0; u < kVb; ++u) {
                        const int i = i0 + u * NT;
                        if (i < r1) { hv[u] = hnew[i]; qv[u] = B.q[i]; dv[u] = B.d[i]; gv[u] = B.g[i]; cv[u] = B.dinv32[i]; }
                    }
#pragma unroll
                    for (int u = 0; u < kVb; ++u) {
                        const int i = i0 + u * NT;
                        if (i < r1) {
                            B.d[i] = fmaf(rho, hv[u], dv[u]);
                            float gi = fmaf(rho, qv[u], gv[u]);
                            B.g[i] = gi;
                            sg = fmaf(gi, cv[u] * gi, sg);
                            sgh = fmaf(gi, hv[u], sgh);
                        }
                    }
                }
                // (g, Cg) and (g, h): the next direction's (g, gamma h - Cg) follows from them
                const float2 t = cta_sum2_f<NT>(sg, sgh, shf);
                gamma = t.x / ig;
                ig = t.x;
                s_gh = fmaf(gamma, t.y, -t.x);
                float *tmp = hold; hold = hnew; hnew = tmp;
                ++inner;
                if (!(ig == ig)) break;
            }
            for (int i = r0 + threadIdx.x; i < r1; i += NT) B.x[i] += (double)B.d[i];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            B.iters[p] = inner;
            B.outers[p] = outer;
            B.conv[p] = conv;
            B.resid[p] = gcg0 > 0 ? sqrt(gcg / gcg0) : 0.0;
        }
        __syncthreads();
    }
}

__global__ void f32_copy_kernel(int64_t n, const double *a, float *b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void reset_queue_kernel(int *q) { *q = 0; }

// union mesh: element k of problem p (toff[p] <= k < toff[p + 1]) gets its vertex numbers
// offset by voff[p]; a vertex number outside [0, nv_p) records the lowest such problem in *bad
__global__ void union_elems_kernel(int nt, int nprob, const int32_t *__restrict__ toff,
                                   const int32_t *__restrict__ voff, int32_t *__restrict__ el, int *bad) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
        int lo = 0, hi = nprob;   // toff[lo] <= k < toff[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (toff[mid] <= k) lo = mid; else hi = mid;
        }
        const int v0 = voff[lo], nvp = voff[lo + 1] - v0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int v = el[3 * (int64_t)k + c];
            if (v < 0 || v >= nvp) atomicMin(bad, lo);
            el[3 * (int64_t)k + c] = v + v0;
        }
    }
}

// problem-local column numbers: row i belongs to the problem p with voff[p] <= i < voff[p + 1]
__global__ void local_col_kernel(int n, int nprob, const int32_t *__restrict__ voff,
                                 const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                 uint16_t *__restrict__ col16) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = nprob;   // voff[lo] <= i < voff[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (voff[mid] <= i) lo = mid; else hi = mid;
        }
        const int r0 = voff[lo];
        for (int k = rp[i]; k < rp[i + 1]; ++k) col16[k] = (uint16_t)(col[k] - r0);
    }
}

typedef void (*BatchKernel)(BatchArgs);

struct Candidate {
    BatchKernel k;
    int nt, lanes, per_sm;
};

}  // namespace ffgpu

using namespace ffgpu;

struct ffgpu_batch {
    ffgpu_ctx *ctx;
    int nprob;
    std::vector<int32_t> voff_h;
    ffgpu_space *space;
    ffgpu_matrix *A;
    double *b;
    int32_t *voff, *order;
    float *work32;
    double *r;
    float *dinv32;
    int *queue, *iters, *outers, *conv;
    double *resid;
    uint16_t *col16;    // problem-local columns (null when a problem has 65 536 DOFs or more)
    bool local16;       // every problem below 65 536 DOFs: the 16-bit column kernels
    int tuned;          // index of the chosen candidate, -1 before tuning
    cudaGraphExec_t exec;
    BatchArgs args;
    float tuned_ms;
};

// tuner candidates: the first kBatchSet with 32-bit global columns, the next kBatchSet with
// 16-bit problem-local columns (the same shapes)
#define FFGPU_BATCH_SET(C16)                                                                          \
    {batch_ir_kernel<256, 2, C16>, 256, 2, 4}, {batch_ir_kernel<256, 4, C16>, 256, 4, 4},             \
        {batch_ir_kernel<512, 2, C16>, 512, 2, 2}, {batch_ir_kernel<512, 4, C16>, 512, 4, 2},         \
        {batch_ir_kernel<1024, 2, C16>, 1024, 2, 1}, {batch_ir_kernel<1024, 4, C16>, 1024, 4, 1},     \
        {batch_ir_kernel<128, 2, C16>, 128, 2, 8}
static Candidate g_cands[] = {FFGPU_BATCH_SET(false), FFGPU_BATCH_SET(true)};
#undef FFGPU_BATCH_SET
constexpr int kBatchSet = 7;
static_assert(sizeof(g_cands) / sizeof(g_cands[0]) == 2 * kBatchSet, "batched tuner: candidate sets");

static int batch_graph(ffgpu_batch *B, int cand) {
    ffgpu_ctx *ctx = B->ctx;
    cudaStream_t s = ctx->stream;
    if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
    const Candidate &c = g_cands[cand];
    int grid = kNumSM * c.per_sm;
    cudaGraph_t g;
    FFGPU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    reset_queue_kernel<<<1, 1, 0, s>>>(B->queue);
    void *args[] = {&B->args};
    cudaLaunchKernel((void *)c.k, grid, c.nt, args, 0, s);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B->exec, g, 0);
    if (e == cudaSuccess) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_error("batch graph: %s", cudaGetErrorString(e));
        B->exec = nullptr;
        return FFGPU_ECUDA;
    }
    return FFGPU_OK;
}

extern "C" {

static int batch_create(ffgpu_ctx *ctx, int nprob, const int32_t *nv, const int32_t *nt, const double *coords,
                        const int32_t *elems, ffgpu_batch **out);

int ffgpu_batch_create(ffgpu_ctx *ctx, int nprob, const int32_t *nv, const int32_t *nt, const double *coords,
                       const int32_t *elems, ffgpu_batch **out) {
    try {
        return batch_create(ctx, nprob, nv, nt, coords, elems, out);
    } catch (const std::bad_alloc &) {
        set_error("ffgpu_batch_create: out of host memory");
        return FFGPU_ENOMEM;
    }
}

static int batch_create(ffgpu_ctx *ctx, int nprob, const int32_t *nv, const int32_t *nt, const double *coords,
                        const int32_t *elems, ffgpu_batch **out) {
    FFGPU_CHECK(ctx && out && nv && nt && coords && elems && nprob > 0, FFGPU_EINVAL,
                "ffgpu_batch_create: bad argument");
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    // per-problem first vertex and first element of the union (nprob + 1 entries each)
    std::vector<int32_t> voff(nprob + 1, 0), toff(nprob + 1, 0);
    for (int p = 0; p < nprob; ++p) {
        FFGPU_CHECK(nv[p] > 0 && nt[p] > 0, FFGPU_EINVAL, "problem %d is empty", p);
        voff[p + 1] = voff[p] + nv[p];
        toff[p + 1] = toff[p] + nt[p];
    }
    const int NV = voff[nprob], NT = toff[nprob];
    // the union's element array on the device: the caller's elements (host or device) copied in,
    // then every vertex number offset by its problem's first vertex and range-checked there
    cudaStream_t s = ctx->stream;
    int32_t *d_el = nullptr, *d_off = nullptr;
    FFGPU_CUDA(dalloc(ctx, (void **)&d_el, sizeof(int32_t) * (size_t)3 * NT));
    if (dalloc(ctx, (void **)&d_off, sizeof(int32_t) * (2 * (size_t)(nprob + 1) + 1))) {
        dfree(ctx, d_el);
        set_error("ffgpu_batch_create: device allocation failed");
        return FFGPU_ENOMEM;
    }
    int32_t *d_toff = d_off, *d_voff = d_off + nprob + 1, *d_bad = d_off + 2 * (nprob + 1);
    const int nobad = nprob;
    int bad = nprob;
    cudaError_t ce = cudaMemcpyAsync(d_el, elems, sizeof(int32_t) * (size_t)3 * NT, cudaMemcpyDefault, s);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(d_toff, toff.data(), sizeof(int32_t) * (nprob + 1), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(d_voff, voff.data(), sizeof(int32_t) * (nprob + 1), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_bad, &nobad, sizeof(int), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) {
        union_elems_kernel<<<4 * kNumSM, 256, 0, s>>>(NT, nprob, d_toff, d_voff, d_el, d_bad);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    dfree(ctx, d_off);
    if (ce != cudaSuccess || bad < nprob) {
        dfree(ctx, d_el);
        if (ce != cudaSuccess) {
            set_error("ffgpu_batch_create: %s", cudaGetErrorString(ce));
            return FFGPU_ECUDA;
        }
        set_error("problem %d: vertex index out of range", bad);
        return FFGPU_EINVAL;
    }
    ffgpu_batch *B = new ffgpu_batch();
    B->ctx = ctx; B->nprob = nprob; B->voff_h = voff; B->space = nullptr; B->A = nullptr; B->tuned = -1;
    B->exec = nullptr; B->b = nullptr; B->work32 = nullptr; B->r = nullptr; B->dinv32 = nullptr;
    B->col16 = nullptr;
    B->local16 = *std::max_element(nv, nv + nprob) < 65536;
    // P1: the DOFs are the vertices (no DOF table)
    int rc = ffgpu_space_create(ctx, 2, NV, coords, NT, d_el, FFGPU_FE_P1, 3, nullptr, NV, &B->space);
    dfree(ctx, d_el);
    if (rc) { delete B; return rc; }
    std::vector<int32_t> order(nprob);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nv[a] > nv[b]; });
    if (cudaMalloc((void **)&B->voff, sizeof(int32_t) * (nprob + 1)) ||
        cudaMalloc((void **)&B->order, sizeof(int32_t) * nprob) ||
        cudaMalloc((void **)&B->queue, sizeof(int) * 4) ||
        cudaMalloc((void **)&B->iters, sizeof(int) * nprob) || cudaMalloc((void **)&B->outers, sizeof(int) * nprob) ||
        cudaMalloc((void **)&B->conv, sizeof(int) * nprob) || cudaMalloc((void **)&B->resid, sizeof(double) * nprob) ||
        cudaMalloc((void **)&B->b, sizeof(double) * NV) || cudaMalloc((void **)&B->r, sizeof(double) * NV) ||
        cudaMalloc((void **)&B->work32, sizeof(float) * (size_t)NV * 6)) {
        set_error("ffgpu_batch_create: device allocation failed");
        ffgpu_space_destroy(B->space);
        delete B;
        return FFGPU_ENOMEM;
    }
    B->dinv32 = B->work32 + (size_t)4 * NV;
    cudaMemcpy(B->voff, voff.data(), sizeof(int32_t) * (nprob + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(B->order, order.data(), sizeof(int32_t) * nprob, cudaMemcpyHostToDevice);
    *out = B;
    return FFGPU_OK;
}

int ffgpu_batch_assemble(ffgpu_batch *B, const double *kappa, double f, const uint8_t *onbc, double tgv) {
    FFGPU_CHECK(B, FFGPU_EINVAL, "ffgpu_batch_assemble: NULL batch");
    ffgpu_varf v;
    memset(&v, 0, sizeof(v));
    v.form = FFGPU_FORM_DIFFUSION;
    v.kappa = kappa;
    v.c_stiff = 1.0;
    v.f_const[0] = f;
    ffgpu_bc bc = {onbc, nullptr, tgv};
    if (!B->A) {
        FFGPU_TRY(ffgpu_matrix_assemble(B->space, &v, &bc, B->b, &B->A));
    } else {
        FFGPU_TRY(ffgpu_matrix_reassemble(B->A, &v, &bc, B->b));
    }
    ffgpu_matrix *A = B->A;
    FFGPU_TRY(matrix_prepare_solver(A));
    FFGPU_TRY(ffgpu_matrix_to_f32(A));
    cudaStream_t s = B->ctx->stream;
    if (B->local16 && !B->col16) {
        // the pattern is fixed by the first assembly: number its columns within their problems
        FFGPU_CUDA(dalloc(B->ctx, (void **)&B->col16, sizeof(uint16_t) * std::max<int64_t>(A->nnz, 1)));
        local_col_kernel<<<4 * kNumSM, 256, 0, s>>>(A->n, B->nprob, B->voff, A->browptr, A->bcol, B->col16);
        FFGPU_TRY(launch_check(B->ctx, "local_col"));
    }
    f32_copy_kernel<<<4 * kNumSM, 256, 0, s>>>(A->n, A->diag_inv, B->dinv32);
    FFGPU_TRY(launch_check(B->ctx, "f32_copy"));
    float *w = B->work32;
    size_t NV = A->n;
    B->args = BatchArgs{B->nprob, B->order, B->voff, A->browptr, A->bcol, B->col16, A->val, A->val32, A->diag_inv,
                        B->dinv32, A->wcl, B->b, nullptr, w, w + NV, w + 2 * NV, w + 3 * NV, w + 5 * NV, B->r, B->queue,
                        B->iters, B->outers, B->conv, B->resid, 1e-8, tgv > 0 ? tgv : 1e30, 1e-4f, 0, 30};
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

int ffgpu_batch_solve(ffgpu_batch *B, double *x, const ffgpu_ir_params *prm, int32_t *iterations,
                      ffgpu_solver_stats *stats) {
    FFGPU_CHECK(B && B->A && x && prm, FFGPU_EINVAL, "ffgpu_batch_solve: assemble the batch first");
    ffgpu_ctx *ctx = B->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int NV = B->A->n;
    DevOut<double> xd(x, NV, ctx, false);
    FFGPU_TRY(xd.err);
    BatchArgs &a = B->args;
    bool changed = a.x != xd.d || a.eps != prm->eps ||
                   a.eps_in != (float)(prm->eps_inner > 0 ? prm->eps_inner : 1e-4) ||
                   a.itmax_in != (prm->itmax_inner > 0 ? prm->itmax_inner : 100000) ||
                   a.max_outer != (prm->max_outer > 0 ? prm->max_outer : 30);
    a.x = xd.d;
    a.eps = prm->eps;
    a.eps_in = (float)(prm->eps_inner > 0 ? prm->eps_inner : 1e-4);
    a.itmax_in = prm->itmax_inner > 0 ? prm->itmax_inner : 100000;
    a.max_outer = prm->max_outer > 0 ? prm->max_outer : 30;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (B->tuned < 0)
        for (const ffgpu_ctx::BatchTuned &t : ctx->btuned)
            if (t.nprob == B->nprob && t.n == NV && t.nnz == B->A->nnz && (t.cand >= kBatchSet) == B->local16)
                B->tuned = t.cand;
    if (B->tuned < 0) {
        // autotune: time every candidate (CTA size x lanes per row) on this batch and keep the
        // first one within the tuner margin of the fastest; the choice is kept in the context
        // for later batches of the same shape
        const int base = B->local16 ? kBatchSet : 0;
        float tms[kBatchSet];
        for (int c = 0; c < kBatchSet; ++c) {
            FFGPU_TRY(batch_graph(B, base + c));
            cudaGraphLaunch(B->exec, s);   // warm
            cudaEventRecord(e0, s);
            cudaGraphLaunch(B->exec, s);
            cudaEventRecord(e1, s);
            FFGPU_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            ctx->launches += 4;
            tms[c] = ms;
            if (getenv("FFGPU_VERBOSE"))
                fprintf(stderr, "ffgpu: batch tuner <%d threads, %d lanes, %d CTAs>: %.3f ms\n", g_cands[base + c].nt,
                        g_cands[base + c].lanes, kNumSM * g_cands[base + c].per_sm, ms);
        }
        const int bi = base + tuned_pick(tms, kBatchSet);
        B->tuned = bi;
        B->tuned_ms = tms[bi - base];
        changed = true;
        ctx->btuned.push_back(ffgpu_ctx::BatchTuned{B->nprob, NV, B->A->nnz, bi});
    }
    if (changed || !B->exec) FFGPU_TRY(batch_graph(B, B->tuned));
    cudaEventRecord(e0, s);
    FFGPU_CUDA(cudaGraphLaunch(B->exec, s));
    cudaEventRecord(e1, s);
    ctx->launches += 2;
    FFGPU_TRY(xd.finish());
    FFGPU_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<int> it(B->nprob), ou(B->nprob), cv(B->nprob);
    cudaMemcpy(it.data(), B->iters, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost);
    cudaMemcpy(ou.data(), B->outers, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost);
    cudaMemcpy(cv.data(), B->conv, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost);
    if (iterations) memcpy(iterations, it.data(), sizeof(int) * B->nprob);
    int nconv = 0;
    long long tot = 0;
    int maxo = 0;
    for (int p = 0; p < B->nprob; ++p) { nconv += cv[p]; tot += it[p]; maxo = max(maxo, ou[p]); }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = (int)tot;
        stats->outer_iterations = maxo;
        stats->converged = nconv == B->nprob;
        stats->elapsed_ms = ms;
    }
    if (nconv != B->nprob) {
        set_error("batch: %d of %d problems did not converge", B->nprob - nconv, B->nprob);
        return FFGPU_ENOCONV;
    }
    return FFGPU_OK;
}

int ffgpu_batch_rhs(const ffgpu_batch *B, double *b) {
    FFGPU_CHECK(B && B->A && b, FFGPU_EINVAL, "ffgpu_batch_rhs: assemble first");
    FFGPU_CUDA(cudaMemcpy(b, B->b, sizeof(double) * B->A->n, cudaMemcpyDefault));
    return FFGPU_OK;
}

ffgpu_matrix *ffgpu_batch_matrix(const ffgpu_batch *B) { return B ? B->A : nullptr; }

int ffgpu_batch_info(const ffgpu_batch *B, int *cta_threads, int *lanes_per_row, float *tuned_ms) {
    FFGPU_CHECK(B, FFGPU_EINVAL, "ffgpu_batch_info: NULL batch");
    int c = B->tuned;
    if (cta_threads) *cta_threads = c >= 0 ? g_cands[c].nt : 0;
    if (lanes_per_row) *lanes_per_row = c >= 0 ? g_cands[c].lanes : 0;
    if (tuned_ms) *tuned_ms = c >= 0 ? B->tuned_ms : 0.0f;
    return FFGPU_OK;
}

int ffgpu_batch_destroy(ffgpu_batch *B) {
    if (!B) return FFGPU_OK;
    cudaStreamSynchronize(B->ctx->stream);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    ffgpu_matrix_destroy(B->A);
    ffgpu_space_destroy(B->space);
    cudaFree(B->voff); cudaFree(B->order); cudaFree(B->queue); cudaFree(B->iters); cudaFree(B->outers);
    cudaFree(B->conv); cudaFree(B->resid); cudaFree(B->b); cudaFree(B->r); cudaFree(B->work32);
    dfree(B->ctx, B->col16);
    delete B;
    return FFGPU_OK;
}

}  // extern "C"
