// ffgpu_mixed.cu -- mixed precision: FP32 inner Jacobi-PCG inside an FP64 iterative
// refinement loop.
//
// FP64 stays where accuracy is decided: the element geometry and assembled values, the
// outer residual r = b - A x (FP64 SpMV on the FP64 matrix) and the update x += d.
// The inner solve of A d = r runs on an FP32 copy of the values with FP32 vectors, SpMV,
// Jacobi and dot products (FP32 accumulation), with the same three fused kernels and CUDA
// graph `while` loop as the FP64 CG.  The outer stopping test is FreeFEM's CG test on the
// true residual: (r, C r) < eps^2 (r0, C r0) with C the FP64 Jacobi preconditioner, so a
// result "to 1e-10" means the same thing as for the plain FP64 CG (CG.cpp:226,247).
// tgv rows (A_ii = 1e30) stay in the FP32 system: 1e30 and 1/tgv are normal FP32 numbers,
// and the corrections on those rows are of order r_i/tgv, also representable.
#include <math.h>
#include <string.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

constexpr int kMxWarps = 8;
constexpr int kMxSpmvBlocks = 16 * kNumSM;
constexpr int kMxVecBlocks = 4 * kNumSM;
constexpr int kMxThreads = 256;

struct InnerScalars {
    float gcg, gcgp, eps2, rho, gamma, s_gh, s_hq, pad0;
    int iter, itmax, done, converged;
    unsigned int ticket;
    int pad1;
};

__device__ __forceinline__ float block_sum_f(float v, float *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    float t = 0;
    if (w == 0) {
        t = lane < nw ? sh[lane] : 0.0f;
        t = warp_sum(t);
    }
    __syncthreads();
    return t;
}

__device__ __forceinline__ bool last_block_f(float partial, float *part, unsigned *ticket, float *tot, float *sh) {
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = partial;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    float s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(part + i);
    s = block_sum_f(s, sh);
    if (threadIdx.x == 0) { *tot = s; *ticket = 0u; return true; }
    return false;
}

template <int T>
__device__ __forceinline__ float csr_row_f(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                           const float *__restrict__ val, const float *__restrict__ x, int r,
                                           int sub) {
    int b = __ldg(rp + r), e = __ldg(rp + r + 1);
    float s = 0;
    for (int k = b + sub; k < e; k += T) s = fmaf(__ldg(val + k), __ldg(x + __ldg(col + k)), s);
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

template <int T>
__device__ __forceinline__ void bsr3_row_f(const int32_t *__restrict__ brp, const int32_t *__restrict__ bcol,
                                           const float *__restrict__ val, const float *__restrict__ x, int a,
                                           int sub, float &y0, float &y1, float &y2) {
    int b = __ldg(brp + a), e = __ldg(brp + a + 1);
    float s0 = 0, s1 = 0, s2 = 0;
    for (int k = b + sub; k < e; k += T) {
        int c = __ldg(bcol + k);
        const float *v = val + (int64_t)k * 9;
        float x0 = __ldg(x + 3 * (int64_t)c), x1 = __ldg(x + 3 * (int64_t)c + 1), x2 = __ldg(x + 3 * (int64_t)c + 2);
        s0 = fmaf(__ldg(v + 0), x0, s0); s0 = fmaf(__ldg(v + 1), x1, s0); s0 = fmaf(__ldg(v + 2), x2, s0);
        s1 = fmaf(__ldg(v + 3), x0, s1); s1 = fmaf(__ldg(v + 4), x1, s1); s1 = fmaf(__ldg(v + 5), x2, s1);
        s2 = fmaf(__ldg(v + 6), x0, s2); s2 = fmaf(__ldg(v + 7), x1, s2); s2 = fmaf(__ldg(v + 8), x2, s2);
    }
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    y0 = s0; y1 = s1; y2 = s2;
}

struct Spmv32 {
    int nb, bs;
    const int32_t *rp, *col;
    const float *val;
    const int32_t *perm;
};

// inner K_a: q = A h (FP32) and (h,q) -> rho
template <int BS, int T>
__global__ void __launch_bounds__(kMxWarps * 32) ir_ka(Spmv32 A, const float *__restrict__ h, float *__restrict__ q,
                                                       InnerScalars *ks, float *part) {
    __shared__ float sh[32];
    if (ks->done) return;
    const int lane = threadIdx.x & 31;
    const int gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    float hq = 0;
    for (int base = 0; base < A.nb; base += gridDim.x * groups) {
        const int slot = base + g;
        const bool ok = slot < A.nb;
        const int a = ok ? __ldg(A.perm + slot) : 0;
        if (BS == 1) {
            float s = csr_row_f<T>(A.rp, A.col, A.val, h, a, ok ? sub : T);
            if (ok && sub == 0) { q[a] = s; hq = fmaf(h[a], s, hq); }
        } else {
            float y0, y1, y2;
            bsr3_row_f<T>(A.rp, A.col, A.val, h, a, ok ? sub : T, y0, y1, y2);
            if (ok && sub == 0) {
                int64_t i = 3 * (int64_t)a;
                q[i] = y0; q[i + 1] = y1; q[i + 2] = y2;
                hq = fmaf(h[i], y0, hq);
                hq = fmaf(h[i + 1], y1, hq);
                hq = fmaf(h[i + 2], y2, hq);
            }
        }
    }
    float tot;
    float p = block_sum_f(hq, sh);
    if (last_block_f(p, part, &ks->ticket, &tot, sh)) { ks->s_hq = tot; ks->rho = -ks->s_gh / tot; }
}

__global__ void __launch_bounds__(kMxThreads) ir_kb(int n, float *__restrict__ x, float *__restrict__ g,
                                                    const float *__restrict__ h, const float *__restrict__ q,
                                                    const float *__restrict__ dinv, InnerScalars *ks, float *part,
                                                    cudaGraphConditionalHandle cond) {
    __shared__ float sh[32];
    if (ks->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0);
        return;
    }
    const float rho = ks->rho;
    float s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fmaf(rho, h[i], x[i]);
        float gi = fmaf(rho, q[i], g[i]);
        g[i] = gi;
        s = fmaf(gi, dinv[i] * gi, s);
    }
    float tot;
    float p = block_sum_f(s, sh);
    if (last_block_f(p, part, &ks->ticket, &tot, sh)) {
        ks->gcgp = ks->gcg;
        ks->gcg = tot;
        ks->gamma = tot / ks->gcgp;
        ks->iter += 1;
        if (tot < ks->eps2) { ks->converged = 1; ks->done = 1; }
        else if (ks->iter >= ks->itmax || !(tot == tot)) ks->done = 1;
        if (ks->done) cudaGraphSetConditional(cond, 0);
    }
}

__global__ void __launch_bounds__(kMxThreads) ir_kc(int n, const float *__restrict__ g, float *__restrict__ h,
                                                    const float *__restrict__ dinv, InnerScalars *ks, float *part) {
    __shared__ float sh[32];
    if (ks->done) return;
    const float gamma = ks->gamma;
    float s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float gi = g[i];
        float hi = gamma * h[i] - dinv[i] * gi;
        h[i] = hi;
        s = fmaf(gi, hi, s);
    }
    float tot;
    float p = block_sum_f(s, sh);
    if (last_block_f(p, part, &ks->ticket, &tot, sh)) ks->s_gh = tot;
}

// Outer step (FP64): r = b - A x from y = A x; (r, C r); inner RHS in FP32; d = 0;
// inner init (d = 0: G = -r, gCg = (G, C G), H = -C G, (G,H)).
__global__ void __launch_bounds__(kMxThreads) ir_outer_kernel(int n, const double *__restrict__ b,
                                                              const double *__restrict__ y,
                                                              const double *__restrict__ dinv64,
                                                              const float *__restrict__ dinv32,
                                                              float *__restrict__ g, float *__restrict__ h,
                                                              float *__restrict__ d, double *part64,
                                                              unsigned *ticket, double *out3) {
    __shared__ double sh[32];
    __shared__ bool s_last;
    double s64 = 0, s32a = 0, s32b = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double r = b[i] - y[i];
        s64 = fma(r, dinv64[i] * r, s64);
        float gi = -(float)r;
        float zi = dinv32[i] * gi;
        g[i] = gi;
        h[i] = -zi;
        d[i] = 0.0f;
        s32a += (double)(gi * zi);
        s32b += (double)(gi * -zi);
    }
    // three totals through the last-block protocol
    double v[3] = {s64, s32a, s32b};
    for (int c = 0; c < 3; ++c) {
        double t = warp_sum(v[c]);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
        __syncthreads();
        if (threadIdx.x < 32) {
            double u = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            u = warp_sum(u);
            if (threadIdx.x == 0) part64[c * gridDim.x + blockIdx.x] = u;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int c = 0; c < 3; ++c) {
        double s = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(part64 + c * gridDim.x + i);
        double t = warp_sum(s);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
        __syncthreads();
        if (threadIdx.x < 32) {
            double u = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            u = warp_sum(u);
            if (threadIdx.x == 0) out3[c] = u;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

__global__ void ir_inner_init(InnerScalars *ks, const double *out3, float eps_in, int itmax) {
    float gcg = (float)out3[1];
    ks->gcg = gcg; ks->gcgp = gcg; ks->s_gh = (float)out3[2];
    ks->eps2 = eps_in * eps_in * gcg;
    ks->iter = 0; ks->itmax = itmax; ks->converged = 0; ks->done = gcg < 1e-30f ? 1 : 0;
    ks->ticket = 0u;
}

__global__ void ir_update_kernel(int n, double *__restrict__ x, const float *__restrict__ d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

__global__ void to_f32_kernel(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void x0_tgv_kernel(int n, double *x, const double *b, const uint8_t *wcl, double tgv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && wcl[i]) x[i] = b[i] / tgv;
}

template <int BS>
static void *ir_ka_fn(int T) {
    switch (T) {
        case 1: return (void *)ir_ka<BS, 1>;
        case 2: return (void *)ir_ka<BS, 2>;
        case 4: return (void *)ir_ka<BS, 4>;
        case 8: return (void *)ir_ka<BS, 8>;
        case 16: return (void *)ir_ka<BS, 16>;
        default: return (void *)ir_ka<BS, 32>;
    }
}

struct IRState {
    cudaGraphExec_t exec = nullptr;
    int unroll = 0;
    float *g = nullptr, *h = nullptr, *q = nullptr, *d = nullptr, *dinv = nullptr;
    InnerScalars *ks = nullptr;
    double *y = nullptr, *out3 = nullptr;
};

static int ir_lanes(const ffgpu_matrix *A) {
    if (A->csr_lanes > 0) return A->csr_lanes;
    double avg = (double)A->nnzb / (double)max(1, A->nb);
    if (A->bs == 3) return avg >= 24 ? 4 : 2;
    if (avg >= 24) return 8;
    if (avg >= 10) return 4;
    return 2;
}

static int ir_grid(const ffgpu_matrix *A, int T) {
    int groups = kMxWarps * (32 / T);
    return max(1, min(kMxSpmvBlocks, (A->nb + groups - 1) / groups));
}

static int ir_build_graph(ffgpu_matrix *A, IRState &S, int unroll) {
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    cudaGraph_t graph, body;
    FFGPU_CUDA(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle cond;
    FFGPU_CUDA(cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault));
    alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
    memset(cp_buf, 0, sizeof(cp_buf));
    cudaGraphNodeParams *cp = reinterpret_cast<cudaGraphNodeParams *>(cp_buf);
    cp->type = cudaGraphNodeTypeConditional;
    cp->conditional.handle = cond;
    cp->conditional.type = cudaGraphCondTypeWhile;
    cp->conditional.size = 1;
    cudaGraphNode_t node;
    FFGPU_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, cp));
    body = cp->conditional.phGraph_out[0];
    FFGPU_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int T = ir_lanes(A);
    Spmv32 sa{A->nb, A->bs, A->browptr, A->bcol, A->val32, A->rowperm};
    void *ka = A->bs == 3 ? ir_ka_fn<3>(T) : ir_ka_fn<1>(T);
    float *part = (float *)ctx->d_part;
    int n = A->n;
    for (int u = 0; u < unroll; ++u) {
        void *aa[] = {&sa, &S.h, &S.q, &S.ks, &part};
        cudaLaunchKernel(ka, ir_grid(A, T), kMxWarps * 32, aa, 0, s);
        ir_kb<<<kMxVecBlocks, kMxThreads, 0, s>>>(n, S.d, S.g, S.h, S.q, S.dinv, S.ks, part, cond);
        ir_kc<<<kMxVecBlocks, kMxThreads, 0, s>>>(n, S.g, S.h, S.dinv, S.ks, part);
    }
    cudaError_t e = cudaStreamEndCapture(s, &body);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&S.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error("mixed-precision graph: %s", cudaGetErrorString(e));
        S.exec = nullptr;
        return FFGPU_ECUDA;
    }
    S.unroll = unroll;
    return FFGPU_OK;
}

static void ir_free(IRState &S, cudaStream_t s) {
    if (S.exec) cudaGraphExecDestroy(S.exec);
    cudaFreeAsync(S.g, s);
    cudaFreeAsync(S.ks, s);
    cudaFreeAsync(S.y, s);
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_matrix_to_f32(ffgpu_matrix *A) {
    FFGPU_CHECK(A, FFGPU_EINVAL, "ffgpu_matrix_to_f32: NULL matrix");
    if (A->val32) return FFGPU_OK;
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    FFGPU_CUDA(cudaMalloc((void **)&A->val32, sizeof(float) * A->nnz));
    to_f32_kernel<<<kMxVecBlocks * 4, kMxThreads, 0, ctx->stream>>>(A->nnz, A->val, A->val32);
    return launch_check(ctx, "to_f32");
}

int ffgpu_solve_ir(ffgpu_matrix *A, const double *b, double *x, const ffgpu_ir_params *prm,
                   ffgpu_solver_stats *stats) {
    FFGPU_CHECK(A && b && x && prm, FFGPU_EINVAL, "ffgpu_solve_ir: NULL argument");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int n = A->n;
    FFGPU_TRY(matrix_prepare_solver(A));
    FFGPU_TRY(ffgpu_matrix_to_f32(A));
    DevIn<double> bd(b, n, s);
    DevOut<double> xd(x, n, s, true);
    FFGPU_TRY(bd.err);
    FFGPU_TRY(xd.err);
    IRState S;
    if (cudaMallocAsync((void **)&S.g, sizeof(float) * (size_t)n * 5, s) != cudaSuccess ||
        cudaMallocAsync((void **)&S.ks, sizeof(InnerScalars), s) != cudaSuccess ||
        cudaMallocAsync((void **)&S.y, sizeof(double) * ((size_t)n + 8), s) != cudaSuccess) {
        set_error("ffgpu_solve_ir: device allocation failed");
        ir_free(S, s);
        return FFGPU_ENOMEM;
    }
    S.h = S.g + n; S.q = S.g + 2 * (size_t)n; S.d = S.g + 3 * (size_t)n; S.dinv = S.g + 4 * (size_t)n;
    S.out3 = S.y + n;
    to_f32_kernel<<<kMxVecBlocks, kMxThreads, 0, s>>>(n, A->diag_inv, S.dinv);
    ctx->launches++;
    int unroll = prm->unroll > 0 ? prm->unroll : 8;
    int rc = ir_build_graph(A, S, unroll);
    if (rc) { ir_free(S, s); return rc; }
    const double tgv = prm->tgv > 0 ? prm->tgv : 1e30;
    const int itmax_in = prm->itmax_inner > 0 ? prm->itmax_inner : n;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 30;
    const double eps = prm->eps;
    const float eps_in = (float)(prm->eps_inner > 0 ? prm->eps_inner : 1e-5);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (A->ntgv > 0) {
        x0_tgv_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, xd.d, bd.d, A->wcl, tgv);
        ctx->launches++;
    }
    double eps2 = 0, gcg = 0, gcg0 = 0;
    int outer = 0, inner_total = 0, converged = 0;
    double *part64 = ctx->d_part;
    for (outer = 0; outer <= max_outer; ++outer) {
        if ((rc = spmv(A, xd.d, S.y, 0, s))) break;
        ir_outer_kernel<<<kMxVecBlocks, kMxThreads, 0, s>>>(n, bd.d, S.y, A->diag_inv, S.dinv, S.g, S.h, S.d,
                                                            part64, ctx->d_ticket, S.out3);
        ctx->launches++;
        double o3[3];
        cudaMemcpyAsync(o3, S.out3, sizeof(o3), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("ffgpu_solve_ir: %s", cudaGetErrorString(cudaGetLastError()));
            rc = FFGPU_ECUDA;
            break;
        }
        gcg = o3[0];
        if (outer == 0) {
            gcg0 = gcg;
            eps2 = eps > 0 ? eps * eps * gcg : eps * eps;
            if (gcg < 1e-30) { converged = 1; break; }
        }
        if (gcg < eps2) { converged = 1; break; }
        if (outer == max_outer) break;
        ir_inner_init<<<1, 1, 0, s>>>(S.ks, S.out3, eps_in, itmax_in);
        ctx->launches++;
        if (cudaGraphLaunch(S.exec, s) != cudaSuccess) { set_error("ffgpu_solve_ir: graph launch failed"); rc = FFGPU_ECUDA; break; }
        InnerScalars hk;
        cudaMemcpyAsync(&hk, S.ks, sizeof(hk), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        inner_total += hk.iter;
        int bodies = hk.iter == 0 ? 1 : (hk.iter + unroll - 1) / unroll;
        ctx->launches += (int64_t)bodies * 3 * unroll;
        ir_update_kernel<<<kMxVecBlocks, kMxThreads, 0, s>>>(n, xd.d, S.d);
        ctx->launches++;
    }
    cudaEventRecord(e1, s);
    cudaStreamSynchronize(s);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ir_free(S, s);
    if (rc) return rc;
    FFGPU_TRY(xd.finish(s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = inner_total;
        stats->outer_iterations = outer;
        stats->converged = converged;
        stats->gcg = gcg;
        stats->eps2 = eps2;
        stats->residual = gcg0 > 0 ? sqrt(gcg / gcg0) : 0.0;
        stats->elapsed_ms = ms;
    }
    if (!converged) {
        set_error("mixed-precision refinement did not reach eps after %d outer steps", outer);
        return FFGPU_ENOCONV;
    }
    return FFGPU_OK;
}

}  // extern "C"
