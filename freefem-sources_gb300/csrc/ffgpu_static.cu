// ffgpu_static.cu -- Jacobi-PCG that allocates nothing: its scratch lives in a fixed array.
//
// Who needs it: a caller that must not allocate device memory once it is running -- for
// example an application that hands the whole GPU to its own memory pool at start-up and
// then calls the solver from its time loop, where a cudaMalloc would fail or stall.  The
// regular entry points (ffgpu_solve_cg and friends) allocate their work vectors and the
// staging buffers for host arrays on first use; this one takes every array in device memory
// from the caller and keeps its own work vectors in the static array below.
//
// Limits and rules:
//   * at most kStaticMaxN = 524288 DOFs (the array holds four FP64 work vectors, the Jacobi
//     diagonal, the tgv-row mask and the reduction partials: about 17 MB, held by every GPU
//     that loads libffgpu.so until the process exits);
//   * the first call on a device (with that device current) looks up the array's device
//     address with cudaGetSymbolAddress and caches it;
//   * every call synchronises the caller's stream (it polls the convergence flag every 32
//     iterations and reads the result at the end), so no call can run under stream capture;
//   * every call shares the one array and leaves its last contents there; each call clears
//     the counters and scalars it needs before use.  Calls that overlap on the GPU (two host
//     threads, or two streams) race on the array: serialise them.
// The algorithm is the one of ffgpu_solve_cg (FreeFEM's ConjugueGradient, CG.cpp:196-265):
// same Jacobi preconditioner and tgv handling, same stopping rule, with the iteration loop
// driven from the host (three kernel launches per iteration, convergence polled every 32).
#include <mutex>
#include <string.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

constexpr int64_t kStaticMaxN = 524288;
constexpr int kStBlocks = 4 * kNumSM;       // vector kernels
constexpr int kStSpmvBlocks = 8 * kNumSM;   // SpMV kernel (8 warps each)
constexpr int kStThreads = 256;
constexpr int64_t kStPart = 4096;           // partial sums (>= 2 * max grid)
constexpr int kPollEvery = 32;

struct StaticScalars {
    double gcg, gcgp, eps2, rho, gamma, s_gh, s_hq, gcg0;
    unsigned long long maxbits, max1bits;
    int iter, itmax, done, converged, count;
    unsigned int ticket;
};

// layout of the array (byte offsets, 256-aligned sections)
constexpr size_t kOffG = 0;
constexpr size_t kOffH = kOffG + 8 * kStaticMaxN;
constexpr size_t kOffQ = kOffH + 8 * kStaticMaxN;
constexpr size_t kOffD = kOffQ + 8 * kStaticMaxN;
constexpr size_t kOffW = kOffD + 8 * kStaticMaxN;         // tgv-row mask (one byte per DOF)
constexpr size_t kOffP = kOffW + ((kStaticMaxN + 255) / 256) * 256;
constexpr size_t kOffS = kOffP + 8 * kStPart;
constexpr size_t kStaticBytes = kOffS + 256;

static __device__ __align__(256) unsigned char g_cg_scratch[kStaticBytes];

struct StaticView {
    double *g, *h, *q, *dinv, *part;
    uint8_t *wcl;
    StaticScalars *ks;
};

__host__ __device__ inline StaticView view_of(unsigned char *base) {
    StaticView v;
    v.g = (double *)(base + kOffG);
    v.h = (double *)(base + kOffH);
    v.q = (double *)(base + kOffQ);
    v.dinv = (double *)(base + kOffD);
    v.wcl = (uint8_t *)(base + kOffW);
    v.part = (double *)(base + kOffP);
    v.ks = (StaticScalars *)(base + kOffS);
    return v;
}

__device__ __forceinline__ double st_block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (w == 0) {
        t = lane < nw ? sh[lane] : 0.0;
        t = warp_sum(t);
    }
    __syncthreads();
    return t;
}

__device__ __forceinline__ bool st_last_block(double partial, double *part, unsigned *ticket, double *tot,
                                              double *sh) {
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
    double s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(part + i);
    s = st_block_sum(s, sh);
    if (threadIdx.x == 0) { *tot = s; *ticket = 0u; return true; }
    return false;
}

// scalars and counters start from zero on every call
__global__ void st_reset(unsigned char *base) {
    StaticView v = view_of(base);
    if (threadIdx.x == 0 && blockIdx.x == 0) memset(v.ks, 0, sizeof(StaticScalars));
}

__global__ void st_diag(int n, const int32_t *rp, const int32_t *col, const double *val, unsigned char *base) {
    StaticView v = view_of(base);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0;
    bool found = false;
    for (int k = rp[i]; k < rp[i + 1]; ++k)
        if (col[k] == i) { d = val[k]; found = true; break; }
    v.dinv[i] = d;
    if (found && d > 0) atomicMax(&v.ks->maxbits, (unsigned long long)__double_as_longlong(d));
}

__global__ void st_diag_second(int n, unsigned char *base) {
    StaticView v = view_of(base);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double top = __longlong_as_double((long long)v.ks->maxbits);
    double d = v.dinv[i];
    if (d == top) atomicAdd(&v.ks->count, 1);
    else if (d > 0 && d < top) atomicMax(&v.ks->max1bits, (unsigned long long)__double_as_longlong(d));
}

// gettgv (HashMatrix.cpp:1341-1371), Jacobi 1/A_ii, x_i = b_i/tgv on tgv rows
__global__ void st_jacobi(int n, const double *b, double *x, double tgv, unsigned char *base) {
    StaticView v = view_of(base);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double top = __longlong_as_double((long long)v.ks->maxbits);
    double max1 = __longlong_as_double((long long)v.ks->max1bits);
    // no positive diagonal at all (top == 0): no tgv rows, as in ffgpu_solve_cg, whose
    // threshold is then out of reach
    bool has_tgv = top > 0 && !(max1 * 1e6 > top) && v.ks->count > 0;
    double d = v.dinv[i];
    bool w = has_tgv && d == top;
    v.wcl[i] = w;
    if (w) x[i] = b[i] / tgv;
    v.dinv[i] = (d * d < 1e-60) ? 1.0 : 1.0 / d;
}

template <int T>
__device__ __forceinline__ double st_row(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                         const double *__restrict__ val, const double *__restrict__ x, int r, int sub) {
    int b = __ldg(rp + r), e = __ldg(rp + r + 1);
    double s = 0;
    for (int k = b + sub; k < e; k += T) s = fma(__ldg(val + k), __ldg(x + __ldg(col + k)), s);
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// y = A x (for the initial residual)
template <int T>
__global__ void __launch_bounds__(256) st_spmv(int n, const int32_t *rp, const int32_t *col, const double *val,
                                               const double *x, double *y) {
    const int lane = threadIdx.x & 31, gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    for (int base = 0; base < n; base += gridDim.x * groups) {
        int a = base + g;
        double s = st_row<T>(rp, col, val, x, a < n ? a : 0, a < n ? sub : T);
        if (a < n && sub == 0) y[a] = s;
    }
}

__global__ void __launch_bounds__(kStThreads) st_init(int n, const double *b, double eps, int itmax,
                                                      unsigned char *base) {
    __shared__ double sh[32];
    __shared__ bool s_last;
    StaticView v = view_of(base);
    double s1 = 0, s2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double gi = v.g[i] - b[i];
        v.g[i] = gi;
        double ci = v.dinv[i] * gi;
        v.h[i] = -ci;
        s1 = fma(gi, ci, s1);
        s2 = fma(gi, -ci, s2);
    }
    double p1 = st_block_sum(s1, sh), p2 = st_block_sum(s2, sh);
    if (threadIdx.x == 0) {
        v.part[blockIdx.x] = p1;
        v.part[gridDim.x + blockIdx.x] = p2;
        __threadfence();
        unsigned t = atomicAdd(&v.ks->ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double a = 0, c = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        a += __ldcg(v.part + i);
        c += __ldcg(v.part + gridDim.x + i);
    }
    a = st_block_sum(a, sh);
    c = st_block_sum(c, sh);
    if (threadIdx.x == 0) {
        StaticScalars *k = v.ks;
        k->gcg = a; k->gcg0 = a; k->gcgp = a; k->s_gh = c;
        k->eps2 = eps > 0 ? eps * eps * a : eps * eps;
        k->iter = 0; k->itmax = itmax; k->converged = 0; k->done = 0;
        if (a < 1e-30) { k->done = 1; k->converged = 2; }
        k->ticket = 0u;
    }
}

template <int T>
__global__ void __launch_bounds__(256) st_ka(int n, const int32_t *rp, const int32_t *col, const double *val,
                                             unsigned char *base) {
    __shared__ double sh[32];
    StaticView v = view_of(base);
    if (v.ks->done) return;
    const int lane = threadIdx.x & 31, gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    double hq = 0;
    for (int b0 = 0; b0 < n; b0 += gridDim.x * groups) {
        int a = b0 + g;
        double s = st_row<T>(rp, col, val, v.h, a < n ? a : 0, a < n ? sub : T);
        if (a < n && sub == 0) { v.q[a] = s; hq = fma(v.h[a], s, hq); }
    }
    double tot;
    double p = st_block_sum(hq, sh);
    if (st_last_block(p, v.part, &v.ks->ticket, &tot, sh)) { v.ks->s_hq = tot; v.ks->rho = -v.ks->s_gh / tot; }
}

__global__ void __launch_bounds__(kStThreads) st_kb(int n, double *x, unsigned char *base) {
    __shared__ double sh[32];
    StaticView v = view_of(base);
    if (v.ks->done) return;
    const double rho = v.ks->rho;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(rho, v.h[i], x[i]);
        double gi = fma(rho, v.q[i], v.g[i]);
        v.g[i] = gi;
        s = fma(gi, v.dinv[i] * gi, s);
    }
    double tot;
    double p = st_block_sum(s, sh);
    if (st_last_block(p, v.part, &v.ks->ticket, &tot, sh)) {
        StaticScalars *k = v.ks;
        k->gcgp = k->gcg;
        k->gcg = tot;
        k->gamma = tot / k->gcgp;
        k->iter += 1;
        if (tot < k->eps2) { k->converged = 1; k->done = 1; }
        else if (k->iter >= k->itmax) k->done = 1;
    }
}

__global__ void __launch_bounds__(kStThreads) st_kc(int n, unsigned char *base) {
    __shared__ double sh[32];
    StaticView v = view_of(base);
    if (v.ks->done) return;
    const double gamma = v.ks->gamma;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double gi = v.g[i];
        double hi = gamma * v.h[i] - v.dinv[i] * gi;
        v.h[i] = hi;
        s = fma(gi, hi, s);
    }
    double tot;
    double p = st_block_sum(s, sh);
    if (st_last_block(p, v.part, &v.ks->ticket, &tot, sh)) v.ks->s_gh = tot;
}

// per-device address of g_cg_scratch, looked up once with the device current
static std::mutex g_static_mu;
static unsigned char *g_static_ptr[64] = {nullptr};

static int static_scratch(unsigned char **out) {
    int dev = -1;
    FFGPU_CUDA(cudaGetDevice(&dev));
    FFGPU_CHECK(dev >= 0 && dev < 64, FFGPU_EINVAL, "ffgpu_solve_cg_csr_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
        if (e != cudaSuccess || !p) {
            set_error("ffgpu_solve_cg_csr_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return FFGPU_ECUDA;
        }
        g_static_ptr[dev] = (unsigned char *)p;
    }
    *out = g_static_ptr[dev];
    return FFGPU_OK;
}

// device memory of the current device `dev`, or managed memory (reachable from every device);
// device memory of another GPU is refused: the kernels here would read it as peer memory
static bool on_device(const void *p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

template <int T>
static void launch_spmv_pair(int n, const int32_t *rp, const int32_t *col, const double *val, const double *x,
                             double *y, cudaStream_t s) {
    int groups = 8 * (32 / T);
    int grid = max(1, min(kStSpmvBlocks, (n + groups - 1) / groups));
    st_spmv<T><<<grid, 256, 0, s>>>(n, rp, col, val, x, y);
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_solve_cg_csr_noalloc(int n, int64_t nnz, const int32_t *rowptr, const int32_t *col, const double *val,
                               const double *b, double *x, double eps, int itmax, double tgv, void *stream,
                               int *iterations, double *gcg_out) {
    FFGPU_CHECK(n > 0 && nnz > 0, FFGPU_EINVAL, "ffgpu_solve_cg_csr_noalloc: empty matrix");
    FFGPU_CHECK(n <= kStaticMaxN, FFGPU_EINVAL,
                "ffgpu_solve_cg_csr_noalloc: n = %d exceeds the fixed scratch capacity of %lld DOFs", n,
                (long long)kStaticMaxN);
    FFGPU_CHECK(rowptr && col && val && b && x, FFGPU_EINVAL, "ffgpu_solve_cg_csr_noalloc: NULL array");
    int dev = -1;
    FFGPU_CUDA(cudaGetDevice(&dev));
    FFGPU_CHECK(on_device(rowptr, dev) && on_device(col, dev) && on_device(val, dev) && on_device(b, dev) &&
                    on_device(x, dev),
                FFGPU_EINVAL, "ffgpu_solve_cg_csr_noalloc: every array must be device memory of the current device "
                "(or managed memory)");
    unsigned char *base = nullptr;
    FFGPU_TRY(static_scratch(&base));
    cudaStream_t s = (cudaStream_t)stream;
    if (tgv <= 0) tgv = 1e30;
    if (itmax <= 0) itmax = n;
    const double avg = (double)nnz / n;
    const int T = avg >= 24 ? 8 : (avg >= 10 ? 4 : 2);
    StaticView v = view_of(base);
    const int gv = (n + 255) / 256;
    st_reset<<<1, 32, 0, s>>>(base);
    st_diag<<<gv, 256, 0, s>>>(n, rowptr, col, val, base);
    st_diag_second<<<gv, 256, 0, s>>>(n, base);
    st_jacobi<<<gv, 256, 0, s>>>(n, b, x, tgv, base);
    if (T == 8) launch_spmv_pair<8>(n, rowptr, col, val, x, v.g, s);
    else if (T == 4) launch_spmv_pair<4>(n, rowptr, col, val, x, v.g, s);
    else launch_spmv_pair<2>(n, rowptr, col, val, x, v.g, s);
    st_init<<<kStBlocks, kStThreads, 0, s>>>(n, b, eps, itmax, base);
    FFGPU_CUDA(cudaGetLastError());
    int groups = 8 * (32 / T);
    int sgrid = max(1, min(kStSpmvBlocks, (n + groups - 1) / groups));
    int done = 0;
    for (int it = 0; it <= itmax; it += kPollEvery) {
        for (int u = 0; u < kPollEvery; ++u) {
            if (T == 8) st_ka<8><<<sgrid, 256, 0, s>>>(n, rowptr, col, val, base);
            else if (T == 4) st_ka<4><<<sgrid, 256, 0, s>>>(n, rowptr, col, val, base);
            else st_ka<2><<<sgrid, 256, 0, s>>>(n, rowptr, col, val, base);
            st_kb<<<kStBlocks, kStThreads, 0, s>>>(n, x, base);
            st_kc<<<kStBlocks, kStThreads, 0, s>>>(n, base);
        }
        FFGPU_CUDA(cudaGetLastError());
        FFGPU_CUDA(cudaMemcpyAsync(&done, &v.ks->done, sizeof(int), cudaMemcpyDeviceToHost, s));
        FFGPU_CUDA(cudaStreamSynchronize(s));
        if (done) break;
    }
    StaticScalars hs;
    FFGPU_CUDA(cudaMemcpyAsync(&hs, v.ks, sizeof(hs), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    if (iterations) *iterations = hs.iter;
    if (gcg_out) { gcg_out[0] = hs.gcg; gcg_out[1] = hs.eps2; }
    if (!hs.converged) {
        set_error("ffgpu_solve_cg_csr_noalloc: no convergence after %d iterations", hs.iter);
        return FFGPU_ENOCONV;
    }
    return FFGPU_OK;
}

}  // extern "C"
