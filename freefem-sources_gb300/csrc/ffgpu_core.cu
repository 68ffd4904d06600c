// ffgpu_core.cu -- context, error reporting, scans and small reductions.
#include <stdarg.h>
#include <string.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

bool is_device_ptr(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int launch_check(ffgpu_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
        return FFGPU_ECUDA;
    }
    return FFGPU_OK;
}

int tuned_layout(const ffgpu_ctx *ctx, const ffgpu_matrix *A, int mode) {
    for (const ffgpu_ctx::Tuned &t : ctx->tuned)
        if (t.nb == A->nb && t.nnzb == A->nnzb && t.bs == A->bs && t.mode == mode) return t.lanes;
    return 0;
}

void tuned_store(ffgpu_ctx *ctx, const ffgpu_matrix *A, int mode, int code) {
    for (ffgpu_ctx::Tuned &t : ctx->tuned)
        if (t.nb == A->nb && t.nnzb == A->nnzb && t.bs == A->bs && t.mode == mode) { t.lanes = code; return; }
    ctx->tuned.push_back(ffgpu_ctx::Tuned{A->nb, A->nnzb, A->bs, code, mode});
}

int tuned_pick(const float *ms, int n) {
    float best = ms[0];
    for (int i = 1; i < n; ++i) best = ms[i] < best ? ms[i] : best;
    for (int i = 0; i < n; ++i)
        if (ms[i] <= best * (1.0f + kTuneMargin)) return i;
    return 0;
}

int check_device_status(ffgpu_ctx *ctx, const char *where) {
    int st = 0;
    FFGPU_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FFGPU_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st != kDevOk) {
        static const char *msg[] = {"ok", "too many candidate neighbours per row (mesh valence)",
                                    "row degree above capacity", "[P2]^3 DOF table is not 3*node+c",
                                    "index out of range in an input table",
                                    "column missing from a row", "a bounded wait in a kernel timed out"};
        set_error("%s: device reported: %s", where, (st > 0 && st < 7) ? msg[st] : "unknown");
        int zero = 0;
        cudaMemcpyAsync(ctx->d_status, &zero, sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (st == kDevTimeout) return FFGPU_ECUDA;
        return st == kDevBadDofLayout || st == kDevBadIndex ? FFGPU_EINVAL : FFGPU_EMESH;
    }
    return FFGPU_OK;
}

// ------------------------------------------------------------------ exclusive scan (int32)
// Three phases: per-block totals, a single-block scan of the totals, per-block scan + offset.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;   // items per thread
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    int pre = (wid > 0 ? sh[wid - 1] : 0) + x - v;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return pre;
}

__global__ void scan_tile_totals(const int32_t *in, int n, int32_t *tot) {
    __shared__ int sh[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    int t;
    block_excl_scan(s, sh, &t);
    if (threadIdx.x == 0) tot[blockIdx.x] = t;
}

__global__ void scan_totals(int32_t *tot, int nb) {
    __shared__ int sh[32];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanThreads) {
        int i = base + threadIdx.x;
        int v = i < nb ? tot[i] : 0;
        int t;
        int pre = block_excl_scan(v, sh, &t);
        if (i < nb) tot[i] = carry + pre;
        carry += t;
    }
    if (threadIdx.x == 0) tot[nb] = carry;
}

__global__ void scan_tiles(const int32_t *in, int n, const int32_t *tot, int32_t *out) {
    __shared__ int sh[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int t;
    int pre = block_excl_scan(s, sh, &t) + tot[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = pre;
        pre += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = tot[gridDim.x];
}

int device_scan_i32(ffgpu_ctx *ctx, const int32_t *in, int32_t *out, int n) {
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) {
        FFGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), ctx->stream));
        return FFGPU_OK;
    }
    int32_t *tot = nullptr;
    FFGPU_CUDA(dalloc(ctx, (void **)&tot, sizeof(int32_t) * (nb + 1)));
    scan_tile_totals<<<nb, kScanThreads, 0, ctx->stream>>>(in, n, tot);
    int r = launch_check(ctx, "scan_tile_totals");
    if (r == FFGPU_OK) {
        scan_totals<<<1, kScanThreads, 0, ctx->stream>>>(tot, nb);
        r = launch_check(ctx, "scan_totals");
    }
    if (r == FFGPU_OK) {
        scan_tiles<<<nb, kScanThreads, 0, ctx->stream>>>(in, n, tot, out);
        r = launch_check(ctx, "scan_tiles");
    }
    dfree(ctx, tot);
    return r;
}

__global__ void max_i32_kernel(const int32_t *in, int n, int *out) {
    int m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, in[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

int device_max_i32(ffgpu_ctx *ctx, const int32_t *in, int n, int *host_max) {
    FFGPU_CUDA(cudaMemsetAsync(ctx->d_iscratch, 0, sizeof(int), ctx->stream));
    int grid = min(kNumSM * 4, max(1, (n + 255) / 256));
    max_i32_kernel<<<grid, 256, 0, ctx->stream>>>(in, n, ctx->d_iscratch);
    FFGPU_TRY(launch_check(ctx, "max_i32"));
    FFGPU_CUDA(cudaMemcpyAsync(host_max, ctx->d_iscratch, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
    FFGPU_CUDA(cudaStreamSynchronize(ctx->stream));
    return FFGPU_OK;
}

// ------------------------------------------------------------------ stable order by key
// Counting sort by decreasing key, stable in the index: per-tile histograms laid out
// (key-major, tile-minor), one exclusive scan, then each tile places its rows in index order
// (32 at a time, ranks among equal keys from __match_any_sync).  Deterministic.
constexpr int kOrdTile = 1024;

__global__ void order_hist_kernel(const int32_t *key, int n, int maxkey, int ntiles, int32_t *hist) {
    extern __shared__ int sh_hist[];
    const int K = maxkey + 1;
    for (int d = threadIdx.x; d < K; d += blockDim.x) sh_hist[d] = 0;
    __syncthreads();
    int64_t i = (int64_t)blockIdx.x * kOrdTile + threadIdx.x;
    for (int k = 0; k < kOrdTile / 1024; ++k, i += 1024)
        if (i < n) atomicAdd(&sh_hist[maxkey - key[i]], 1);
    __syncthreads();
    for (int d = threadIdx.x; d < K; d += blockDim.x) hist[(int64_t)d * ntiles + blockIdx.x] = sh_hist[d];
}

__global__ void order_place_kernel(const int32_t *key, int n, int maxkey, int ntiles, const int32_t *off,
                                   int32_t *order) {
    extern __shared__ int sh_run[];
    const int K = maxkey + 1, lane = threadIdx.x;
    for (int d = lane; d < K; d += 32) sh_run[d] = off[(int64_t)d * ntiles + blockIdx.x];
    __syncwarp();
    for (int c = 0; c < kOrdTile; c += 32) {
        int64_t i = (int64_t)blockIdx.x * kOrdTile + c + lane;
        bool ok = i < n;
        int d = ok ? maxkey - key[i] : -1;
        unsigned same = __match_any_sync(0xffffffffu, d);
        int rank = __popc(same & ((1u << lane) - 1u));
        int pos = ok ? sh_run[d] + rank : 0;
        __syncwarp();
        if (ok) order[pos] = (int32_t)i;
        if (ok && rank == __popc(same) - 1) sh_run[d] += __popc(same);
        __syncwarp();
    }
}

int device_order_by_key_desc(ffgpu_ctx *ctx, const int32_t *key, int n, int maxkey, int32_t *order) {
    if (n <= 0) return FFGPU_OK;
    const int ntiles = (n + kOrdTile - 1) / kOrdTile;
    const int K = maxkey + 1;
    int64_t m = (int64_t)K * ntiles;
    FFGPU_CHECK(m < (int64_t)1 << 30, FFGPU_EINVAL, "row ordering: %d keys x %d tiles too large", K, ntiles);
    int32_t *hist = nullptr;
    FFGPU_CUDA(dalloc(ctx, (void **)&hist, sizeof(int32_t) * (2 * m + 1)));
    int32_t *off = hist + m;
    size_t smem = sizeof(int) * K;
    order_hist_kernel<<<ntiles, 1024, smem, ctx->stream>>>(key, n, maxkey, ntiles, hist);
    int r = launch_check(ctx, "order_hist");
    if (!r) r = device_scan_i32(ctx, hist, off, (int)m);
    if (!r) {
        order_place_kernel<<<ntiles, 32, smem, ctx->stream>>>(key, n, maxkey, ntiles, off, order);
        r = launch_check(ctx, "order_place");
    }
    dfree(ctx, hist);
    return r;
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

const char *ffgpu_last_error(void) { return g_err; }

int ffgpu_ctx_create(int device, ffgpu_ctx **out) {
    FFGPU_CHECK(out, FFGPU_EINVAL, "ffgpu_ctx_create: out is NULL");
    int ndev = 0;
    FFGPU_CUDA(cudaGetDeviceCount(&ndev));
    FFGPU_CHECK(device >= 0 && device < ndev, FFGPU_EINVAL, "ffgpu_ctx_create: no device %d", device);
    FFGPU_CUDA(cudaSetDevice(device));
    ffgpu_ctx *c = new ffgpu_ctx();   // value-initialised: every plain member starts at zero
    c->device = device;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    uint64_t keep = UINT64_MAX;  // freed blocks stay mapped for the next object of the context
    if (cudaMemPoolCreate(&c->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void **)&c->d_part, sizeof(double) * 8192) != cudaSuccess ||
        cudaMalloc((void **)&c->d_status, sizeof(int) * 4) != cudaSuccess ||
        cudaMalloc((void **)&c->d_ticket, sizeof(unsigned int) * 16) != cudaSuccess ||
        cudaMalloc((void **)&c->d_iscratch, sizeof(int) * 16) != cudaSuccess) {
        set_error("ffgpu_ctx_create: CUDA setup failed: %s", cudaGetErrorString(cudaGetLastError()));
        if (c->pool) cudaMemPoolDestroy(c->pool);
        delete c;
        return FFGPU_ECUDA;
    }
    cudaMemset(c->d_status, 0, sizeof(int) * 4);
    cudaMemset(c->d_ticket, 0, sizeof(unsigned int) * 16);
    cudaDeviceSynchronize();
    *out = c;
    return FFGPU_OK;
}

int ffgpu_ctx_destroy(ffgpu_ctx *c) {
    if (!c) return FFGPU_OK;
    cudaStreamSynchronize(c->stream);
    cudaFree(c->d_part);
    cudaFree(c->d_status);
    cudaFree(c->d_ticket);
    cudaFree(c->d_iscratch);
    cudaStreamDestroy(c->stream);
    // blocks of objects still alive are released when those objects free them
    cudaMemPoolDestroy(c->pool);
    delete c;
    return FFGPU_OK;
}

int64_t ffgpu_ctx_kernel_launches(const ffgpu_ctx *c) { return c ? c->launches : 0; }

void *ffgpu_ctx_stream(const ffgpu_ctx *c) { return c ? (void *)c->stream : nullptr; }

}  // extern "C"
