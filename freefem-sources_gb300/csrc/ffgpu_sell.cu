// ffgpu_sell.cu -- the SELL-32 copy of an assembled matrix used by the Krylov SpMVs.
//
// The assembled matrix stays in block CSR (FreeFEM's pattern, sorted columns); that is what
// export, the transpose and the diagonal read.  The CG/IR SpMVs read a sliced copy instead:
//   * block rows are sorted by decreasing degree inside windows of 1024 consecutive rows
//     (rows stay near their neighbours, so the x gathers of a warp stay local), stable;
//   * 32 consecutive sorted rows form a chunk, one row per lane; a chunk is padded to its
//     longest row (the first one) with zero blocks;
//   * entry j of lane r of chunk c is stored at slot row soff[c] + j, lane r: a warp reads
//     32 consecutive column indices and, for each of the bs*bs values, 32 consecutive values.
// Every lane of a warp runs the same trip count, every load is a full 128/256-byte line, and
// no lane-group reductions are needed.  Each warp of a launch owns a contiguous range of
// chunks holding an equal share of the slots (sell_partition): windows start with their
// longest rows, so a fixed stride over chunks would give some warps only long chunks.
// Within a row the entries keep their column order, so the row sums are formed in the same
// order as the block-CSR kernels form them.
// For bs == 1 the column is stored as the 16-bit difference column - row whenever the
// matrix bandwidth allows (2 instead of 4 bytes per entry).
#include <string.h>

#include <algorithm>

#include "ffgpu_internal.cuh"

namespace ffgpu {

constexpr int kSellWin = 1024;    // rows per sorting window (32 chunks)

// window sort: key = (max - degree, position) so that ascending order is decreasing degree,
// ties by row; rows past nb sort last and become padding lanes (-1)
__global__ void __launch_bounds__(kSellWin) sell_sort_kernel(int nb, const int32_t *__restrict__ rp,
                                                             int32_t *__restrict__ perm) {
    __shared__ uint32_t key[kSellWin];
    const int t = threadIdx.x;
    const int64_t r = (int64_t)blockIdx.x * kSellWin + t;
    uint32_t k = 0xFFFFFFFFu;
    if (r < nb) {
        int deg = rp[r + 1] - rp[r];
        k = ((uint32_t)(0x1FFFFF - deg) << 10) | (uint32_t)t;
    }
    key[t] = k;
    __syncthreads();
    for (int size = 2; size <= kSellWin; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int p = t ^ stride;
            if (p > t) {
                const uint32_t a = key[t], b = key[p];
                const bool up = (t & size) == 0;
                if ((a > b) == up) { key[t] = b; key[p] = a; }
            }
            __syncthreads();
        }
    }
    const uint32_t s = key[t];
    perm[(int64_t)blockIdx.x * kSellWin + t] =
        s == 0xFFFFFFFFu ? -1 : (int32_t)((int64_t)blockIdx.x * kSellWin + (s & 1023u));
}

__global__ void sell_len_kernel(int nchunk, const int32_t *__restrict__ perm, const int32_t *__restrict__ rp,
                                int32_t *__restrict__ len) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nchunk) {
        const int a = perm[(int64_t)c * 32];
        len[c] = a >= 0 ? rp[a + 1] - rp[a] : 0;
    }
}

// largest |column - row| of each row
__global__ void sell_band_kernel(int nb, const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                 int32_t *__restrict__ band) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nb) return;
    int m = 0;
    for (int k = rp[a]; k < rp[a + 1]; ++k) m = max(m, abs(col[k] - (int)a));
    band[a] = m;
}

// column slots: padding entries repeat the row's last column (a valid, cached x entry)
template <bool C16>
__global__ void sell_col_kernel(int nchunk, const int32_t *__restrict__ perm, const int32_t *__restrict__ len,
                                const int32_t *__restrict__ off, const int32_t *__restrict__ rp,
                                const int32_t *__restrict__ col, int32_t *__restrict__ scol,
                                int16_t *__restrict__ scol16) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nchunk * 32) return;
    const int c = (int)(t >> 5), lane = (int)(t & 31);
    const int a = perm[t];
    const int L = len[c];
    const int64_t base = (int64_t)off[c] * 32 + lane;
    const int b = a >= 0 ? rp[a] : 0, deg = a >= 0 ? rp[a + 1] - b : 0;
    for (int j = 0; j < L; ++j) {
        const int cj = deg > 0 ? col[b + min(j, deg - 1)] : (a >= 0 ? a : 0);
        if (C16) scol16[base + (int64_t)j * 32] = (int16_t)(cj - (a >= 0 ? a : 0));
        else scol[base + (int64_t)j * 32] = cj;
    }
}

struct ToF64 { __device__ double operator()(double v) const { return v; } };
struct ToF32 { __device__ float operator()(double v) const { return __double2float_rn(v); } };
struct ToDF {
    __device__ float2 operator()(double v) const {
        const float hi = __double2float_rn(v);
        return make_float2(hi, __double2float_rn(v - (double)hi));
    }
};

// values: lane r, slot j, entry m at ((off[c] + j) * bs2 + m) * 32 + r; padding is zero
template <int BS, typename Out, typename Conv>
__global__ void sell_val_kernel(int nchunk, const int32_t *__restrict__ perm, const int32_t *__restrict__ len,
                                const int32_t *__restrict__ off, const int32_t *__restrict__ rp,
                                const double *__restrict__ val, Out *__restrict__ out) {
    constexpr int B2 = BS * BS;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nchunk * 32) return;
    const int c = (int)(t >> 5), lane = (int)(t & 31);
    const int a = perm[t];
    const int L = len[c];
    const int64_t base = (int64_t)off[c] * B2 * 32 + lane;
    const int b = a >= 0 ? rp[a] : 0, deg = a >= 0 ? rp[a + 1] - b : 0;
    Conv conv;
    for (int j = 0; j < L; ++j) {
        const double *src = val + (int64_t)(b + j) * B2;
#pragma unroll
        for (int m = 0; m < B2; ++m) out[base + ((int64_t)j * B2 + m) * 32] = conv(j < deg ? src[m] : 0.0);
    }
}

// start chunk of warp w: the first chunk whose first slot row is at or past w * nslot / nw
__global__ void sell_part_kernel(int nchunk, const int32_t *__restrict__ off, int nw, int32_t *__restrict__ part) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w > nw) return;
    const int64_t target = (int64_t)off[nchunk] * w / nw;
    int lo = 0, hi = nchunk;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    part[w] = w == nw ? nchunk : lo;
}

int sell_partition(ffgpu_matrix *A, int nw, const int32_t **part) {
    for (int i = 0; i < 4; ++i)
        if (A->spart[i] && A->spart_nw[i] == nw) { *part = A->spart[i]; return FFGPU_OK; }
    int slot = 0;
    while (slot < 4 && A->spart[slot]) ++slot;
    if (slot == 4) { dfree(A->ctx, A->spart[3]); A->spart[3] = nullptr; slot = 3; }
    FFGPU_CUDA(dalloc(A->ctx, (void **)&A->spart[slot], sizeof(int32_t) * ((size_t)nw + 1)));
    A->spart_nw[slot] = nw;
    sell_part_kernel<<<(nw + 256) / 256, 256, 0, A->ctx->stream>>>(A->nchunk, A->soff, nw, A->spart[slot]);
    FFGPU_TRY(launch_check(A->ctx, "sell_partition"));
    *part = A->spart[slot];
    return FFGPU_OK;
}

int resident_grid(const void *kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return per_sm * kNumSM;
}

int sized_grid(const void *kernel, int threads, int64_t need, size_t smem) {
    const int64_t g = resident_grid(kernel, threads, smem);
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, need));
}

int sell_prepare(ffgpu_matrix *A) {
    if (A->sperm) return FFGPU_OK;
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    FFGPU_CHECK(A->max_deg < 0x1FFFFF, FFGPU_EINVAL, "SELL layout: row degree %d too large", A->max_deg);
    const int nb = A->nb;
    const int nwin = (nb + kSellWin - 1) / kSellWin;
    const int nchunk = (nb + 31) / 32;
    A->nchunk = nchunk;
    FFGPU_CUDA(dalloc(ctx, (void **)&A->sperm, sizeof(int32_t) * (size_t)nwin * kSellWin));
    FFGPU_CUDA(dalloc(ctx, (void **)&A->slen, sizeof(int32_t) * ((size_t)nchunk + 1)));
    FFGPU_CUDA(dalloc(ctx, (void **)&A->soff, sizeof(int32_t) * ((size_t)nchunk + 1)));
    sell_sort_kernel<<<nwin, kSellWin, 0, s>>>(nb, A->browptr, A->sperm);
    FFGPU_TRY(launch_check(ctx, "sell_sort"));
    sell_len_kernel<<<(nchunk + 255) / 256, 256, 0, s>>>(nchunk, A->sperm, A->browptr, A->slen);
    FFGPU_TRY(launch_check(ctx, "sell_len"));
    FFGPU_TRY(device_scan_i32(ctx, A->slen, A->soff, nchunk));
    int32_t nslot = 0;
    FFGPU_CUDA(cudaMemcpyAsync(&nslot, A->soff + nchunk, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    A->nslot = nslot;
    bool c16 = false;
    if (A->bs == 1) {
        int32_t *band = nullptr;
        FFGPU_CUDA(dalloc(ctx, (void **)&band, sizeof(int32_t) * (size_t)nb));
        sell_band_kernel<<<(nb + 255) / 256, 256, 0, s>>>(nb, A->browptr, A->bcol, band);
        int rc = launch_check(ctx, "sell_band");
        int bw = 0;
        if (!rc) rc = device_max_i32(ctx, band, nb, &bw);
        dfree(ctx, band);
        FFGPU_TRY(rc);
        c16 = bw < 32768;
    }
    const int64_t ent = (int64_t)nslot * 32;
    const int64_t thr = (int64_t)nchunk * 32;
    const int grid = (int)((thr + 255) / 256);
    if (c16) {
        FFGPU_CUDA(dalloc(ctx, (void **)&A->scol16, sizeof(int16_t) * (size_t)ent));
        sell_col_kernel<true><<<grid, 256, 0, s>>>(nchunk, A->sperm, A->slen, A->soff, A->browptr, A->bcol,
                                                   nullptr, A->scol16);
    } else {
        FFGPU_CUDA(dalloc(ctx, (void **)&A->scol, sizeof(int32_t) * (size_t)ent));
        sell_col_kernel<false><<<grid, 256, 0, s>>>(nchunk, A->sperm, A->slen, A->soff, A->browptr, A->bcol,
                                                    A->scol, nullptr);
    }
    return launch_check(ctx, "sell_col");
}

template <typename Out, typename Conv>
static int sell_fill(ffgpu_matrix *A, const double *src, Out **dst) {
    if (*dst) return FFGPU_OK;
    ffgpu_ctx *ctx = A->ctx;
    const int64_t ent = A->nslot * 32 * A->bs * A->bs;
    FFGPU_CUDA(dalloc(ctx, (void **)dst, sizeof(Out) * (size_t)ent));
    const int64_t thr = (int64_t)A->nchunk * 32;
    const int grid = (int)((thr + 255) / 256);
    if (A->bs == 3)
        sell_val_kernel<3, Out, Conv><<<grid, 256, 0, ctx->stream>>>(A->nchunk, A->sperm, A->slen, A->soff,
                                                                    A->browptr, src, *dst);
    else
        sell_val_kernel<1, Out, Conv><<<grid, 256, 0, ctx->stream>>>(A->nchunk, A->sperm, A->slen, A->soff,
                                                                    A->browptr, src, *dst);
    return launch_check(ctx, "sell_values");
}

int sell_values(ffgpu_matrix *A, int kind) {
    FFGPU_TRY(sell_prepare(A));
    if (kind == kSell64T || kind == kSellXT) FFGPU_TRY(matrix_prepare_transpose(A));
    switch (kind) {
        case kSell64: return sell_fill<double, ToF64>(A, A->val, &A->sval);
        case kSell64T: return sell_fill<double, ToF64>(A, A->val_t, &A->sval_t);
        case kSellX: return sell_fill<float2, ToDF>(A, A->val, &A->svalx);
        case kSellXT: return sell_fill<float2, ToDF>(A, A->val_t, &A->svalx_t);
        default: return sell_fill<float, ToF32>(A, A->val, &A->sval32);
    }
}

void sell_release(ffgpu_matrix *A) {
    sell_release_values(A);
    dfree(A->ctx, A->sperm); dfree(A->ctx, A->slen); dfree(A->ctx, A->soff); dfree(A->ctx, A->scol); dfree(A->ctx, A->scol16);
    for (int i = 0; i < 4; ++i) dfree(A->ctx, A->spart[i]);
}

void sell_release_values(ffgpu_matrix *A) {
    dfree(A->ctx, A->sval); dfree(A->ctx, A->sval_t); dfree(A->ctx, A->svalx); dfree(A->ctx, A->svalx_t); dfree(A->ctx, A->sval32);
    A->sval = A->sval_t = nullptr;
    A->svalx = A->svalx_t = nullptr;
    A->sval32 = nullptr;
}

}  // namespace ffgpu
