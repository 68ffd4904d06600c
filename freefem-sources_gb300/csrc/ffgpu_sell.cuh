// ffgpu_sell.cuh -- device row kernels of the SELL-32 SpMV (layout in ffgpu_sell.cu) and the
// block reductions shared by the fused Krylov kernels.
#pragma once
#include "ffgpu_internal.cuh"

namespace ffgpu {

// ------------------------------------------------------------------ block reductions
// Block sum; the block total is returned in every thread of warp 0 (thread 0 uses it).
template <typename T>
__device__ __forceinline__ T block_sum_t(T v, T *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    T t = 0;
    if (w == 0) {
        t = lane < nw ? sh[lane] : T(0);
        t = warp_sum(t);
    }
    __syncthreads();
    return t;
}

// Stores this block's partial; returns true in exactly one thread of the last block to finish,
// whose `tot` receives the sum of all partials in block order (deterministic).
template <typename T>
__device__ __forceinline__ bool last_block_sum(T partial, T *part, unsigned *ticket, T *tot, T *sh) {
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
    T s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(part + i);
    s = block_sum_t(s, sh);
    if (threadIdx.x == 0) {
        *tot = s;
        *ticket = 0u;
        return true;
    }
    return false;
}

// ------------------------------------------------------------------ double-float arithmetic
// FP64 values and vectors split exactly into FP32 pairs v = hi + lo (48 of the 53 bits); a
// product hi*hi is formed exactly as p + e (e = fma(a, x, -p)), the cross terms are added in
// FP32, and sums are kept as an unevaluated pair (S, C) with Knuth's TwoSum.  The row result
// (double)S + (double)C is accurate to about 2^-44 relative.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void df_fma(float2 a, float2 x, float &S, float &C) {
    float p = __fmul_rn(a.x, x.x);
    float pe = __fmaf_rn(a.x, x.x, -p);
    float t = __fmaf_rn(a.x, x.y, __fmaf_rn(a.y, x.x, pe));
    float s2, e;
    two_sum(S, p, s2, e);
    S = s2;
    C = __fadd_rn(C, __fadd_rn(e, t));
}

__device__ __forceinline__ float2 split_f64(double v) {
    float hi = __double2float_rn(v);
    float lo = __double2float_rn(v - (double)hi);
    return make_float2(hi, lo);
}

// ------------------------------------------------------------------ SELL-32 chunk assignment
// kSellRanges: warp w takes the contiguous chunks [part[w], part[w+1]) (equal slot shares).
// kSellRotated: pass k of warp w takes chunk k*nw + (w + 5k) mod nw -- the chunks in flight at
//   a time stay one contiguous band of the matrix, and the rotation by an odd step walks every
//   warp through all 32 positions of the degree-sorted windows.
// The tuners time both, each with two unroll depths of the row loop (DEEP).
enum SellAssign { kSellRanges = 0, kSellRotated = 1 };

template <int ASSIGN>
struct ChunkWalk {
    int c, ce, k, w, nw;
    __device__ __forceinline__ ChunkWalk(const SellArgs &S) {
        w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        nw = (gridDim.x * blockDim.x) >> 5;
        k = 0;
        if constexpr (ASSIGN == kSellRanges) {
            c = __ldg(S.part + w);
            ce = __ldg(S.part + w + 1);
        } else {
            ce = S.nchunk;
            c = at(0);
        }
    }
    __device__ __forceinline__ int at(int kk) const { return kk * nw + (w + 5 * kk) % nw; }
    // next chunk of this warp (>= ce when done)
    __device__ __forceinline__ int next() {
        if constexpr (ASSIGN == kSellRanges) return c + 1;
        return (int64_t)(k + 1) * nw < ce ? at(k + 1) : ce;
    }
    __device__ __forceinline__ void advance(int cn) { c = cn; ++k; }
};

// Calls body(c, a, L, sr) for every chunk of this warp (a: the lane's row, L: slots, sr: first
// slot row), loading the next chunk's row, length and offset while the current one runs.
template <int ASSIGN, typename F>
__device__ __forceinline__ void sell_for_chunks(const SellArgs &S, F &&body) {
    const int lane = threadIdx.x & 31;
    ChunkWalk<ASSIGN> it(S);
    // the rotated stride can land past the last chunk on a warp's final pass
    while (it.c < it.ce && it.c >= S.nchunk) it.advance(it.next());
    if (it.c >= it.ce) return;
    int a = __ldg(S.perm + (int64_t)it.c * 32 + lane), L = __ldg(S.len + it.c);
    int64_t sr = __ldg(S.off + it.c);
    for (;;) {
        int cn = it.next();
        while (cn < it.ce && cn >= S.nchunk) { it.advance(cn); cn = it.next(); }
        int an = 0, Ln = 0;
        int64_t srn = 0;
        if (cn < it.ce) {
            an = __ldg(S.perm + (int64_t)cn * 32 + lane);
            Ln = __ldg(S.len + cn);
            srn = __ldg(S.off + cn);
        }
        body(it.c, a, L, sr);
        if (cn >= it.ce) break;
        it.advance(cn);
        a = an; L = Ln; sr = srn;
    }
}

// ------------------------------------------------------------------ SELL-32 rows
// One block row per lane: lane `lane` of chunk c holds row a (a < 0: padding lane, its
// entries are zero blocks on column 0).  Entries are read in column order; matrix streams use
// evict-first loads so that the gathered vector stays in L2.
template <bool C16>
__device__ __forceinline__ int sell_col(const SellArgs &S, int64_t e, int ar) {
    if (C16) return ar + (int)__ldcs(S.col16 + e);
    return __ldcs(S.col + e);
}

template <int BS, bool C16, bool DEEP>
__device__ __forceinline__ void sell_row64(const SellArgs &S, const double *__restrict__ val,
                                           const double *__restrict__ x, int L, int64_t sr, int lane, int a,
                                           double *y) {
    const int ar = a < 0 ? 0 : a;
    const int64_t ce = sr * 32 + lane;
    const double *v = val + sr * (BS * BS * 32) + lane;
    double s0 = 0, s1 = 0, s2 = 0;
    // slots in flight (the column -> gather dependency): scalar rows 8 or 16, 3x3 blocks 2 or 4
    constexpr int UNR = BS == 1 ? (DEEP ? 16 : 8) : (DEEP ? 4 : 2);
#pragma unroll UNR
    for (int j = 0; j < L; ++j) {
        const int col = sell_col<C16>(S, ce + (int64_t)j * 32, ar);
        if (BS == 1) {
            s0 = fma(__ldcs(v + (int64_t)j * 32), __ldg(x + col), s0);
        } else {
            const double x0 = __ldg(x + 3 * (int64_t)col), x1 = __ldg(x + 3 * (int64_t)col + 1),
                         x2 = __ldg(x + 3 * (int64_t)col + 2);
            const double *w = v + (int64_t)j * 288;
            s0 = fma(__ldcs(w), x0, s0); s0 = fma(__ldcs(w + 32), x1, s0); s0 = fma(__ldcs(w + 64), x2, s0);
            s1 = fma(__ldcs(w + 96), x0, s1); s1 = fma(__ldcs(w + 128), x1, s1); s1 = fma(__ldcs(w + 160), x2, s1);
            s2 = fma(__ldcs(w + 192), x0, s2); s2 = fma(__ldcs(w + 224), x1, s2); s2 = fma(__ldcs(w + 256), x2, s2);
        }
    }
    y[0] = s0;
    if (BS == 3) { y[1] = s1; y[2] = s2; }
}

template <int BS, bool C16, bool DEEP>
__device__ __forceinline__ void sell_rowx(const SellArgs &S, const float2 *__restrict__ val,
                                          const float2 *__restrict__ x, int L, int64_t sr, int lane, int a,
                                          double *y) {
    const int ar = a < 0 ? 0 : a;
    const int64_t ce = sr * 32 + lane;
    const float2 *v = val + sr * (BS * BS * 32) + lane;
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f, S2 = 0.f, C2 = 0.f;
    constexpr int UNR = BS == 1 ? (DEEP ? 16 : 8) : (DEEP ? 4 : 2);
#pragma unroll UNR
    for (int j = 0; j < L; ++j) {
        const int col = sell_col<C16>(S, ce + (int64_t)j * 32, ar);
        if (BS == 1) {
            df_fma(__ldcs(v + (int64_t)j * 32), __ldg(x + col), S0, C0);
        } else {
            const float2 x0 = __ldg(x + 3 * (int64_t)col), x1 = __ldg(x + 3 * (int64_t)col + 1),
                         x2 = __ldg(x + 3 * (int64_t)col + 2);
            const float2 *w = v + (int64_t)j * 288;
            df_fma(__ldcs(w), x0, S0, C0); df_fma(__ldcs(w + 32), x1, S0, C0); df_fma(__ldcs(w + 64), x2, S0, C0);
            df_fma(__ldcs(w + 96), x0, S1, C1); df_fma(__ldcs(w + 128), x1, S1, C1); df_fma(__ldcs(w + 160), x2, S1, C1);
            df_fma(__ldcs(w + 192), x0, S2, C2); df_fma(__ldcs(w + 224), x1, S2, C2); df_fma(__ldcs(w + 256), x2, S2, C2);
        }
    }
    y[0] = (double)S0 + (double)C0;
    if (BS == 3) {
        y[1] = (double)S1 + (double)C1;
        y[2] = (double)S2 + (double)C2;
    }
}

template <int BS, bool C16, bool DEEP>
__device__ __forceinline__ void sell_row32(const SellArgs &S, const float *__restrict__ val,
                                           const float *__restrict__ x, int L, int64_t sr, int lane, int a,
                                           float *y) {
    const int ar = a < 0 ? 0 : a;
    const int64_t ce = sr * 32 + lane;
    const float *v = val + sr * (BS * BS * 32) + lane;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    constexpr int UNR = BS == 1 ? (DEEP ? 16 : 8) : (DEEP ? 8 : 4);
#pragma unroll UNR
    for (int j = 0; j < L; ++j) {
        const int col = sell_col<C16>(S, ce + (int64_t)j * 32, ar);
        if (BS == 1) {
            s0 = fmaf(__ldcs(v + (int64_t)j * 32), __ldg(x + col), s0);
        } else {
            const float x0 = __ldg(x + 3 * (int64_t)col), x1 = __ldg(x + 3 * (int64_t)col + 1),
                        x2 = __ldg(x + 3 * (int64_t)col + 2);
            const float *w = v + (int64_t)j * 288;
            s0 = fmaf(__ldcs(w), x0, s0); s0 = fmaf(__ldcs(w + 32), x1, s0); s0 = fmaf(__ldcs(w + 64), x2, s0);
            s1 = fmaf(__ldcs(w + 96), x0, s1); s1 = fmaf(__ldcs(w + 128), x1, s1); s1 = fmaf(__ldcs(w + 160), x2, s1);
            s2 = fmaf(__ldcs(w + 192), x0, s2); s2 = fmaf(__ldcs(w + 224), x1, s2); s2 = fmaf(__ldcs(w + 256), x2, s2);
        }
    }
    y[0] = s0;
    if (BS == 3) { y[1] = s1; y[2] = s2; }
}

}  // namespace ffgpu
