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
// FP64 values and vectors split into FP32 pairs v ~ hi + lo (48 of the 53 bits kept); a
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
// Entries are read in column order; matrix streams use evict-first loads so that the gathered
// vector stays in L2.
template <bool C16>
__device__ __forceinline__ int sell_col(const SellArgs &S, int64_t e, int ar) {
    if (C16) return ar + (int)__ldcs(S.col16 + e);
    return __ldcs(S.col + e);
}

// FP32 and double-float rows process entries in batches of B slots: all column, value and vector
// loads of a batch are issued before its first product, so a lane keeps B independent gathers
// in flight (a runtime-length loop unrolled B deep runs its remainder one dependent load at a
// time, and most P1 chunks are shorter than 16 slots).  The last, partial batch of a chunk
// loads only its `rem` slots (warp-uniform predicate) and applies exactly that many products
// through a compile-time case chain, so the products and their order are those of the plain
// j = 0..L-1 loop.
struct AccF32 {
    float s = 0.f;
    __device__ __forceinline__ void fma_(float a, float x) { s = fmaf(a, x, s); }
    __device__ __forceinline__ float get() const { return s; }
};
struct AccDF {
    float S = 0.f, C = 0.f;
    __device__ __forceinline__ void fma_(float2 a, float2 x) { df_fma(a, x, S, C); }
    __device__ __forceinline__ double get() const { return (double)S + (double)C; }
};

template <typename V, int BS, int B>
struct SellBatch {
    V a[B][BS * BS];
    V xv[B][BS];
    template <bool C16, bool GUARD>
    __device__ __forceinline__ void load(const SellArgs &S, const V *__restrict__ v, const V *__restrict__ x,
                                         int64_t ce, int ar, int j, int rem) {
#pragma unroll
        for (int u = 0; u < B; ++u) {
            if (GUARD && u >= rem) continue;
            const int col = sell_col<C16>(S, ce + (int64_t)(j + u) * 32, ar);
            const V *w = v + (int64_t)(j + u) * (BS * BS * 32);
#pragma unroll
            for (int k = 0; k < BS * BS; ++k) a[u][k] = __ldcs(w + 32 * k);
#pragma unroll
            for (int m = 0; m < BS; ++m) xv[u][m] = __ldg(x + (int64_t)BS * col + m);
        }
    }
    template <typename Acc>
    __device__ __forceinline__ void apply(int u, Acc *acc) {
#pragma unroll
        for (int r = 0; r < BS; ++r)
#pragma unroll
            for (int m = 0; m < BS; ++m) acc[r].fma_(a[u][r * BS + m], xv[u][m]);
    }
};

// applies slots 0..rem-1 of a partial batch (1 <= rem < K+1), each case fully unrolled
template <int K>
struct SellTail {
    template <typename Bt, typename Acc>
    __device__ __forceinline__ static void run(Bt &t, int rem, Acc *acc) {
        if (rem == K) {
#pragma unroll
            for (int u = 0; u < K; ++u) t.apply(u, acc);
        } else {
            SellTail<K - 1>::run(t, rem, acc);
        }
    }
};
template <>
struct SellTail<0> {
    template <typename Bt, typename Acc>
    __device__ __forceinline__ static void run(Bt &, int, Acc *) {}
};

// One block row per lane: lane `lane` of chunk c holds row a (a < 0: padding lane, its entries
// are zero blocks on column 0), L slots starting at slot row sr.
template <typename V, int BS, int B, bool C16, typename Acc>
__device__ __forceinline__ void sell_row(const SellArgs &S, const V *__restrict__ val, const V *__restrict__ x,
                                         int L, int64_t sr, int lane, int a, Acc *acc) {
    const int ar = a < 0 ? 0 : a;
    const int64_t ce = sr * 32 + lane;
    const V *v = val + sr * (BS * BS * 32) + lane;
    int j = 0;
    for (; j + B <= L; j += B) {
        SellBatch<V, BS, B> t;
        t.template load<C16, false>(S, v, x, ce, ar, j, B);
#pragma unroll
        for (int u = 0; u < B; ++u) t.apply(u, acc);
    }
    const int rem = L - j;
    if (rem > 0) {
        SellBatch<V, BS, B> t;
        t.template load<C16, true>(S, v, x, ce, ar, j, rem);
        SellTail<B - 1>::run(t, rem, acc);
    }
}

// batch depth: scalar rows 8 or 16 slots, 3x3 blocks 2 or 4 (FP32: 4 or 8)
template <int BS, bool DEEP, bool F32 = false>
struct SellDepth {
    static constexpr int B = BS == 1 ? (DEEP ? 16 : 8) : (F32 ? (DEEP ? 8 : 4) : (DEEP ? 4 : 2));
};

// FP64 rows: LOOP 0/1 keep a plain loop unrolled UNR deep -- the large FP64 kernels are bound by
// the FP64 pipe, and the compiler's software pipelining of the unrolled loop (loads of later
// slots under the FMAs of earlier ones) measured faster there than the batched form; LOOP 2/3
// use the batched form (B = 8/16 slots, 2/4 blocks), which wins where latency, not the FP64
// pipe, sets the time (small matrices, short rows).  The tuner times all four.
struct AccF64 {
    double s = 0;
    __device__ __forceinline__ void fma_(double a, double x) { s = fma(a, x, s); }
    __device__ __forceinline__ double get() const { return s; }
};

template <int BS, bool C16, int LOOP>
__device__ __forceinline__ void sell_row64(const SellArgs &S, const double *__restrict__ val,
                                           const double *__restrict__ x, int L, int64_t sr, int lane, int a,
                                           double *y) {
    if constexpr (LOOP >= 2) {
        AccF64 acc[BS];
        sell_row<double, BS, SellDepth<BS, LOOP == 3>::B, C16>(S, val, x, L, sr, lane, a, acc);
#pragma unroll
        for (int m = 0; m < BS; ++m) y[m] = acc[m].get();
        return;
    } else {
        const int ar = a < 0 ? 0 : a;
        const int64_t ce = sr * 32 + lane;
        const double *v = val + sr * (BS * BS * 32) + lane;
        double s0 = 0, s1 = 0, s2 = 0;
        // slots in flight (the column -> gather dependency): scalar rows 8 or 16, 3x3 blocks 2 or 4
        constexpr int UNR = BS == 1 ? (LOOP ? 16 : 8) : (LOOP ? 4 : 2);
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
}

template <int BS, bool C16, bool DEEP>
__device__ __forceinline__ void sell_rowx(const SellArgs &S, const float2 *__restrict__ val,
                                          const float2 *__restrict__ x, int L, int64_t sr, int lane, int a,
                                          double *y) {
    AccDF acc[BS];
    sell_row<float2, BS, SellDepth<BS, DEEP>::B, C16>(S, val, x, L, sr, lane, a, acc);
#pragma unroll
    for (int m = 0; m < BS; ++m) y[m] = acc[m].get();
}

template <int BS, bool C16, bool DEEP>
__device__ __forceinline__ void sell_row32(const SellArgs &S, const float *__restrict__ val,
                                           const float *__restrict__ x, int L, int64_t sr, int lane, int a,
                                           float *y) {
    AccF32 acc[BS];
    sell_row<float, BS, SellDepth<BS, DEEP, true>::B, C16>(S, val, x, L, sr, lane, a, acc);
#pragma unroll
    for (int m = 0; m < BS; ++m) y[m] = acc[m].get();
}

}  // namespace ffgpu
