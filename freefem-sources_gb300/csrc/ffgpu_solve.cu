// ffgpu_solve.cu -- SpMV, Jacobi PCG (CUDA-graph loop) and FGMRES on the device.
//
// The PCG is FreeFEM's ConjugueGradient (src/femlib/CG.cpp:196-265) step for step:
//   G = Ax - b; gCg = (G, CG); H = -CG; eps2 = eps^2 gCg (eps > 0)
//   loop: rho = -(G,H)/(H,AH); x += rho H; G += rho AH; gCg' = (G,CG); gamma = gCg'/gCg;
//         H = gamma H - CG; stop when gCg' < eps2
// with C = Jacobi (1/A_ii, 1 if |A_ii|^2 < 1e-60) and x_i = b_i/tgv on tgv rows
// (VirtualSolverCG.hpp:27-99).  One iteration = three fused kernels:
//   K_a  AH = A H (SpMV) with (H,AH) -> rho                     [last block]
//   K_b  x += rho H, G += rho AH, (G, C G) -> gamma, stop test  [last block]
//   K_c  H = gamma H - C G with (G,H)                            [last block]
// CG = C G is recomputed where it is used instead of being stored.  Small scalar systems (the
// matrix in L2, an iteration bound by kernel boundaries) run two kernels per iteration: K_b
// stores C G and the next K_a forms H = gamma H - C G at every column it gathers (cg_kca_sell).
// The iteration loop is a CUDA graph `while` node whose condition K_b clears on convergence or
// at itmax, so a whole solve is one graph launch with no host round trip.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ffgpu_internal.cuh"
#include "ffgpu_sell.cuh"

namespace ffgpu {

constexpr int kSpmvWarps = 8;                 // warps per SpMV block
constexpr int kSpmvBlocks = 16 * kNumSM;      // persistent grid of the fused SpMV
constexpr int kVecBlocks = 4 * kNumSM;        // grid of the fused vector kernels
constexpr int kVecThreads = 256;

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double block_sum(double v, double *sh) { return block_sum_t(v, sh); }

// The two-kernel iteration leaves no last block behind: each kernel writes its blocks' partials
// and every block of the next kernel sums them itself, in the order the last block of the
// writing kernel would have used (thread-strided over the partials, then block_sum_t, with the
// same block size), so every block gets the bits that last block would have.
__device__ __forceinline__ double partials_total(const double *part, int n, double *sh, double *bc) {
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(part + i);
    s = block_sum_t(s, sh);
    if (threadIdx.x == 0) *bc = s;
    __syncthreads();
    s = *bc;
    __syncthreads();
    return s;
}

__device__ __forceinline__ bool last_block_total(double partial, double *part, unsigned *ticket,
                                                  double *tot, double *sh) {
    return last_block_sum(partial, part, ticket, tot, sh);
}

// cudaGraphSetConditional out of line: inlined, its call sequence raises the register count
// of the whole kernel
__device__ __noinline__ void graph_stop(cudaGraphConditionalHandle cond) { cudaGraphSetConditional(cond, 0); }

// ------------------------------------------------------------------ SpMV rows
// CSR (block size 1): T lanes per row, lanes stride the row.
template <int T>
__device__ __forceinline__ double csr_row(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                          const double *__restrict__ val, const double *__restrict__ x,
                                          int r, int sub) {
    int b = __ldg(rp + r), e = __ldg(rp + r + 1);
    double s = 0;
    for (int k = b + sub; k < e; k += T) s = fma(__ldg(val + k), __ldg(x + __ldg(col + k)), s);
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// BSR 3x3: T lanes per block row, each lane whole blocks (9 values, 3 outputs).
template <int T>
__device__ __forceinline__ void bsr3_row(const int32_t *__restrict__ brp, const int32_t *__restrict__ bcol,
                                         const double *__restrict__ val, const double *__restrict__ x,
                                         int a, int sub, double y[3]) {
    int b = __ldg(brp + a), e = __ldg(brp + a + 1);
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = b + sub; k < e; k += T) {
        int c = __ldg(bcol + k);
        const double *v = val + (int64_t)k * 9;
        double x0 = __ldg(x + 3 * (int64_t)c), x1 = __ldg(x + 3 * (int64_t)c + 1), x2 = __ldg(x + 3 * (int64_t)c + 2);
        s0 = fma(__ldg(v + 0), x0, s0); s0 = fma(__ldg(v + 1), x1, s0); s0 = fma(__ldg(v + 2), x2, s0);
        s1 = fma(__ldg(v + 3), x0, s1); s1 = fma(__ldg(v + 4), x1, s1); s1 = fma(__ldg(v + 5), x2, s1);
        s2 = fma(__ldg(v + 6), x0, s2); s2 = fma(__ldg(v + 7), x1, s2); s2 = fma(__ldg(v + 8), x2, s2);
    }
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    y[0] = s0; y[1] = s1; y[2] = s2;
}

struct SpmvArgs {
    int nb, bs;
    const int32_t *rp, *col;
    const double *val;
    const int32_t *perm;   // row order (rows of equal degree share a warp)
};

// y = A x, optionally with the partial of (w, y) (w may alias x); persistent grid.
template <int BS, int T>
__global__ void __launch_bounds__(kSpmvWarps * 32) spmv_kernel(SpmvArgs A, const double *__restrict__ x,
                                                               double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    for (int base = 0; base < A.nb; base += gridDim.x * groups) {
        const int slot = base + g;
        const bool ok = slot < A.nb;
        const int a = ok ? __ldg(A.perm + slot) : 0;
        if (BS == 1) {
            double s = csr_row<T>(A.rp, A.col, A.val, x, a, ok ? sub : T);
            if (ok && sub == 0) y[a] = s;
        } else {
            double v[3];
            bsr3_row<T>(A.rp, A.col, A.val, x, a, ok ? sub : T, v);
            if (ok && sub == 0) {
                y[3 * (int64_t)a] = v[0];
                y[3 * (int64_t)a + 1] = v[1];
                y[3 * (int64_t)a + 2] = v[2];
            }
        }
    }
}

// K_a: AH = A H and (H, AH) -> rho = -(G,H)/(H,AH)
template <int BS, int T>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_ka(SpmvArgs A, const double *__restrict__ h,
                                                         double *__restrict__ q, KrylovScalars *ks,
                                                         double *part) {
    __shared__ double sh[32];
    griddep_wait();
    if (ks->done) return;
    const int lane = threadIdx.x & 31;
    const int gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    double hq = 0;
    for (int base = 0; base < A.nb; base += gridDim.x * groups) {
        const int slot = base + g;
        const bool ok = slot < A.nb;
        const int a = ok ? __ldg(A.perm + slot) : 0;
        if (BS == 1) {
            double s = csr_row<T>(A.rp, A.col, A.val, h, a, ok ? sub : T);
            if (ok && sub == 0) { q[a] = s; hq = fma(h[a], s, hq); }
        } else {
            double v[3];
            bsr3_row<T>(A.rp, A.col, A.val, h, a, ok ? sub : T, v);
            if (ok && sub == 0) {
                int64_t i = 3 * (int64_t)a;
                q[i] = v[0]; q[i + 1] = v[1]; q[i + 2] = v[2];
                hq = fma(h[i], v[0], hq);
                hq = fma(h[i + 1], v[1], hq);
                hq = fma(h[i + 2], v[2], hq);
            }
        }
    }
    double tot;
    double p = block_sum(hq, sh);
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) {
        ks->s_hq = tot;
        ks->rho = -ks->s_gh / tot;
    }
}

// The vector kernels run on a resident grid and read/write two elements per access (all
// work vectors are 16-byte aligned); an odd last element is done by thread 0 of block 0.
// K_b: x += rho H; G += rho AH; C G into cgv (read by K_c's direction update, or by the fused
// one of cg_kca_sell); (G, C G) -> gamma, convergence.  In the two-kernel iteration (FUSED) rho
// comes from K_ca's nba pairs of partials at part (summed here by every block) and (G, C G)
// leaves as partials at part + 2 nba, summed by the next K_ca (fused_prologue).
template <bool FUSED>
__global__ void __launch_bounds__(kVecThreads) cg_kb(int n, double *__restrict__ x, double *__restrict__ g,
                                                     const double *__restrict__ h, const double *__restrict__ q,
                                                     const double *__restrict__ dinv, double *__restrict__ cgv,
                                                     KrylovScalars *ks, double *part, int nba,
                                                     cudaGraphConditionalHandle cond, int in_graph) {
    __shared__ double sh[32];
    __shared__ double bc;
    griddep_wait();
    if (ks->done) {
        if (in_graph && blockIdx.x == 0 && threadIdx.x == 0) graph_stop(cond);
        return;
    }
    double rho;
    if (FUSED) {
        const double tgh = partials_total(part, nba, sh, &bc);
        const double thq = partials_total(part + nba, nba, sh, &bc);
        rho = -tgh / thq;
        if (blockIdx.x == 0 && threadIdx.x == 0) { ks->s_gh = tgh; ks->s_hq = thq; ks->rho = rho; }
    } else {
        rho = ks->rho;
    }
    double s = 0;
    const int n2 = n >> 1;
    double2 *x2 = reinterpret_cast<double2 *>(x), *g2 = reinterpret_cast<double2 *>(g);
    const double2 *h2 = reinterpret_cast<const double2 *>(h), *q2 = reinterpret_cast<const double2 *>(q),
                  *d2 = reinterpret_cast<const double2 *>(dinv);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double2 hv = h2[i], qv = q2[i], dv = d2[i];
        double2 xv = x2[i], gv = g2[i];
        xv.x = fma(rho, hv.x, xv.x); xv.y = fma(rho, hv.y, xv.y);
        gv.x = fma(rho, qv.x, gv.x); gv.y = fma(rho, qv.y, gv.y);
        x2[i] = xv;
        g2[i] = gv;
        const double c0 = __dmul_rn(dv.x, gv.x), c1 = __dmul_rn(dv.y, gv.y);
        reinterpret_cast<double2 *>(cgv)[i] = make_double2(c0, c1);
        s = fma(gv.x, c0, s);
        s = fma(gv.y, c1, s);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int i = n - 1;
        x[i] = fma(rho, h[i], x[i]);
        const double gi = fma(rho, q[i], g[i]);
        g[i] = gi;
        const double ci = __dmul_rn(dinv[i], gi);
        cgv[i] = ci;
        s = fma(gi, ci, s);
    }
    double tot;
    double p = block_sum(s, sh);
    if (FUSED) {
        if (threadIdx.x == 0) part[2 * nba + blockIdx.x] = p;
        return;
    }
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) {
        ks->gcgp = ks->gcg;
        ks->gcg = tot;
        ks->gamma = tot / ks->gcgp;
        ks->iter += 1;
        if (tot < ks->eps2) { ks->converged = 1; ks->done = 1; }
        else if (ks->iter >= ks->itmax) ks->done = 1;
        if (ks->done && in_graph) graph_stop(cond);
    }
}

// K_c: H = gamma H - C G (C G as K_b stored it) and (G, H); with hx != NULL also the split
// copy of H for the next double-float SpMV
template <bool SPLIT>
__global__ void __launch_bounds__(kVecThreads) cg_kc_t(int n, const double *__restrict__ g, double *__restrict__ h,
                                                       float2 *__restrict__ hx, const double *__restrict__ cgv,
                                                       KrylovScalars *ks, double *part) {
    __shared__ double sh[32];
    griddep_wait();
    if (ks->done) return;
    const double gamma = ks->gamma;
    double s = 0;
    const int n2 = n >> 1;
    double2 *h2 = reinterpret_cast<double2 *>(h);
    const double2 *g2 = reinterpret_cast<const double2 *>(g), *c2 = reinterpret_cast<const double2 *>(cgv);
    float4 *hx2 = reinterpret_cast<float4 *>(hx);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double2 gv = g2[i], cv = c2[i];
        double2 hv = h2[i];
        // C G rounded once (__dmul_rn in K_b): the fused update of cg_kca_sell forms the same bits
        hv.x = fma(gamma, hv.x, -cv.x);
        hv.y = fma(gamma, hv.y, -cv.y);
        h2[i] = hv;
        if (SPLIT) {
            const float2 a = split_f64(hv.x), b = split_f64(hv.y);
            hx2[i] = make_float4(a.x, a.y, b.x, b.y);
        }
        s = fma(gv.x, hv.x, s);
        s = fma(gv.y, hv.y, s);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int i = n - 1;
        const double gi = g[i];
        const double hi = fma(gamma, h[i], -cgv[i]);
        h[i] = hi;
        if (SPLIT) hx[i] = split_f64(hi);
        s = fma(gi, hi, s);
    }
    double tot;
    double p = block_sum(s, sh);
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) ks->s_gh = tot;
}

// ------------------------------------------------------------------ double-float SpMV
// FP64 values and vectors with the products formed on the FP32 pipe (df_fma): GB300 issues 64
// FP32 FMAs per FP64 FMA, so this moves the SpMV from the FP64-pipe bound to the HBM bound.
__device__ __forceinline__ void df_add_shfl(float &S, float &C, int o) {
    float S2 = __shfl_xor_sync(0xffffffffu, S, o), C2 = __shfl_xor_sync(0xffffffffu, C, o);
    float s2, e;
    two_sum(S, S2, s2, e);
    S = s2;
    C = __fadd_rn(__fadd_rn(C, C2), e);
}

__global__ void split_kernel(int64_t n, const double *__restrict__ v, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = split_f64(v[i]);
}

struct SpmvArgsX {
    int nb, bs;
    const int32_t *rp, *col;
    const float2 *val;
    const int32_t *perm;
};

template <int T>
__device__ __forceinline__ double csr_row_x(const SpmvArgsX &A, const float2 *__restrict__ x, int r, int sub) {
    int b = __ldg(A.rp + r), e = __ldg(A.rp + r + 1);
    float S = 0.f, C = 0.f;
    for (int k = b + sub; k < e; k += T) {
        float2 a = A.val[k];
        float2 xv = x[__ldg(A.col + k)];
        df_fma(a, xv, S, C);
    }
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) df_add_shfl(S, C, o);
    return (double)S + (double)C;
}

template <int T>
__device__ __forceinline__ void bsr3_row_x(const SpmvArgsX &A, const float2 *__restrict__ x, int a, int sub,
                                           double y[3]) {
    int b = __ldg(A.rp + a), e = __ldg(A.rp + a + 1);
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f, S2 = 0.f, C2 = 0.f;
    for (int k = b + sub; k < e; k += T) {
        int c = __ldg(A.col + k);
        const float2 *v = A.val + (int64_t)k * 9;
        float2 x0 = x[3 * (int64_t)c], x1 = x[3 * (int64_t)c + 1], x2 = x[3 * (int64_t)c + 2];
        df_fma(v[0], x0, S0, C0); df_fma(v[1], x1, S0, C0); df_fma(v[2], x2, S0, C0);
        df_fma(v[3], x0, S1, C1); df_fma(v[4], x1, S1, C1); df_fma(v[5], x2, S1, C1);
        df_fma(v[6], x0, S2, C2); df_fma(v[7], x1, S2, C2); df_fma(v[8], x2, S2, C2);
    }
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) {
        df_add_shfl(S0, C0, o);
        df_add_shfl(S1, C1, o);
        df_add_shfl(S2, C2, o);
    }
    if (T >= 4) {
        // conversions to FP64 issue on the FP64 pipe: lane `sub` < 3 forms output `sub` only
        const float S = sub == 0 ? S0 : (sub == 1 ? S1 : S2), C = sub == 0 ? C0 : (sub == 1 ? C1 : C2);
        y[0] = (double)S + (double)C;
    } else {
        y[0] = (double)S0 + (double)C0;
        y[1] = (double)S1 + (double)C1;
        y[2] = (double)S2 + (double)C2;
    }
}

// K_a with the double-float SpMV: AH = A H from the split H, (H, AH) in FP64
template <int BS, int T>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_ka_x(SpmvArgsX A, const float2 *__restrict__ hx,
                                                           const double *__restrict__ h, double *__restrict__ q,
                                                           KrylovScalars *ks, double *part) {
    __shared__ double sh[32];
    griddep_wait();
    if (ks->done) return;
    const int lane = threadIdx.x & 31;
    const int gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    int g = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    double hq = 0;
    for (int base = 0; base < A.nb; base += gridDim.x * groups) {
        const int slot = base + g;
        const bool ok = slot < A.nb;
        const int a = ok ? __ldg(A.perm + slot) : 0;
        if (BS == 1) {
            double s = csr_row_x<T>(A, hx, a, ok ? sub : T);
            if (ok && sub == 0) { q[a] = s; hq = fma(h[a], s, hq); }
        } else {
            double v[3];
            bsr3_row_x<T>(A, hx, a, ok ? sub : T, v);
            if (T >= 4) {
                if (ok && sub < 3) {
                    int64_t i = 3 * (int64_t)a + sub;
                    q[i] = v[0];
                    hq = fma(h[i], v[0], hq);
                }
            } else if (ok && sub == 0) {
                int64_t i = 3 * (int64_t)a;
                q[i] = v[0]; q[i + 1] = v[1]; q[i + 2] = v[2];
                hq = fma(h[i], v[0], hq);
                hq = fma(h[i + 1], v[1], hq);
                hq = fma(h[i + 2], v[2], hq);
            }
        }
    }
    double tot;
    double p = block_sum(hq, sh);
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) {
        ks->s_hq = tot;
        ks->rho = -ks->s_gh / tot;
    }
}

// ------------------------------------------------------------------ SELL-32 K_a
// One block row per lane, one chunk of 32 rows per warp (resident grid, chunks strided over
// warps).  FP64: AH = A H and (H, AH) -> rho; padding lanes (a < 0) write nothing.
// (Six blocks per SM at 40 registers -- the unrolled loops fit without spilling -- measured
// slower than the compiler's 64 registers at four: [P2]^3 K_a 1.110 against 1.055 ms, P1
// cube(160) 0.185 against 0.146 ms; fewer loads in flight per thread.)
template <int BS, bool C16, int ASSIGN, int LOOP>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_ka_sell(SellArgs S, const double *__restrict__ val,
                                                              const double *__restrict__ h, double *__restrict__ q,
                                                              KrylovScalars *ks, double *part) {
    __shared__ double sh[32];
    griddep_wait();
    if (ks->done) return;
    const int lane = threadIdx.x & 31;
    double hq = 0;
    sell_for_chunks<ASSIGN>(S, [&](int c, int a, int L, int64_t sr) {
        double y[BS];
        sell_row64<BS, C16, LOOP>(S, val, h, L, sr, lane, a, y);
        if (a >= 0) {
#pragma unroll
            for (int m = 0; m < BS; ++m) {
                const int64_t i = (int64_t)BS * a + m;
                q[i] = y[m];
                hq = fma(h[i], y[m], hq);
            }
        }
    });
    double tot;
    double p = block_sum(hq, sh);
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) {
        ks->s_hq = tot;
        ks->rho = -ks->s_gh / tot;
    }
}

// Fused direction update and SpMV for small scalar systems (two kernels per CG iteration
// instead of three): H' = gamma H - C G is formed where it is used -- at every gathered column
// and for the lane's own row, which is written to the other H buffer -- and AH' = A H',
// (G, H') and (H', AH') -> rho come out of one pass.  C G was stored by K_b.  Each gathered
// entry costs one FP64 FMA more, so this runs only where the iteration is latency-bound.
// Prologue of K_ca (parity p of its launch): the previous K_b's (G, C G) from its partials,
// then what that K_b's last block did in the three-kernel loop -- gamma, the iteration count,
// FreeFEM's stopping test.  Every block takes the same decision; block 0 records it.  The first
// K_ca after cg_init takes gamma = 1 (cg_fuse_start).  Returns false when the solve is over.
__device__ __forceinline__ bool fused_prologue(KrylovScalars *ks, const double *partb, int nbb, int p,
                                               cudaGraphConditionalHandle cond, int in_graph, double *sh,
                                               double *bc, double *gamma) {
    const double pg = ks->fs[p ^ 1].gcg;
    const int pit = ks->fs[p ^ 1].iter, first = ks->fs[p ^ 1].first;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (first) {
        *gamma = 1.0;
        if (lead) { ks->fs[p].gcg = pg; ks->fs[p].iter = pit; ks->fs[p].first = 0; }
        return true;
    }
    const double tot = partials_total(partb, nbb, sh, bc);
    const int iter = pit + 1;
    const bool conv = tot < ks->eps2;
    const bool done = conv || iter >= ks->itmax;
    *gamma = tot / pg;
    if (lead) {
        ks->gcgp = pg;
        ks->gcg = tot;
        ks->gamma = *gamma;
        ks->iter = iter;
        ks->fs[p].gcg = tot; ks->fs[p].iter = iter; ks->fs[p].first = 0;
        if (conv) ks->converged = 1;
        if (done) {
            ks->done = 1;
            if (in_graph) graph_stop(cond);
        }
    }
    return !done;
}

template <bool C16, int ASSIGN>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_kca_sell(SellArgs S, const double *__restrict__ val,
                                                               const double *__restrict__ hold,
                                                               const double *__restrict__ cgv,
                                                               const double *__restrict__ g,
                                                               double *__restrict__ hnew, double *__restrict__ q,
                                                               KrylovScalars *ks, double *part, const double *partb,
                                                               int nbb, int parity, cudaGraphConditionalHandle cond,
                                                               int in_graph) {
    __shared__ double sh[32];
    __shared__ double bc;
    griddep_wait();
    if (ks->done) return;
    double gamma;
    if (!fused_prologue(ks, partb, nbb, parity, cond, in_graph, sh, &bc, &gamma)) return;
    const int lane = threadIdx.x & 31;
    double hq = 0, gh = 0;
    sell_for_chunks<ASSIGN>(S, [&](int c, int a, int L, int64_t sr) {
        const int ar = a < 0 ? 0 : a;
        const int64_t ce = sr * 32 + lane;
        const double *v = val + sr * 32 + lane;
        double y = 0;
#pragma unroll 8
        for (int j = 0; j < L; ++j) {
            const int col = sell_col<C16>(S, ce + (int64_t)j * 32, ar);
            const double hc = fma(gamma, __ldg(hold + col), -__ldg(cgv + col));
            y = fma(__ldcs(v + (int64_t)j * 32), hc, y);
        }
        if (a >= 0) {
            const double ha = fma(gamma, hold[a], -cgv[a]);
            hnew[a] = ha;
            q[a] = y;
            hq = fma(ha, y, hq);
            gh = fma(g[a], ha, gh);
        }
    });
    const double pgh = block_sum(gh, sh);
    const double phq = block_sum(hq, sh);
    // the partials only: K_b sums them (partials_total)
    if (threadIdx.x == 0) {
        part[blockIdx.x] = pgh;
        part[gridDim.x + blockIdx.x] = phq;
    }
}

// the same with block CSR rows (T lanes per row, rows in the degree order of rowperm)
template <int T>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_kca_csr(SpmvArgs A, const double *__restrict__ hold,
                                                              const double *__restrict__ cgv,
                                                              const double *__restrict__ g,
                                                              double *__restrict__ hnew, double *__restrict__ q,
                                                              KrylovScalars *ks, double *part, const double *partb,
                                                              int nbb, int parity, cudaGraphConditionalHandle cond,
                                                              int in_graph) {
    __shared__ double sh[32];
    __shared__ double bc;
    griddep_wait();
    if (ks->done) return;
    double gamma;
    if (!fused_prologue(ks, partb, nbb, parity, cond, in_graph, sh, &bc, &gamma)) return;
    const int lane = threadIdx.x & 31;
    const int gsub = lane / T, sub = lane % T;
    const int groups = (blockDim.x / 32) * (32 / T);
    const int gi = blockIdx.x * groups + (threadIdx.x / 32) * (32 / T) + gsub;
    double hq = 0, gh = 0;
    for (int base = 0; base < A.nb; base += gridDim.x * groups) {
        const int slot = base + gi;
        const bool ok = slot < A.nb;
        const int a = ok ? __ldg(A.perm + slot) : 0;
        const int b0 = __ldg(A.rp + a), e0 = __ldg(A.rp + a + 1);
        double y = 0;
        for (int k = b0 + (ok ? sub : T); k < e0; k += T) {
            const int col = __ldg(A.col + k);
            y = fma(__ldg(A.val + k), fma(gamma, __ldg(hold + col), -__ldg(cgv + col)), y);
        }
#pragma unroll
        for (int o = T / 2; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        if (ok && sub == 0) {
            const double ha = fma(gamma, hold[a], -cgv[a]);
            hnew[a] = ha;
            q[a] = y;
            hq = fma(ha, y, hq);
            gh = fma(g[a], ha, gh);
        }
    }
    const double pgh = block_sum(gh, sh);
    const double phq = block_sum(hq, sh);
    // the partials only: K_b sums them (partials_total)
    if (threadIdx.x == 0) {
        part[blockIdx.x] = pgh;
        part[gridDim.x + blockIdx.x] = phq;
    }
}

// the fused loop starts from H = -C G (cg_init) with gamma = 1 and C G = 0, so that its first
// update reproduces that H; the first K_ca (parity 0) reads slot 1
__global__ void cg_fuse_start(KrylovScalars *ks) {
    if (threadIdx.x == 0) {
        ks->gamma = 1.0;
        ks->fs[1].gcg = ks->gcg;
        ks->fs[1].iter = ks->iter;
        ks->fs[1].first = 1;
    }
}

// double-float: AH = A H from the split H, (H, AH) in FP64
template <int BS, bool C16, int ASSIGN, bool DEEP>
__global__ void __launch_bounds__(kSpmvWarps * 32) cg_kax_sell(SellArgs S, const float2 *__restrict__ val,
                                                               const float2 *__restrict__ hx,
                                                               const double *__restrict__ h, double *__restrict__ q,
                                                               KrylovScalars *ks, double *part) {
    __shared__ double sh[32];
    griddep_wait();
    if (ks->done) return;
    const int lane = threadIdx.x & 31;
    double hq = 0;
    sell_for_chunks<ASSIGN>(S, [&](int c, int a, int L, int64_t sr) {
        double y[BS];
        sell_rowx<BS, C16, DEEP>(S, val, hx, L, sr, lane, a, y);
        if (a >= 0) {
#pragma unroll
            for (int m = 0; m < BS; ++m) {
                const int64_t i = (int64_t)BS * a + m;
                q[i] = y[m];
                hq = fma(h[i], y[m], hq);
            }
        }
    });
    double tot;
    double p = block_sum(hq, sh);
    if (last_block_total(p, part, &ks->ticket, &tot, sh)) {
        ks->s_hq = tot;
        ks->rho = -ks->s_gh / tot;
    }
}

// y = A x (FP64)
template <int BS, bool C16, int ASSIGN, int LOOP>
__global__ void __launch_bounds__(kSpmvWarps * 32) spmv_sell(SellArgs S, const double *__restrict__ val,
                                                             const double *__restrict__ x, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    sell_for_chunks<ASSIGN>(S, [&](int c, int a, int L, int64_t sr) {
        double r[BS];
        sell_row64<BS, C16, LOOP>(S, val, x, L, sr, lane, a, r);
        if (a >= 0) {
#pragma unroll
            for (int m = 0; m < BS; ++m) y[(int64_t)BS * a + m] = r[m];
        }
    });
}

__global__ void split_vec_kernel(int n, const double *__restrict__ h, float2 *__restrict__ hx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        hx[i] = split_f64(h[i]);
}

// init: x_i = b_i/tgv on tgv rows (done before the SpMV), then with G = A x:
//   G -= b; gCg = (G, CG); H = -CG; (G,H); eps2; done if gCg < 1e-30
__global__ void cg_x0_kernel(int n, double *x, const double *b, const uint8_t *wcl, double tgv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && wcl[i]) x[i] = b[i] / tgv;
}

__global__ void __launch_bounds__(kVecThreads) cg_init(int n, double *__restrict__ g, const double *__restrict__ b,
                                                       double *__restrict__ h, const double *__restrict__ dinv,
                                                       KrylovScalars *ks, double eps, int itmax, double *part) {
    __shared__ double sh[32];
    double s1 = 0, s2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double gi = g[i] - b[i];
        g[i] = gi;
        double ci = dinv[i] * gi;
        h[i] = -ci;
        s1 = fma(gi, ci, s1);
        s2 = fma(gi, -ci, s2);
    }
    double p1 = block_sum(s1, sh);
    double p2 = block_sum(s2, sh);
    // two totals: use two passes of the last-block protocol on separate partial slots
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = p1;
        part[gridDim.x + blockIdx.x] = p2;
        __threadfence();
        unsigned t = atomicAdd(&ks->ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double a = 0, c = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        a += __ldcg(part + i);
        c += __ldcg(part + gridDim.x + i);
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        ks->gcg = a;
        ks->gcg0 = a;
        ks->gcgp = a;
        ks->s_gh = c;
        ks->eps2 = eps > 0 ? eps * eps * a : eps * eps;
        ks->iter = 0;
        ks->itmax = itmax;
        ks->converged = 0;
        ks->done = 0;
        if (a < 1e-30) { ks->done = 1; ks->converged = 2; }
        ks->ticket = 0u;
    }
}

// ------------------------------------------------------------------ Jacobi + gettgv
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// diagonal entries through the recorded diagonal block positions; max diagonal for gettgv
__global__ void diag_kernel(int64_t n, int bs, const int32_t *diagpos, const double *val, double *diag,
                            unsigned long long *maxbits) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    unsigned long long m = 0;
    if (t < n) {
        int a = (int)(t / bs), c = (int)(t % bs);
        int p = diagpos[a];
        double d = p >= 0 ? val[(int64_t)p * bs * bs + c * bs + c] : 0.0;
        diag[t] = d;
        if (p >= 0 && d > 0) m = (unsigned long long)__double_as_longlong(d);
    }
    m = warp_max_u64(m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(maxbits, m);
}

__global__ void diag_second_kernel(int64_t n, const double *diag, double top, unsigned long long *max1bits,
                                   int *count) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    unsigned long long m = 0;
    int c = 0;
    if (i < n) {
        double d = diag[i];
        if (d == top) c = 1;
        else if (d > 0 && d < top) m = (unsigned long long)__double_as_longlong(d);
    }
    m = warp_max_u64(m);
    unsigned bal = __ballot_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) {
        if (m) atomicMax(max1bits, m);
        if (bal) atomicAdd(count, __popc(bal));
    }
}

__global__ void jacobi_kernel(int64_t n, double *diag, uint8_t *wcl, double tgve, int ntgv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = diag[i];
    wcl[i] = ntgv ? (d == tgve) : 0;
    diag[i] = (d * d < 1e-60) ? 1.0 : 1.0 / d;
}

// transpose values on the (structurally symmetric) pattern: At(a,b) = A(b,a)^T blockwise
__global__ void transpose_kernel(int nb, int bs, const int32_t *brp, const int32_t *bcol, const double *val,
                                 double *valt, int *status) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nb) return;
    for (int k = brp[a]; k < brp[a + 1]; ++k) {
        int b = bcol[k];
        int lo = brp[b], hi = brp[b + 1] - 1, pos = -1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            int c = bcol[mid];
            if (c == a) { pos = mid; break; }
            if (c < a) lo = mid + 1; else hi = mid - 1;
        }
        if (pos < 0) { dev_fail(status, kDevNotFound); return; }
        for (int r = 0; r < bs; ++r)
            for (int c = 0; c < bs; ++c)
                valt[(int64_t)k * bs * bs + r * bs + c] = val[(int64_t)pos * bs * bs + c * bs + r];
    }
}

// ------------------------------------------------------------------ host side
// tuner codes of the SELL-32 kernels (one row per lane): 64 + chunk assignment
// (sell_for_chunks) + 2 * deep unroll; block CSR is coded by its lanes per row
constexpr int kSellCode = 64;
// SELL codes: kSellCode + assign + 2 * loop; loop 0/1: unrolled row loop (plain, deep), 2/3
// (FP64 kernels only): batched row loop (plain, deep)
static bool is_sell(int T) { return T >= kSellCode && T < kSellCode + 8; }
static int sell_assign(int T) { return (T - kSellCode) & 1; }
static const char *sell_name(int T) {
    static const char *names[8] = {"sell32 ranges", "sell32 rotated", "sell32 ranges deep", "sell32 rotated deep",
                                   "sell32 ranges batch", "sell32 rotated batch", "sell32 ranges batch deep",
                                   "sell32 rotated batch deep"};
    return names[T - kSellCode];
}

#define FFGPU_SELL_FN(K)                                                                             \
    static void *K##_fn(int bs, bool c16, int code) {                                               \
        void *t[3][4] = {{(void *)K<1, false, 0, false>, (void *)K<1, false, 1, false>,               \
                          (void *)K<1, false, 0, true>, (void *)K<1, false, 1, true>},                \
                         {(void *)K<1, true, 0, false>, (void *)K<1, true, 1, false>,                 \
                          (void *)K<1, true, 0, true>, (void *)K<1, true, 1, true>},                  \
                         {(void *)K<3, false, 0, false>, (void *)K<3, false, 1, false>,               \
                          (void *)K<3, false, 0, true>, (void *)K<3, false, 1, true>}};               \
        return t[bs == 3 ? 2 : (c16 ? 1 : 0)][code - kSellCode];                                     \
    }
FFGPU_SELL_FN(cg_kax_sell)
#undef FFGPU_SELL_FN
// FP64 kernels: the four row loops
#define FFGPU_SELL64_FN(K)                                                                           \
    static void *K##_fn(int bs, bool c16, int code) {                                               \
        void *t[3][8] = {{(void *)K<1, false, 0, 0>, (void *)K<1, false, 1, 0>, (void *)K<1, false, 0, 1>,   \
                          (void *)K<1, false, 1, 1>, (void *)K<1, false, 0, 2>, (void *)K<1, false, 1, 2>,   \
                          (void *)K<1, false, 0, 3>, (void *)K<1, false, 1, 3>},                          \
                         {(void *)K<1, true, 0, 0>, (void *)K<1, true, 1, 0>, (void *)K<1, true, 0, 1>,      \
                          (void *)K<1, true, 1, 1>, (void *)K<1, true, 0, 2>, (void *)K<1, true, 1, 2>,      \
                          (void *)K<1, true, 0, 3>, (void *)K<1, true, 1, 3>},                            \
                         {(void *)K<3, false, 0, 0>, (void *)K<3, false, 1, 0>, (void *)K<3, false, 0, 1>,   \
                          (void *)K<3, false, 1, 1>, (void *)K<3, false, 0, 2>, (void *)K<3, false, 1, 2>,   \
                          (void *)K<3, false, 0, 3>, (void *)K<3, false, 1, 3>}};                         \
        return t[bs == 3 ? 2 : (c16 ? 1 : 0)][code - kSellCode];                                     \
    }
FFGPU_SELL64_FN(cg_ka_sell)
FFGPU_SELL64_FN(spmv_sell)
#undef FFGPU_SELL64_FN

// lanes per block row of the block-CSR kernels
static int pick_lanes(const ffgpu_matrix *A) {
    if (A->csr_lanes > 0 && !is_sell(A->csr_lanes)) return A->csr_lanes;
    double avg = (double)A->nnzb / (double)max(1, A->nb);
    if (A->bs == 3) return avg >= 24 ? 4 : 2;
    if (avg >= 24) return 8;
    if (avg >= 10) return 4;
    return 2;
}

template <int BS>
static void *spmv_fn(int T) {
    switch (T) {
        case 1: return (void *)spmv_kernel<BS, 1>;
        case 2: return (void *)spmv_kernel<BS, 2>;
        case 4: return (void *)spmv_kernel<BS, 4>;
        case 8: return (void *)spmv_kernel<BS, 8>;
        case 16: return (void *)spmv_kernel<BS, 16>;
        default: return (void *)spmv_kernel<BS, 32>;
    }
}
template <int BS>
static void *ka_fn(int T) {
    switch (T) {
        case 1: return (void *)cg_ka<BS, 1>;
        case 2: return (void *)cg_ka<BS, 2>;
        case 4: return (void *)cg_ka<BS, 4>;
        case 8: return (void *)cg_ka<BS, 8>;
        case 16: return (void *)cg_ka<BS, 16>;
        default: return (void *)cg_ka<BS, 32>;
    }
}

template <int BS>
static void *kax_fn(int T) {
    switch (T) {
        case 1: return (void *)cg_ka_x<BS, 1>;
        case 2: return (void *)cg_ka_x<BS, 2>;
        case 4: return (void *)cg_ka_x<BS, 4>;
        case 8: return (void *)cg_ka_x<BS, 8>;
        case 16: return (void *)cg_ka_x<BS, 16>;
        default: return (void *)cg_ka_x<BS, 32>;
    }
}

static int spmv_grid(const ffgpu_matrix *A, int T) {
    int groups = kSpmvWarps * (32 / T);
    int need = (A->nb + groups - 1) / groups;
    return max(1, min(kSpmvBlocks, need));
}

static SpmvArgs spmv_args(const ffgpu_matrix *A, int trans) {
    SpmvArgs s;
    s.nb = A->nb; s.bs = A->bs; s.rp = A->browptr; s.col = A->bcol;
    s.val = trans ? A->val_t : A->val;
    s.perm = A->rowperm;
    return s;
}

// One K_a launch of the CG loop, with its argument storage.
struct KaCall {
    void *fn = nullptr;
    int grid = 0;
    SpmvArgs sa;
    SpmvArgsX sx;
    SellArgs sl;
    const double *v64 = nullptr;
    const float2 *vx = nullptr;
    const float2 *hx = nullptr;
    const double *h = nullptr;
    double *q = nullptr;
    KrylovScalars *ks = nullptr;
    double *part = nullptr;
    void *args[7];
    cudaError_t launch(cudaStream_t s, bool pdl = false) {
        return launch_ex(fn, grid, kSpmvWarps * 32, args, 0, s, pdl);
    }
};

// K_a for mode (0 FP64, 1 double-float) and layout choice T (SELL-32 codes or BSR lanes)
static int ka_setup(ffgpu_matrix *A, int mode, int trans, int T, const double *h, double *q, KaCall &k) {
    k.h = h; k.q = q; k.ks = A->ks; k.part = A->ctx->d_part; k.hx = A->hx;
    if (is_sell(T)) {
        FFGPU_TRY(sell_values(A, mode == 1 ? (trans ? kSellXT : kSellX) : (trans ? kSell64T : kSell64)));
        // the column format is known only once the layout exists
        const bool c16 = A->scol16 != nullptr;
        const bool range = sell_assign(T) == kSellRanges;
        k.sl = sell_args(A);
        if (mode == 1) {
            k.vx = trans ? A->svalx_t : A->svalx;
            k.fn = cg_kax_sell_fn(A->bs, c16, T);
            k.args[0] = &k.sl; k.args[1] = &k.vx; k.args[2] = &k.hx; k.args[3] = &k.h; k.args[4] = &k.q;
            k.args[5] = &k.ks; k.args[6] = &k.part;
        } else {
            k.v64 = trans ? A->sval_t : A->sval;
            k.fn = cg_ka_sell_fn(A->bs, c16, T);
            k.args[0] = &k.sl; k.args[1] = &k.v64; k.args[2] = &k.h; k.args[3] = &k.q; k.args[4] = &k.ks;
            k.args[5] = &k.part;
        }
        k.grid = sized_grid(k.fn, kSpmvWarps * 32, ((int64_t)A->nchunk + kSpmvWarps - 1) / kSpmvWarps);
        if (range) FFGPU_TRY(sell_partition(A, k.grid * kSpmvWarps, &k.sl.part));
        return FFGPU_OK;
    }
    if (mode == 1) {
        FFGPU_TRY(matrix_prepare_split(A, trans));
        k.sx = SpmvArgsX{A->nb, A->bs, A->browptr, A->bcol, trans ? A->valx_t : A->valx, A->rowperm};
        k.fn = A->bs == 3 ? kax_fn<3>(T) : kax_fn<1>(T);
        k.args[0] = &k.sx; k.args[1] = &k.hx; k.args[2] = &k.h; k.args[3] = &k.q; k.args[4] = &k.ks;
        k.args[5] = &k.part;
    } else {
        if (trans) FFGPU_TRY(matrix_prepare_transpose(A));
        k.sa = spmv_args(A, trans);
        k.fn = A->bs == 3 ? ka_fn<3>(T) : ka_fn<1>(T);
        k.args[0] = &k.sa; k.args[1] = &k.h; k.args[2] = &k.q; k.args[3] = &k.ks; k.args[4] = &k.part;
    }
    k.grid = spmv_grid(A, T);
    return FFGPU_OK;
}

// Candidate layouts of the K_a kernel, in the tuner's order (the first one wins ties).
// FP64 block CSR: reductions across lanes cost FP64 adds, so few lanes per row; double-float:
// reductions are FP32, so wider lane groups.
static const int kCands64[] = {kSellCode, kSellCode + 1, kSellCode + 2, kSellCode + 3, kSellCode + 4,
                               kSellCode + 5, kSellCode + 6, kSellCode + 7, 1, 2, 4, 8};
static const int kCandsX[] = {kSellCode, kSellCode + 1, kSellCode + 2, kSellCode + 3, 4, 8, 16, 32};
// matrices with fewer stored entries than this take the first candidate without timing: their
// K_a is launch-latency bound and the candidates' times differ by noise only
constexpr int64_t kTuneMinEntries = 1 << 16;

static bool layout_valid(int mode, int code) {
    const int *c = mode == 1 ? kCandsX : kCands64;
    const int n = mode == 1 ? 8 : 12;
    for (int i = 0; i < n; ++i)
        if (c[i] == code) return true;
    return false;
}

// Times the K_a kernel of one mode (0: FP64, 1: double-float) for the SELL-32 layout and for
// block CSR with each candidate lanes-per-row on this matrix, and keeps the first candidate
// within the tuner margin of the fastest (tuned_pick).  The choice is cached per matrix shape
// in the context, so every matrix of a shape gets the same layout (and the same summation
// order) for the context's lifetime.  Value arrays of the losing layout are released.
static int tune_lanes(ffgpu_matrix *A, int mode) {
    int *slot = mode == 1 ? &A->csr_lanes_x : &A->csr_lanes;
    if (*slot > 0) return FFGPU_OK;
    ffgpu_ctx *ctx = A->ctx;
    if (const int known = tuned_layout(ctx, A, mode)) {
        *slot = known;
        return FFGPU_OK;
    }
    if (!A->vec) { *slot = kSellCode; return FFGPU_OK; }
    const int *cands = mode == 1 ? kCandsX : kCands64;
    const int ncand = mode == 1 ? 8 : 12;
    const int64_t vs = vstride(A->n);
    double *y = A->vec + 6 * vs, *x = A->vec + 5 * vs;
    cudaStream_t s = ctx->stream;
    if (mode == 1 && !A->hx) FFGPU_CUDA(dalloc(ctx, (void **)&A->hx, sizeof(float2) * vs));
    int bestT = cands[0];
    if (A->nnz >= kTuneMinEntries) {
        FFGPU_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * A->n, s));
        if (mode == 1) FFGPU_CUDA(cudaMemsetAsync(A->hx, 0, sizeof(float2) * A->n, s));
        KrylovScalars *ks = A->ks;
        FFGPU_CUDA(cudaMemsetAsync(ks, 0, sizeof(KrylovScalars), s));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        // two passes over all candidates, each candidate's time the faster of its two
        float tms[12];
        for (int c = 0; c < ncand; ++c) tms[c] = 1e30f;
        for (int pass = 0; pass < 2; ++pass)
            for (int c = 0; c < ncand; ++c) {
                KaCall k;
                FFGPU_TRY(ka_setup(A, mode, 0, cands[c], x, y, k));
                k.launch(s);   // warm
                cudaEventRecord(e0, s);
                for (int r = 0; r < 3; ++r) k.launch(s);
                cudaEventRecord(e1, s);
                FFGPU_CUDA(cudaEventSynchronize(e1));
                FFGPU_CUDA(cudaGetLastError());
                ctx->launches += 4;
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                tms[c] = fminf(tms[c], ms / 3);
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        bestT = cands[tuned_pick(tms, ncand)];
        if (getenv("FFGPU_VERBOSE"))
            for (int c = 0; c < ncand; ++c)
                fprintf(stderr, "ffgpu: SpMV tuner (mode %d, %d block rows, %lld blocks): %s%s %d %.4f ms\n", mode,
                        A->nb, (long long)A->nnzb, cands[c] == bestT ? "* " : "",
                        is_sell(cands[c]) ? sell_name(cands[c]) : "bsr lanes", cands[c], tms[c]);
        FFGPU_CUDA(cudaMemsetAsync(ks, 0, sizeof(KrylovScalars), s));
        FFGPU_CUDA(cudaStreamSynchronize(s));
    }
    if (is_sell(bestT)) {
        if (mode == 1) { dfree(ctx, A->valx); A->valx = nullptr; }
    } else if (mode == 1) {
        dfree(ctx, A->svalx); A->svalx = nullptr;
    } else {
        dfree(ctx, A->sval); A->sval = nullptr;
    }
    *slot = bestT;
    tuned_store(ctx, A, mode, bestT);
    return FFGPU_OK;
}

// A layout fixed by the caller (ffgpu_solver_params.spmv_layout, else the environment variable
// FFGPU_SPMV_LAYOUT for the FP64 CG) replaces the tuned one for this matrix.
static int pin_layout(ffgpu_matrix *A, int mode, int code) {
    A->layout_pinned = 0;
    if (code == 0) {
        const char *e = mode == 0 ? getenv("FFGPU_SPMV_LAYOUT") : nullptr;
        if (!e || !e[0]) return FFGPU_OK;
        code = atoi(e);
    }
    FFGPU_CHECK(layout_valid(mode, code), FFGPU_EINVAL,
                "spmv_layout %d is not a layout of SpMV mode %d (SELL-32: 64..%d, block CSR lanes: %s)", code, mode,
                mode == 1 ? 67 : 71, mode == 1 ? "4, 8, 16, 32" : "1, 2, 4, 8");
    A->layout_pinned = 1;
    int *slot = mode == 1 ? &A->csr_lanes_x : &A->csr_lanes;
    if (*slot == code) return FFGPU_OK;
    *slot = code;
    if (A->cg_exec) { cudaGraphExecDestroy(A->cg_exec); A->cg_exec = nullptr; }
    if (!is_sell(code)) {
        // spmv() takes the SELL copy whenever it exists: drop it so every SpMV uses the pin
        ffgpu_ctx *ctx = A->ctx;
        if (mode == 1) { dfree(ctx, A->svalx); dfree(ctx, A->svalx_t); A->svalx = A->svalx_t = nullptr; }
        else { dfree(ctx, A->sval); dfree(ctx, A->sval_t); A->sval = A->sval_t = nullptr; }
    }
    return FFGPU_OK;
}

int spmv(ffgpu_matrix *A, const double *x, double *y, int trans, cudaStream_t st) {
    const double *sv = trans ? A->sval_t : A->sval;
    if (sv) {
        SellArgs sl = sell_args(A);
        const int code = is_sell(A->csr_lanes) ? A->csr_lanes : kSellCode;
        const bool range = sell_assign(code) == kSellRanges;
        void *fn = spmv_sell_fn(A->bs, A->scol16 != nullptr, code);
        const int grid = sized_grid(fn, kSpmvWarps * 32, ((int64_t)A->nchunk + kSpmvWarps - 1) / kSpmvWarps);
        if (range) FFGPU_TRY(sell_partition(A, grid * kSpmvWarps, &sl.part));
        void *args[] = {&sl, &sv, &x, &y};
        FFGPU_CUDA(cudaLaunchKernel(fn, grid, kSpmvWarps * 32, args, 0, st));
        return launch_check(A->ctx, "spmv");
    }
    if (trans) FFGPU_TRY(matrix_prepare_transpose(A));
    int T = pick_lanes(A);
    SpmvArgs s = spmv_args(A, trans);
    void *fn = A->bs == 3 ? spmv_fn<3>(T) : spmv_fn<1>(T);
    void *args[] = {&s, &x, &y};
    FFGPU_CUDA(cudaLaunchKernel(fn, spmv_grid(A, T), kSpmvWarps * 32, args, 0, st));
    return launch_check(A->ctx, "spmv");
}

int matrix_prepare_split(ffgpu_matrix *A, int trans) {
    ffgpu_ctx *ctx = A->ctx;
    if (!A->hx) FFGPU_CUDA(dalloc(ctx, (void **)&A->hx, sizeof(float2) * vstride(A->n)));
    float2 **dst = trans ? &A->valx_t : &A->valx;
    if (*dst) return FFGPU_OK;
    if (trans) FFGPU_TRY(matrix_prepare_transpose(A));
    FFGPU_CUDA(dalloc(ctx, (void **)dst, sizeof(float2) * A->nnz));
    split_kernel<<<8 * kNumSM, 256, 0, ctx->stream>>>(A->nnz, trans ? A->val_t : A->val, *dst);
    return launch_check(ctx, "split");
}

int matrix_prepare_transpose(ffgpu_matrix *A) {
    if (A->val_t) return FFGPU_OK;
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(dalloc(ctx, (void **)&A->val_t, sizeof(double) * A->nnz));
    transpose_kernel<<<(A->nb + 127) / 128, 128, 0, ctx->stream>>>(A->nb, A->bs, A->browptr, A->bcol, A->val,
                                                                   A->val_t, ctx->d_status);
    FFGPU_TRY(launch_check(ctx, "transpose"));
    return check_device_status(ctx, "transpose (pattern not structurally symmetric)");
}

int matrix_prepare_solver(ffgpu_matrix *A) {
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    int64_t n = A->n;
    if (!A->vec) {
        FFGPU_CUDA(dalloc(ctx, (void **)&A->vec, sizeof(double) * vstride(n) * 8));
        FFGPU_CUDA(dalloc(ctx, (void **)&A->diag_inv, sizeof(double) * vstride(n)));
        FFGPU_CUDA(dalloc(ctx, (void **)&A->wcl, n));
        FFGPU_CUDA(dalloc(ctx, (void **)&A->ks, sizeof(KrylovScalars)));
        FFGPU_CUDA(cudaMemsetAsync(A->ks, 0, sizeof(KrylovScalars), s));
        // pool memory comes back with an earlier object's contents: the work vectors (and
        // their padding slots) start from zero, as freshly mapped memory does
        FFGPU_CUDA(cudaMemsetAsync(A->vec, 0, sizeof(double) * vstride(n) * 8, s));
        FFGPU_CUDA(cudaMemsetAsync(A->diag_inv, 0, sizeof(double) * vstride(n), s));
    }
    FFGPU_TRY(tune_lanes(A, 0));
    if (A->ntgv >= 0) return FFGPU_OK;
    unsigned long long *bits = (unsigned long long *)ctx->d_iscratch;   // [0] max, [1] max1
    int *cnt = ctx->d_iscratch + 4;
    FFGPU_CUDA(cudaMemsetAsync(ctx->d_iscratch, 0, sizeof(int) * 8, s));
    diag_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(n, A->bs, A->diagpos, A->val, A->diag_inv, bits);
    FFGPU_TRY(launch_check(ctx, "diag"));
    unsigned long long hb[2] = {0, 0};
    FFGPU_CUDA(cudaMemcpyAsync(hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    double top;
    memcpy(&top, &hb[0], sizeof(double));
    diag_second_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(n, A->diag_inv, top, bits + 1, cnt);
    FFGPU_TRY(launch_check(ctx, "diag_second"));
    int hc = 0;
    FFGPU_CUDA(cudaMemcpyAsync(hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaMemcpyAsync(&hc, cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    double max1;
    memcpy(&max1, &hb[1], sizeof(double));
    // HashMatrix::gettgv (HashMatrix.cpp:1341-1371): no tgv when max1*1e6 > ttgv
    double ttgv = top;
    int ntgv = hc;
    if (max1 * 1e6 > ttgv) { ttgv = 0; ntgv = 0; }
    A->ntgv = ntgv;
    A->tgv_found = ttgv;
    jacobi_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(n, A->diag_inv, A->wcl, ttgv > 0 ? ttgv : 1e200, ntgv);
    return launch_check(ctx, "jacobi");
}

// grids of K_b / K_c: resident, at most 4096 blocks, no more than the n/2 double2 pairs need
static int vec_grid_kb(int n) {
    static int g = 0;
    if (!g) g = min(4096, min(resident_grid((const void *)cg_kb<false>, kVecThreads),
                              resident_grid((const void *)cg_kb<true>, kVecThreads)));
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, ((int64_t)n / 2 + kVecThreads - 1) / kVecThreads));
}
static int vec_grid_kc(int n) {
    static int g = 0;
    if (!g) g = min(4096, max(resident_grid((const void *)cg_kc_t<false>, kVecThreads),
                              resident_grid((const void *)cg_kc_t<true>, kVecThreads)));
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, ((int64_t)n / 2 + kVecThreads - 1) / kVecThreads));
}

// K_b and K_c launches (optionally with programmatic dependent launch)
static void launch_kb(bool fused, int n, double *x, double *g, const double *h, const double *q,
                      const double *dinv, double *cgv, KrylovScalars *ks, double *part, int nba,
                      cudaGraphConditionalHandle cond, int in_graph, cudaStream_t s, bool pdl) {
    void *args[] = {&n, &x, &g, &h, &q, &dinv, &cgv, &ks, &part, &nba, &cond, &in_graph};
    launch_ex(fused ? (const void *)cg_kb<true> : (const void *)cg_kb<false>, vec_grid_kb(n), kVecThreads, args, 0,
              s, pdl);
}
static void launch_kc(bool split, int n, const double *g, double *h, float2 *hx, const double *cgv,
                      KrylovScalars *ks, double *part, cudaStream_t s, bool pdl) {
    void *args[] = {&n, &g, &h, &hx, &cgv, &ks, &part};
    launch_ex(split ? (const void *)cg_kc_t<true> : (const void *)cg_kc_t<false>, vec_grid_kc(n), kVecThreads, args,
              0, s, pdl);
}

// One CG iteration (K_a K_b K_c) on stream s.
static void cg_body(KaCall &ka, int mode, int n, double *x, double *g, double *h, double *q, const double *dinv,
                    double *cgv, float2 *hx, KrylovScalars *ks, double *part, cudaGraphConditionalHandle cond,
                    int in_graph, cudaStream_t s, bool pdl = false) {
    ka.launch(s, pdl);
    launch_kb(false, n, x, g, h, q, dinv, cgv, ks, part, 0, cond, in_graph, s, pdl);
    launch_kc(mode == 1, n, g, h, mode == 1 ? hx : nullptr, cgv, ks, part, s, pdl);
}

// ------------------------------------------------------------------ fused two-kernel iteration
// Scalar FP64 systems in the SELL-32 layout whose matrix is small enough that an iteration is
// bound by kernel boundaries (the matrix and vectors stay in L2): K_ca (direction update + SpMV
// + both dots, cg_kca_sell) and K_b (storing C G).  H alternates between two buffers.
constexpr int64_t kFuseMaxEntries = 1 << 20;

struct KcaCall {
    void *fn = nullptr;
    int grid = 0;
    SellArgs sl;
    SpmvArgs sa;
    const double *v64 = nullptr, *hold = nullptr, *cgv = nullptr, *g = nullptr;
    double *hnew = nullptr, *q = nullptr;
    KrylovScalars *ks = nullptr;
    double *part = nullptr;           // this kernel's partial pairs (grid of them)
    const double *partb = nullptr;    // K_b's partials (nbb of them), after this kernel's
    int nbb = 0, parity = 0;
    cudaGraphConditionalHandle cond = 0;
    int in_graph = 0;
    void *args[14];
    cudaError_t launch(cudaStream_t s, bool pdl = false) {
        return launch_ex(fn, grid, kSpmvWarps * 32, args, 0, s, pdl);
    }
};

static bool cg_fused_fits(const ffgpu_matrix *A, int mode) {
    const char *e = getenv("FFGPU_CG_FUSE");
    if (e && e[0] == '0') return false;
    return mode == 0 && A->bs == 1 && A->nnz <= kFuseMaxEntries;
}

static int kca_setup(ffgpu_matrix *A, int trans, const double *hold, double *hnew, const double *cgv,
                     const double *g, double *q, int parity, KcaCall &k) {
    k.hold = hold; k.hnew = hnew; k.cgv = cgv; k.g = g; k.q = q;
    k.ks = A->ks; k.part = A->ctx->d_part;
    k.nbb = vec_grid_kb(A->n);
    k.parity = parity;
    if (!is_sell(A->csr_lanes)) {
        // block CSR with the tuned lanes per row
        if (trans) FFGPU_TRY(matrix_prepare_transpose(A));
        const int T = pick_lanes(A);
        k.sa = spmv_args(A, trans);
        k.fn = T == 1 ? (void *)cg_kca_csr<1> : T == 2 ? (void *)cg_kca_csr<2> : T == 4 ? (void *)cg_kca_csr<4>
                                                                                     : (void *)cg_kca_csr<8>;
        k.grid = spmv_grid(A, T);
        FFGPU_CHECK(2 * k.grid + k.nbb <= 4 * kRedBlocks, FFGPU_EINVAL,
                    "fused CG: grid %d above the reduction buffer", k.grid);
        k.partb = k.part + 2 * k.grid;
        k.args[0] = &k.sa; k.args[1] = &k.hold; k.args[2] = &k.cgv; k.args[3] = &k.g; k.args[4] = &k.hnew;
        k.args[5] = &k.q; k.args[6] = &k.ks; k.args[7] = &k.part; k.args[8] = &k.partb; k.args[9] = &k.nbb;
        k.args[10] = &k.parity; k.args[11] = &k.cond; k.args[12] = &k.in_graph;
        return FFGPU_OK;
    }
    FFGPU_TRY(sell_values(A, trans ? kSell64T : kSell64));
    const bool c16 = A->scol16 != nullptr;
    const int assign = sell_assign(A->csr_lanes);
    k.fn = c16 ? (assign ? (void *)cg_kca_sell<true, 1> : (void *)cg_kca_sell<true, 0>)
               : (assign ? (void *)cg_kca_sell<false, 1> : (void *)cg_kca_sell<false, 0>);
    k.sl = sell_args(A);
    k.grid = sized_grid(k.fn, kSpmvWarps * 32, ((int64_t)A->nchunk + kSpmvWarps - 1) / kSpmvWarps);
    // two partial slots per block in the reduction buffer, then K_b's partials
    FFGPU_CHECK(2 * k.grid + k.nbb <= 4 * kRedBlocks, FFGPU_EINVAL, "fused CG: grid %d above the reduction buffer",
                k.grid);
    k.partb = k.part + 2 * k.grid;
    if (assign == kSellRanges) FFGPU_TRY(sell_partition(A, k.grid * kSpmvWarps, &k.sl.part));
    k.v64 = trans ? A->sval_t : A->sval;
    k.args[0] = &k.sl; k.args[1] = &k.v64; k.args[2] = &k.hold; k.args[3] = &k.cgv; k.args[4] = &k.g;
    k.args[5] = &k.hnew; k.args[6] = &k.q; k.args[7] = &k.ks; k.args[8] = &k.part; k.args[9] = &k.partb;
    k.args[10] = &k.nbb; k.args[11] = &k.parity; k.args[12] = &k.cond; k.args[13] = &k.in_graph;
    return FFGPU_OK;
}

// iteration u of a body: K_ca from H buffer u % 2 into the other one, then K_b on the new H
static void cg_body_fused(KcaCall (&kc)[2], int u, int n, double *x, double *g, double *const h[2], double *q,
                          const double *dinv, double *cgv, KrylovScalars *ks, double *part,
                          cudaGraphConditionalHandle cond, int in_graph, cudaStream_t s, bool pdl = false) {
    KcaCall &k = kc[u & 1];
    k.cond = cond;
    k.in_graph = in_graph;
    k.launch(s, pdl);
    launch_kb(true, n, x, g, h[(u + 1) & 1], q, dinv, cgv, ks, part, k.grid, cond, in_graph, s, pdl);
}

// Builds (or reuses) the graph [while(cond){ (K_a K_b K_c) x unroll }] (fused: (K_ca K_b) x unroll).
static int cg_graph(ffgpu_matrix *A, int trans, int unroll, int mode, double *x, double *g, double *h, double *q,
                    bool fused, double *h2, double *cgv) {
    const int gmode = mode + (fused ? 2 : 0);
    if (A->cg_exec && A->cg_unroll == unroll && A->cg_trans == trans && A->cg_mode == gmode) return FFGPU_OK;
    if (A->cg_exec) { cudaGraphExecDestroy(A->cg_exec); A->cg_exec = nullptr; }
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    KaCall ka;
    KcaCall kc[2];
    double *const hb[2] = {h, h2};
    if (fused) {
        FFGPU_TRY(kca_setup(A, trans, h, h2, cgv, g, q, 0, kc[0]));
        FFGPU_TRY(kca_setup(A, trans, h2, h, cgv, g, q, 1, kc[1]));
    } else {
        FFGPU_TRY(ka_setup(A, mode, trans, mode == 1 ? A->csr_lanes_x : A->csr_lanes, h, q, ka));
    }
    vec_grid_kb(A->n);
    vec_grid_kc(A->n);
    // with programmatic dependent launch between the body's kernels first; a device or driver
    // that refuses the programmatic edges in a conditional body gets the plain graph
    cudaError_t e = cudaErrorUnknown;
    for (int attempt = 0; attempt < 2 && e != cudaSuccess; ++attempt) {
        const bool pdl = attempt == 0 && pdl_default();
        if (attempt == 1 && !pdl_default()) break;
        cudaGraph_t graph = nullptr, body = nullptr;
        FFGPU_CUDA(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle cond;
        FFGPU_CUDA(cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault));
        // cudaGraphNodeParams has no usable default constructor: build it in zeroed storage
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
        for (int u = 0; u < unroll; ++u) {
            if (fused)
                cg_body_fused(kc, u, A->n, x, g, hb, q, A->diag_inv, cgv, A->ks, ctx->d_part, cond, 1, s, pdl);
            else
                cg_body(ka, mode, A->n, x, g, h, q, A->diag_inv, cgv, A->hx, A->ks, ctx->d_part, cond, 1, s, pdl);
        }
        e = cudaStreamEndCapture(s, &body);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&A->cg_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            A->cg_exec = nullptr;
            cudaGetLastError();
            if (getenv("FFGPU_VERBOSE"))
                fprintf(stderr, "ffgpu: CG graph %s programmatic launch failed: %s\n", pdl ? "with" : "without",
                        cudaGetErrorString(e));
        }
    }
    if (e != cudaSuccess) {
        set_error("CG graph capture failed: %s", cudaGetErrorString(e));
        return FFGPU_ECUDA;
    }
    A->cg_unroll = unroll;
    A->cg_trans = trans;
    A->cg_mode = gmode;
    A->cg_kernels_body = (fused ? 2 : 3) * unroll;
    return FFGPU_OK;
}

// one right-hand side; x/b device pointers of length n
static int cg_one(ffgpu_matrix *A, const double *b, double *x, int trans, const ffgpu_solver_params *prm,
                  ffgpu_solver_stats *st) {
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    int n = A->n;
    const int64_t vs = vstride(n);
    // the cached graph only ever touches matrix-owned buffers: the caller's x is staged in
    // slot 4 of the work vectors and copied back after the solve
    double *g = A->vec, *h = A->vec + vs, *q = A->vec + 2 * vs;
    double *xu = x;
    x = A->vec + 4 * vs;
    double tgv = prm->tgv > 0 ? prm->tgv : 1e30;
    int itmax = prm->itmax > 0 ? prm->itmax : n;
    int unroll = prm->unroll > 0 ? prm->unroll : 8;
    const int mode = prm->spmv_mode == 1 ? 1 : 0;
    // the second H buffer and C G of the fused iteration
    double *h2 = A->vec + 7 * vs, *cgv = A->vec + 3 * vs;
    if (mode == 1) {
        if (!A->hx) FFGPU_CUDA(dalloc(ctx, (void **)&A->hx, sizeof(float2) * vs));
        FFGPU_TRY(tune_lanes(A, 1));
    }
    // small scalar systems: the whole iteration loop in one thread-block cluster
    // (ffgpu_cluster.cu), unless a layout is fixed by the caller
    const bool cluster = mode == 0 && !A->layout_pinned && cluster_cg_fits(A, trans);
    A->last_cluster = cluster;
    const bool fused = !cluster && cg_fused_fits(A, mode);
    if (fused) unroll += unroll & 1;   // the H buffers alternate: an even number of iterations per body
    if (!cluster) FFGPU_TRY(cg_graph(A, trans, unroll, mode, x, g, h, q, fused, h2, cgv));
    FFGPU_CUDA(cudaMemcpyAsync(x, xu, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (A->ntgv > 0) {
        cg_x0_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, x, b, A->wcl, tgv);
        FFGPU_TRY(launch_check(ctx, "cg_x0"));
    }
    FFGPU_TRY(spmv(A, x, g, trans, s));
    cg_init<<<kVecBlocks, kVecThreads, 0, s>>>(n, g, b, h, A->diag_inv, A->ks, prm->eps, itmax, ctx->d_part);
    FFGPU_TRY(launch_check(ctx, "cg_init"));
    if (mode == 1) {
        split_vec_kernel<<<kVecBlocks, kVecThreads, 0, s>>>(n, h, A->hx);
        FFGPU_TRY(launch_check(ctx, "split_vec"));
    }
    if (fused) {
        FFGPU_CUDA(cudaMemsetAsync(cgv, 0, sizeof(double) * n, s));
        cg_fuse_start<<<1, 32, 0, s>>>(A->ks);
        FFGPU_TRY(launch_check(ctx, "cg_fuse_start"));
    }
    const char *ge = getenv("FFGPU_CG_GRAPH");
    int bodies_host = -1;
    bool use_graph = !cluster;
    if (cluster) {
        const int rc = cluster_cg_run(A, trans, x, g, h, s);
        if (rc == kClusterRefused) {
            // the device refused this cluster shape: the regular path from the same state
            A->last_cluster = 0;
            FFGPU_TRY(cg_graph(A, trans, unroll, mode, x, g, h, q, false, h2, cgv));
            use_graph = true;
        } else {
            FFGPU_TRY(rc);
            bodies_host = 0;
        }
    }
    if (use_graph && ge && ge[0] == '0') {
        // Same kernels launched from the host (for profilers that do not trace conditional
        // graph nodes): poll the done flag after every `unroll` iterations.
        KaCall ka;
        KcaCall kc[2];
        double *const hb[2] = {h, h2};
        if (fused) {
            FFGPU_TRY(kca_setup(A, trans, h, h2, cgv, g, q, 0, kc[0]));
            FFGPU_TRY(kca_setup(A, trans, h2, h, cgv, g, q, 1, kc[1]));
        } else {
            FFGPU_TRY(ka_setup(A, mode, trans, mode == 1 ? A->csr_lanes_x : A->csr_lanes, h, q, ka));
        }
        bodies_host = 0;
        for (int it = 0; it <= itmax; it += unroll) {
            for (int u = 0; u < unroll; ++u) {
                if (fused)
                    cg_body_fused(kc, u, n, x, g, hb, q, A->diag_inv, cgv, A->ks, ctx->d_part, 0, 0, s);
                else
                    cg_body(ka, mode, n, x, g, h, q, A->diag_inv, cgv, A->hx, A->ks, ctx->d_part, 0, 0, s);
            }
            ++bodies_host;
            int done = 0;
            FFGPU_CUDA(cudaMemcpyAsync(&done, &A->ks->done, sizeof(int), cudaMemcpyDeviceToHost, s));
            FFGPU_CUDA(cudaStreamSynchronize(s));
            if (done) break;
        }
    } else if (use_graph) {
        FFGPU_CUDA(cudaGraphLaunch(A->cg_exec, s));
    }
    FFGPU_CUDA(cudaMemcpyAsync(xu, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    cudaEventRecord(e1, s);
    KrylovScalars hk;
    FFGPU_CUDA(cudaMemcpyAsync(&hk, A->ks, sizeof(hk), cudaMemcpyDeviceToHost, s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // graph bodies run: the three-kernel loop stops in the body of its last K_b; the fused one
    // in the body of the K_ca after it (K_ca number iter counted from 0)
    int bodies = bodies_host >= 0 ? bodies_host
                                  : (fused ? hk.iter / unroll + 1 : (hk.iter == 0 ? 1 : (hk.iter + unroll - 1) / unroll));
    if (use_graph) ctx->launches += (int64_t)bodies * A->cg_kernels_body;
    if (st) {
        st->iterations = hk.iter;
        st->converged = hk.converged != 0;
        st->gcg = hk.gcg;
        st->eps2 = hk.eps2;
        st->elapsed_ms += ms;
    }
    return hk.converged ? FFGPU_OK : FFGPU_ENOCONV;
}

}  // namespace ffgpu

using namespace ffgpu;

typedef int (*one_solver)(ffgpu_matrix *, const double *, double *, int, const ffgpu_solver_params *,
                          ffgpu_solver_stats *);

static int solve_many(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                      const ffgpu_solver_params *prm, ffgpu_solver_stats *stats, one_solver fn) {
    FFGPU_CHECK(A && b && x && prm && nrhs >= 1, FFGPU_EINVAL, "solve: bad argument");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    int64_t n = A->n;
    FFGPU_TRY(pin_layout(A, fn == cg_one && prm->spmv_mode == 1 ? 1 : 0, prm->spmv_layout));
    FFGPU_TRY(matrix_prepare_solver(A));
    if (trans) FFGPU_TRY(matrix_prepare_transpose(A));
    DevIn<double> bd(b, (size_t)n * nrhs, ctx);
    DevOut<double> xd(x, (size_t)n * nrhs, ctx, true);
    FFGPU_TRY(bd.err);
    FFGPU_TRY(xd.err);
    ffgpu_solver_stats acc;
    memset(&acc, 0, sizeof(acc));
    int err = 0, total_it = 0;
    ffgpu_solver_stats one;
    for (int k = 0; k < nrhs; ++k) {
        memset(&one, 0, sizeof(one));
        int r = fn(A, bd.d + k * n, xd.d + k * n, trans, prm, &one);
        if (r == FFGPU_ENOCONV) err++;
        else if (r != FFGPU_OK) return r;
        total_it += one.iterations;
        acc.elapsed_ms += one.elapsed_ms;
    }
    FFGPU_TRY(xd.finish());
    if (stats) {
        *stats = one;
        stats->iterations = nrhs == 1 ? one.iterations : total_it;
        stats->elapsed_ms = acc.elapsed_ms;
        stats->converged = err == 0;
    }
    if (err) {
        set_error("Krylov solver did not converge for %d of %d right-hand sides", err, nrhs);
        return FFGPU_ENOCONV;
    }
    return FFGPU_OK;
}

extern "C" {

int ffgpu_solve_cg(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                   const ffgpu_solver_params *prm, ffgpu_solver_stats *stats) {
    return solve_many(A, b, x, nrhs, trans, prm, stats, cg_one);
}

int ffgpu_solve_gmres(ffgpu_matrix *A, const double *b, double *x, int nrhs, int trans,
                      const ffgpu_solver_params *prm, ffgpu_solver_stats *stats) {
    return solve_many(A, b, x, nrhs, trans, prm, stats, gmres_one);
}

int ffgpu_matrix_spmv_layout(const ffgpu_matrix *A, int mode) {
    if (!A) return 0;
    if (mode == 3) return A->scol16 != nullptr;
    if (mode == 5) return A->last_cluster;
    if (mode == 4) return A->nslot > 0 && A->nslot * 32 <= INT32_MAX ? (int)(A->nslot * 32) : (A->nslot ? -1 : 0);
    return mode == 2 ? A->sell32_kind : (mode == 1 ? A->csr_lanes_x : A->csr_lanes);
}

int ffgpu_matrix_time_spmv(ffgpu_matrix *A, int mode, int nrep, float *ms) {
    FFGPU_CHECK(A && ms && nrep > 0 && mode >= 0 && mode <= 2, FFGPU_EINVAL,
                "ffgpu_matrix_time_spmv: bad argument");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    if (mode == 2) return ir_time_ka(A, nrep, ms);
    const int T = mode == 1 ? A->csr_lanes_x : A->csr_lanes;
    FFGPU_CHECK(A->vec && T > 0 && (mode == 0 || A->hx), FFGPU_EINVAL,
                "ffgpu_matrix_time_spmv: solve the matrix in mode %d first", mode);
    cudaStream_t s = ctx->stream;
    const int64_t vs = vstride(A->n);
    KaCall k;
    // input: the staged solution of the last solve; output: the tuner's scratch vector
    FFGPU_TRY(ka_setup(A, mode, 0, T, A->vec + 4 * vs, A->vec + 6 * vs, k));
    // K_a returns at once when the Krylov scalars say the solve is done: clear them
    FFGPU_CUDA(cudaMemsetAsync(A->ks, 0, sizeof(KrylovScalars), s));
    cudaEvent_t e0, e1;
    FFGPU_CUDA(cudaEventCreate(&e0));
    FFGPU_CUDA(cudaEventCreate(&e1));
    k.launch(s);
    cudaEventRecord(e0, s);
    for (int r = 0; r < nrep; ++r) k.launch(s);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->launches += nrep + 1;
    FFGPU_CUDA(e);
    FFGPU_CUDA(cudaGetLastError());
    // the fused dot left partial sums in the Krylov scalars: clear them as the tuner does
    FFGPU_CUDA(cudaMemsetAsync(A->ks, 0, sizeof(KrylovScalars), s));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    *ms = t / nrep;
    return FFGPU_OK;
}

int ffgpu_matrix_mult(ffgpu_matrix *A, const double *x, double *y, int trans) {
    FFGPU_CHECK(A && x && y, FFGPU_EINVAL, "ffgpu_matrix_mult: NULL argument");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevIn<double> xd(x, A->n, ctx);
    DevOut<double> yd(y, A->n, ctx, false);
    FFGPU_TRY(xd.err);
    FFGPU_TRY(yd.err);
    FFGPU_TRY(spmv(A, xd.d, yd.d, trans, s));
    FFGPU_TRY(yd.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

}  // extern "C"
