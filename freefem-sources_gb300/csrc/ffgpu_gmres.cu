// ffgpu_gmres.cu -- FreeFEM's right-preconditioned FGMRES (CG.cpp:348-517, driven by
// SolverGMRES::dosolver, VirtualSolverCG.hpp:195-257) on the device.
//
// FreeFEM's Arnoldi step orthogonalises w = A C v_it against v_0..v_it by modified Gram-Schmidt:
//   for i = 0..it: H(i,it) = (w, v_i); w -= H(i,it) v_i
// i.e. 2(it+1) dependent passes over n-vectors.  Here the same coefficients come from ONE pass:
// with s_i = (w_0, v_i) (the unmodified w) and the Gram entries G(i,j) = (v_i, v_j), j < i,
// modified Gram-Schmidt's coefficients are the solution of the unit lower-triangular system
//   h_i = s_i - sum_{j<i} h_j G(i,j)
// (low-synchronisation MGS, Swirydowicz, Langou, Ananthan, Yang & Thomas, Numer. Linear Algebra
// Appl. 28 (2021)).  The new Gram row G(it, .) = (v_it, v_j) is formed in the same pass as s.
// The recurrence is evaluated to first order in the Gram entries, h = s - L s with L the strictly
// lower Gram triangle: the dropped terms are O(|L|^2 |s|), below the rounding of s itself while
// the basis is orthonormal to working accuracy, and the coefficients then come from a parallel
// matrix-vector product instead of a sequential substitution (GB300 runs ~2 FP64 FMAs per clock
// per SM: O(it^2) sequential work in one block cost more than the whole step at it ~ 500).
// One Arnoldi step is five kernels, none with a host round trip:
//   gm_prep    v_it *= 1/||w_prev|| (FreeFEM's Vi[it] = (1/aux) w), vp = C v_it (Jacobi)
//   SpMV       w = A vp
//   gm_dots    s = V' w and the Gram row in one pass over V: blocks are (slab of the vectors'
//              elements) x (group of basis vectors), w and v_it of a slab staged in shared
//              memory, one warp reduction per vector per 2048 elements; last block: the sums
//   gm_coef    h = s - L s (a warp per row, all SMs)
//   gm_update  v_{it+1} = w - V h, ||v_{it+1}||^2; last block: Givens rotations of the new
//              Hessenberg column (staged in shared memory), residual estimate |g_{it+1}|,
//              FreeFEM's stopping tests
// and the Arnoldi loop of one restart cycle is a CUDA-graph `while` node.  The host reads the
// scalars once per restart cycle.  All reductions sum in a fixed order (warp order inside a
// block, block order across blocks), so results are reproducible run to run.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ffgpu_internal.cuh"
#include "ffgpu_sell.cuh"

namespace ffgpu {

constexpr int kGmThreads = 256;
constexpr int kGmWarps = kGmThreads / 32;
constexpr int kGmSub = 2048;                 // elements of w and v_it staged per sub-tile of gm_dots
constexpr int kGmMaxSlabs = 256;             // slabs of gm_dots (partials summed by its last block)
constexpr int kGmHs = 1024;                  // Hessenberg columns up to this length stay in shared memory

struct GmScal {
    double normb, relres, eps;
    int it, iter, itmax, m, conv, stop, steps, itf;
    unsigned ticket;
};

struct GmArgs {
    int n, m;
    int64_t vs;
    int nslab, ngrp;                         // gm_dots grid: nslab x ngrp blocks
    int64_t slab_len;                        // elements per slab (a multiple of kGmSub)
    double *V, *Vp, *vpc, *w, *x;
    const double *b, *dinv;
    const uint8_t *wcl;
    int use_wcl;
    double *H, *rot0, *rot1, *g, *y, *vnorm, *Gm, *h, *red, *part;
    GmScal *sc;
    cudaGraphConditionalHandle cond;
    int in_graph;
};

__device__ __noinline__ void gm_set_cond(cudaGraphConditionalHandle c, unsigned v) { cudaGraphSetConditional(c, v); }

// Last-block protocol for a vector of K partial sums per block: part[k * gridDim.x + block].
// Returns true in the last block to finish (all its threads), after red[k] = sum over blocks in
// block order (one warp per k, lanes striding the blocks, fixed shuffle tree).
__device__ bool gm_last_block(const double *mine, int K, double *part, double *red, unsigned *ticket) {
    __shared__ bool s_last;
    for (int k = threadIdx.x; k < K; k += blockDim.x) part[(int64_t)k * gridDim.x + blockIdx.x] = mine[k];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = warp; k < K; k += blockDim.x >> 5) {
        double s = 0;
        for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(part + (int64_t)k * gridDim.x + b);
        s = warp_sum(s);
        if (lane == 0) red[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// block sum of one value per thread into sh[0] (sh: kGmWarps doubles + 1)
__device__ double gm_block_sum(double v, double *sh) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    v = warp_sum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kGmWarps; ++w) t += sh[w];
        sh[kGmWarps] = t;
    }
    __syncthreads();
    return sh[kGmWarps];
}

// ||b||, the tgv rows left out (FreeFEM zeroes them in wi before mysnrm2); initialises the scalars
__global__ void __launch_bounds__(kGmThreads) gm_init(GmArgs a, double eps, int itmax) {
    __shared__ double sh[kGmWarps + 1];
    double s = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        const double v = (a.use_wcl && a.wcl[k]) ? 0.0 : a.b[k];
        s = fma(v, v, s);
    }
    const double t = gm_block_sum(s, sh);
    if (gm_last_block(&t, 1, a.part, a.red, &a.sc->ticket) && threadIdx.x == 0) {
        GmScal *c = a.sc;
        c->normb = sqrt(a.red[0]);
        c->relres = 1e100;
        c->eps = eps;
        c->iter = 0;
        c->itmax = itmax;
        c->m = a.m;
        c->conv = 0;
        c->steps = 0;
    }
}

// start of a restart cycle: V[0] holds A x; r = -(A x - b) into V[0], g[0] = ||r||
__global__ void __launch_bounds__(kGmThreads) gm_resid(GmArgs a) {
    __shared__ double sh[kGmWarps + 1];
    double s = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        const double r = -(a.V[k] - a.b[k]);
        a.V[k] = r;
        s = fma(r, r, s);
    }
    const double t = gm_block_sum(s, sh);
    if (gm_last_block(&t, 1, a.part, a.red, &a.sc->ticket) && threadIdx.x == 0) {
        GmScal *c = a.sc;
        const double g0 = sqrt(a.red[0]);
        a.g[0] = g0;
        a.vnorm[0] = g0;
        if (c->normb < 1.e-20 || c->eps < 0) c->normb = 1.;
        c->it = 0;
        c->stop = 0;
        // an exact initial guess: FreeFEM would divide by zero here; the solve is converged
        if (g0 == 0.0) {
            c->conv = 1;
            c->stop = 1;
            c->relres = 0.0;
            c->itf = -1;
            if (a.in_graph) gm_set_cond(a.cond, 0);
        }
    }
}

// v_it *= 1/||.|| (FreeFEM: Vi[it] = (1./aux)*wi), vp = C v_it into Vp[it] and the SpMV input
__global__ void __launch_bounds__(kGmThreads) gm_prep(GmArgs a) {
    const int it = a.sc->it;
    double *v = a.V + it * a.vs, *vp = a.Vp + it * a.vs;
    const double inv = 1. / a.vnorm[it];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        const double vk = inv * v[k];
        v[k] = vk;
        const double p = a.dinv[k] * vk;
        vp[k] = p;
        a.vpc[k] = p;
    }
}

// s_i = (w, v_i), i <= it, and the Gram row (v_it, v_j), j < it, in one pass over V.
// Block (slab, group): the elements [slab * slab_len, +slab_len) of the vectors i = group +
// ngrp * r; per sub-tile of kGmSub elements w and v_it are staged in shared memory and each warp
// runs its vectors over the sub-tile (64 elements per lane, then one warp reduction per sum).
// Partials part[k * nslab + slab], k < 2(it+1); the last block sums them in slab order.
__global__ void __launch_bounds__(kGmThreads) gm_dots(GmArgs a) {
    extern __shared__ __align__(16) double smd[];
    double *wsh = smd, *vsh = smd + kGmSub, *acc = smd + 2 * kGmSub;
    const int it = a.sc->it;
    const int ni = it + 1, K = 2 * ni;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slab = blockIdx.x % a.nslab, grp = blockIdx.x / a.nslab;
    for (int k = threadIdx.x; k < K; k += blockDim.x) acc[k] = 0;
    const double *vit = a.V + it * a.vs;
    const int64_t e0 = (int64_t)slab * a.slab_len;
    const int64_t e1 = e0 + a.slab_len < a.n ? e0 + a.slab_len : (int64_t)a.n;
    for (int64_t t0 = e0; t0 < e1; t0 += kGmSub) {
        const int len = e1 - t0 < kGmSub ? (int)(e1 - t0) : kGmSub;
        __syncthreads();   // the previous sub-tile's readers are done (and acc is zeroed)
        for (int e = threadIdx.x; e < len; e += blockDim.x) {
            wsh[e] = a.w[t0 + e];
            vsh[e] = vit[t0 + e];
        }
        __syncthreads();
        const int len2 = len & ~1;   // pairs of elements as 16-byte loads; an odd last element apart
        for (int i = grp + a.ngrp * warp; i < ni; i += a.ngrp * kGmWarps) {
            const double *vi = a.V + i * a.vs + t0;   // 16-byte aligned: vs and t0 are even
            double ts = 0, tl = 0;
#pragma unroll 8
            for (int e = 2 * lane; e < len2; e += 64) {
                const double2 q = __ldcs(reinterpret_cast<const double2 *>(vi + e));
                const double2 w2 = *reinterpret_cast<const double2 *>(wsh + e);
                const double2 v2 = *reinterpret_cast<const double2 *>(vsh + e);
                ts = fma(q.x, w2.x, ts);
                tl = fma(q.x, v2.x, tl);
                ts = fma(q.y, w2.y, ts);
                tl = fma(q.y, v2.y, tl);
            }
            if (len2 < len && lane == 0) {
                const double q = __ldcs(vi + len2);
                ts = fma(q, wsh[len2], ts);
                tl = fma(q, vsh[len2], tl);
            }
            ts = warp_sum(ts);
            tl = warp_sum(tl);
            if (lane == 0) { acc[i] += ts; acc[ni + i] += tl; }   // vector i belongs to this warp
        }
    }
    __syncthreads();
    for (int i = grp + a.ngrp * warp; i < ni; i += a.ngrp * kGmWarps)
        if (lane == 0) {
            a.part[(int64_t)i * a.nslab + slab] = acc[i];
            a.part[(int64_t)(ni + i) * a.nslab + slab] = acc[ni + i];
        }
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&a.sc->ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int ld = a.m + 1;
    // a thread per sum, slabs in order (independent loads in flight, no shuffle chain per sum)
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const double *pk = a.part + (int64_t)k * a.nslab;
        double t = 0;
        for (int b = 0; b < a.nslab; ++b) t += __ldcg(pk + b);
        if (k < ni) a.red[k] = t;                                    // s
        else if (k - ni < it) a.Gm[(int64_t)it * ld + (k - ni)] = t;   // Gram row of v_it
    }
    __syncthreads();
    if (threadIdx.x == 0) a.sc->ticket = 0u;
}

// modified Gram-Schmidt's coefficients of this step to first order in the Gram entries:
// h_i = s_i - sum_{j<i} G(i,j) s_j (a warp per row, rows over the whole grid)
__global__ void __launch_bounds__(kGmThreads) gm_coef(GmArgs a) {
    const int it = a.sc->it;
    const int ni = it + 1, ld = a.m + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = blockIdx.x * kGmWarps + warp; i < ni; i += gridDim.x * kGmWarps) {
        const double *gi = a.Gm + (int64_t)i * ld;
        double t = 0;
        for (int j = lane; j < i; j += 32) t = fma(__ldcg(gi + j), __ldcg(a.red + j), t);
        t = warp_sum(t);
        if (lane == 0) {
            const double hi = __ldcg(a.red + i) - t;
            a.h[i] = hi;
            a.H[(int64_t)i * ld + it] = hi;
        }
    }
}

// v_{it+1} = w - sum_i h_i v_i (FreeFEM's order: i = 0..it), ||v_{it+1}||^2; last block: the
// Hessenberg column's Givens rotations and FreeFEM's stopping tests
__global__ void __launch_bounds__(kGmThreads) gm_update(GmArgs a) {
    __shared__ double hs[kGmHs], rc[kGmHs], rs[kGmHs];
    __shared__ double sh[kGmWarps + 1];
    const int it = a.sc->it;
    const int ni = it + 1;
    const double *hh = a.h;
    const bool in_smem = ni <= kGmHs;
    if (in_smem)
        for (int i = threadIdx.x; i < ni; i += blockDim.x) hs[i] = a.h[i];
    __syncthreads();
    if (in_smem) hh = hs;
    double *vn = a.V + (it + 1) * a.vs;
    double s = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        double t = a.w[k];
        // FreeFEM's order i = 0..it; the loads of 16 vectors are issued before their products,
        // and the next 16 before the products of these (two batches in flight)
        int i = 0;
        if (ni >= 16) {
            double q[16], r[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) q[u] = __ldcs(a.V + (i + u) * a.vs + k);
            for (; i + 32 <= ni; i += 16) {
#pragma unroll
                for (int u = 0; u < 16; ++u) r[u] = __ldcs(a.V + (i + 16 + u) * a.vs + k);
#pragma unroll
                for (int u = 0; u < 16; ++u) t = fma(-hh[i + u], q[u], t);
#pragma unroll
                for (int u = 0; u < 16; ++u) q[u] = r[u];
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) t = fma(-hh[i + u], q[u], t);
            i += 16;
        }
        for (; i < ni; ++i) t = fma(-hh[i], __ldcs(a.V + i * a.vs + k), t);
        vn[k] = t;
        s = fma(t, t, s);
    }
    const double tot = gm_block_sum(s, sh);
    if (!gm_last_block(&tot, 1, a.part, a.red + 2 * (a.m + 1), &a.sc->ticket)) return;
    GmScal *c = a.sc;
    const int ld = a.m + 1;
    double *H = a.H;
    const double aux = sqrt(a.red[2 * (a.m + 1)]);
    // the new column's rotations by the earlier ones: a chain through i, staged in shared memory
    double *col = in_smem ? hs : nullptr;
    if (in_smem) {
        for (int i = threadIdx.x; i < it; i += blockDim.x) {
            rc[i] = a.rot0[i];
            rs[i] = a.rot1[i];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.vnorm[it + 1] = aux;
        if (in_smem) {
            double hi = col[0];
            for (int i = 0; i < it; i++) {
                const double hi1 = col[i + 1];
                const double aa = rc[i] * hi + rs[i] * hi1;
                const double bb = -rs[i] * hi + rc[i] * hi1;
                col[i] = aa;
                hi = bb;
            }
            col[it] = hi;
        } else {
            for (int i = 0; i < it; i++) {
                const double hi = H[(int64_t)i * ld + it], hi1 = H[(int64_t)(i + 1) * ld + it];
                const double aa = a.rot0[i] * hi + a.rot1[i] * hi1;
                const double bb = -a.rot1[i] * hi + a.rot0[i] * hi1;
                H[(int64_t)i * ld + it] = aa;
                H[(int64_t)(i + 1) * ld + it] = bb;
            }
        }
        const double hd = in_smem ? col[it] : H[(int64_t)it * ld + it], hs1 = aux;
        const double sq = sqrt(hd * hd + hs1 * hs1);
        a.rot0[it] = hd / sq;
        a.rot1[it] = hs1 / sq;
        const double top = a.rot0[it] * hd + a.rot1[it] * hs1;
        if (in_smem) col[it] = top; else H[(int64_t)it * ld + it] = top;
        H[(int64_t)(it + 1) * ld + it] = 0.;
        a.g[it + 1] = -a.rot1[it] * a.g[it];
        a.g[it] = a.rot0[it] * a.g[it];
        const double relres = fabs(a.g[it + 1]);
        c->relres = relres;
        c->steps += 1;
        c->itf = it;
        bool stop = false;
        if (relres / c->normb < fabs(c->eps)) {
            c->conv = 1;
            stop = true;
        } else if (it > c->itmax) {
            stop = true;                       // FreeFEM: `if (it > nbitermx) break;`
        } else {
            c->it = it + 1;                    // the loop increment it++, iter++
            c->iter += 1;
            if (it + 1 >= a.m) { stop = true; c->itf = a.m - 1; }
        }
        c->stop = stop;
        if (stop && a.in_graph) gm_set_cond(a.cond, 0);
    }
    if (in_smem) {
        __syncthreads();
        for (int i = threadIdx.x; i <= it; i += blockDim.x) H[(int64_t)i * ld + it] = col[i];
    }
}

// y = H^-1 g on the it+1 leading rows (back substitution, one warp per row dot)
__global__ void gm_back(GmArgs a) {
    const int it = a.sc->itf;
    if (it < 0) return;
    const int ld = a.m + 1, lane = threadIdx.x;
    for (int i = it; i >= 0; i--) {
        double t = 0;
        for (int j = i + 1 + lane; j < it + 1; j += 32) t = fma(a.H[(int64_t)i * ld + j], a.y[j], t);
        t = warp_sum(t);
        if (lane == 0) a.y[i] = (a.g[i] - t) / a.H[(int64_t)i * ld + i];
        __syncwarp();
    }
}

// x = (sum_i y_i Vp_i) + x  (FreeFEM: wi = 0; wi += y_i Vpi[i]; uni = wi + x0)
__global__ void __launch_bounds__(kGmThreads) gm_xupd(GmArgs a) {
    const int it = a.sc->itf;
    if (it < 0) return;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        double t = 0;
        int i = 0;
        for (; i + 16 <= it + 1; i += 16) {
            double q[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) q[u] = __ldcs(a.Vp + (i + u) * a.vs + k);
#pragma unroll
            for (int u = 0; u < 16; ++u) t = fma(a.y[i + u], q[u], t);
        }
        for (; i <= it; ++i) t = fma(a.y[i], __ldcs(a.Vp + i * a.vs + k), t);
        a.x[k] = t + a.x[k];
    }
}

__global__ void gm_x0_kernel(int n, double *x, const double *b, const uint8_t *wcl, double tgv) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && wcl[i]) x[i] = b[i] / tgv;
}

// grids: vector kernels resident and capped by the work; the dot kernel by tiles
static int gm_vec_grid(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(4 * kNumSM, (n + kGmThreads - 1) / kGmThreads));
}
// gm_dots: sub-tiles of kGmSub elements grouped into at most kGmMaxSlabs slabs, and enough
// vector groups for about two blocks per SM
static void gm_dot_shape(int64_t n, int &nslab, int &ngrp, int64_t &slab_len) {
    const int64_t nsub = std::max<int64_t>(1, (n + kGmSub - 1) / kGmSub);
    const int64_t per = (nsub + kGmMaxSlabs - 1) / kGmMaxSlabs;
    nslab = (int)((nsub + per - 1) / per);
    slab_len = per * kGmSub;
    // at most two blocks per SM (a block is 8 warps and ~49 KB of shared memory): a third block on
    // some SMs sets the kernel's time while most SMs idle
    ngrp = std::max(1, (2 * kNumSM) / nslab);
}
static int gm_coef_grid(int m) { return std::max(1, std::min(kNumSM, (m + 1 + kGmWarps - 1) / kGmWarps)); }

// one right-hand side; b, x device pointers of length n (x: initial guess, then solution)
int gmres_one(ffgpu_matrix *A, const double *b, double *x, int trans, const ffgpu_solver_params *prm,
              ffgpu_solver_stats *st) {
    ffgpu_ctx *ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    const int n = A->n;
    // FreeFEM's default restart (Data_Sparse_Solver::NbSpace, VirtualSolver.hpp:79)
    const int m = prm->dim_krylov > 0 ? prm->dim_krylov : 1000;
    const int itmax = prm->itmax > 0 ? prm->itmax : n;
    const double tgv = prm->tgv > 0 ? prm->tgv : 1e30;
    const size_t dsmem = sizeof(double) * (2 * (size_t)kGmSub + 2 * (size_t)(m + 1));
    FFGPU_CHECK(dsmem <= 200 * 1024, FFGPU_EINVAL, "gmres: dim_krylov %d above the supported 10000", m);
    const int64_t vs = vstride(n);
    int nslab = 1, ngrp = 1;
    int64_t slab_len = kGmSub;
    gm_dot_shape(n, nslab, ngrp, slab_len);
    const int Gv = gm_vec_grid(n), Gd = nslab * ngrp, Gc = gm_coef_grid(m);
    // workspace: V (m+1 vectors), Vp (m), the SpMV input and output, the small arrays
    // H, rot0 rot1 g y vnorm, Gram, h, red, part, then the scalars (in doubles, rounded up)
    const size_t nscal = (sizeof(GmScal) + sizeof(double) - 1) / sizeof(double);
    const size_t small = (size_t)(m + 2) * (m + 1) + 5 * (size_t)(m + 2) + (size_t)(m + 1) * (m + 1) +
                         (size_t)(m + 2) + (2 * (size_t)(m + 1) + 2) + 2 * (size_t)(m + 1) * std::max(Gv, nslab) +
                         nscal;
    double *ws = nullptr;
    const size_t nvec = (size_t)(2 * m + 3);
    FFGPU_CUDA(dalloc(ctx, (void **)&ws, sizeof(double) * (nvec * vs + small)));
    GmArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n; a.m = m; a.vs = vs;
    a.nslab = nslab; a.ngrp = ngrp; a.slab_len = slab_len;
    a.V = ws; a.Vp = ws + (size_t)(m + 1) * vs; a.vpc = a.Vp + (size_t)m * vs; a.w = a.vpc + vs;
    double *sm = a.w + vs;
    a.H = sm; sm += (size_t)(m + 2) * (m + 1);
    a.rot0 = sm; sm += m + 2;
    a.rot1 = sm; sm += m + 2;
    a.g = sm; sm += m + 2;
    a.y = sm; sm += m + 2;
    a.vnorm = sm; sm += m + 2;
    a.Gm = sm; sm += (size_t)(m + 1) * (m + 1);
    a.h = sm; sm += m + 2;
    a.red = sm; sm += 2 * (m + 1) + 2;
    a.part = sm; sm += 2 * (size_t)(m + 1) * std::max(Gv, nslab);
    a.sc = reinterpret_cast<GmScal *>(sm);
    sm += nscal;
    if ((size_t)(sm - ws) != nvec * vs + small) {
        dfree(ctx, ws);
        FFGPU_CHECK(false, FFGPU_EINVAL, "gmres: workspace layout mismatch");
    }
    a.x = x; a.b = b; a.dinv = A->diag_inv; a.wcl = A->wcl; a.use_wcl = A->ntgv > 0;
    FFGPU_CUDA(cudaMemsetAsync(a.sc, 0, sizeof(GmScal), s));
    FFGPU_CUDA(cudaFuncSetAttribute((const void *)gm_dots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
    int rc = FFGPU_OK;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (A->ntgv > 0) {
        gm_x0_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, x, b, A->wcl, tgv);   // SetInitWithBC
        rc = launch_check(ctx, "gmres x0");
    }
    if (!rc) {
        gm_init<<<Gv, kGmThreads, 0, s>>>(a, prm->eps, itmax);
        rc = launch_check(ctx, "gmres init");
    }
    // the SpMV's launch data (SELL partition) are set up by this first call, before the capture
    if (!rc) rc = spmv(A, a.vpc, a.w, trans, s);
    const bool host_loop = getenv("FFGPU_CG_GRAPH") && getenv("FFGPU_CG_GRAPH")[0] == '0';
    if (!rc && !host_loop) {
        // graph of one restart cycle: [A x -> V0, residual, while(!stop){prep, SpMV, dots, coef, update},
        // back substitution, x update]
        cudaGraph_t graph = nullptr;
        cudaGraphConditionalHandle cond;
        cudaError_t e = cudaGraphCreate(&graph, 0);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
        GmArgs ag = a;
        ag.cond = cond;
        ag.in_graph = 1;
        cudaGraphNode_t pre_last = nullptr, wnode = nullptr;
        cudaGraph_t body = nullptr;
        // prologue: captured into the parent graph
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            int r2 = spmv(A, x, a.V, trans, s);
            gm_resid<<<Gv, kGmThreads, 0, s>>>(ag);
            cudaError_t ec = cudaStreamEndCapture(s, &graph);
            if (r2 || ec != cudaSuccess) e = ec != cudaSuccess ? ec : cudaErrorUnknown;
        }
        // the while node after the prologue's last node
        if (e == cudaSuccess) {
            size_t nn = 0;
            e = cudaGraphGetNodes(graph, nullptr, &nn);
            std::vector<cudaGraphNode_t> nodes(nn);
            if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nodes.data(), &nn);
            // the prologue is a chain; its sink is the node with no dependents
            for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
                size_t nd = 0;
                e = cudaGraphNodeGetDependentNodes(nodes[i], nullptr, nullptr, &nd);
                if (e == cudaSuccess && nd == 0) pre_last = nodes[i];
            }
            alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
            memset(cp_buf, 0, sizeof(cp_buf));
            cudaGraphNodeParams *cp = reinterpret_cast<cudaGraphNodeParams *>(cp_buf);
            cp->type = cudaGraphNodeTypeConditional;
            cp->conditional.handle = cond;
            cp->conditional.type = cudaGraphCondTypeWhile;
            cp->conditional.size = 1;
            if (e == cudaSuccess) e = cudaGraphAddNode(&wnode, graph, &pre_last, nullptr, 1, cp);
            if (e == cudaSuccess) body = cp->conditional.phGraph_out[0];
        }
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            gm_prep<<<Gv, kGmThreads, 0, s>>>(ag);
            int r2 = spmv(A, a.vpc, a.w, trans, s);
            gm_dots<<<Gd, kGmThreads, dsmem, s>>>(ag);
            gm_coef<<<Gc, kGmThreads, 0, s>>>(ag);
            gm_update<<<Gv, kGmThreads, 0, s>>>(ag);
            cudaError_t ec = cudaStreamEndCapture(s, &body);
            if (r2 || ec != cudaSuccess) e = ec != cudaSuccess ? ec : cudaErrorUnknown;
        }
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, graph, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            gm_back<<<1, 32, 0, s>>>(ag);
            gm_xupd<<<Gv, kGmThreads, 0, s>>>(ag);
            e = cudaStreamEndCapture(s, &graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            set_error("gmres graph: %s", cudaGetErrorString(e));
            cudaGetLastError();
            rc = FFGPU_ECUDA;
        }
    }
    GmScal hs;
    memset(&hs, 0, sizeof(hs));
    int cycles = 0;
    int64_t steps_seen = 0;
    while (!rc) {
        if (host_loop) {
            // the same kernels launched from the host, for profilers that do not trace conditional
            // graph nodes; the stop flag is read after every Arnoldi step
            if ((rc = spmv(A, x, a.V, trans, s))) break;
            gm_resid<<<Gv, kGmThreads, 0, s>>>(a);
            for (;;) {
                if ((rc = launch_check(ctx, "gmres resid"))) break;
                FFGPU_CUDA(cudaMemcpyAsync(&hs, a.sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
                FFGPU_CUDA(cudaStreamSynchronize(s));
                if (hs.stop) break;
                gm_prep<<<Gv, kGmThreads, 0, s>>>(a);
                if ((rc = spmv(A, a.vpc, a.w, trans, s))) break;
                gm_dots<<<Gd, kGmThreads, dsmem, s>>>(a);
                gm_coef<<<Gc, kGmThreads, 0, s>>>(a);
                gm_update<<<Gv, kGmThreads, 0, s>>>(a);
                ctx->launches += 4;
            }
            if (rc) break;
            gm_back<<<1, 32, 0, s>>>(a);
            gm_xupd<<<Gv, kGmThreads, 0, s>>>(a);
            ctx->launches += 2;
        } else {
            FFGPU_CUDA(cudaGraphLaunch(exec, s));
        }
        FFGPU_CUDA(cudaMemcpyAsync(&hs, a.sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("gmres: %s", cudaGetErrorString(e));
            rc = FFGPU_ECUDA;
            break;
        }
        ++cycles;
        if (!host_loop) ctx->launches += 4 + 5 * (hs.steps - steps_seen);
        steps_seen = hs.steps;
        if (hs.conv) break;
        if (hs.iter > itmax) break;
    }
    cudaEventRecord(e1, s);
    cudaStreamSynchronize(s);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (exec) cudaGraphExecDestroy(exec);
    dfree(ctx, ws);
    cudaStreamSynchronize(s);
    if (rc) return rc;
    if (getenv("FFGPU_VERBOSE"))
        fprintf(stderr, "ffgpu: fgmres %d iterations, %d restart cycles, relative residual %.3e\n", hs.iter, cycles,
                hs.relres / hs.normb);
    if (st) {
        st->iterations = hs.iter;
        st->converged = hs.conv != 0;
        st->residual = hs.relres / hs.normb;
        st->elapsed_ms += ms;
    }
    return hs.conv ? FFGPU_OK : FFGPU_ENOCONV;
}

}  // namespace ffgpu
