// ffgpu_cluster.cu -- the whole Jacobi-PCG of a small system in ONE thread-block cluster.
//
// A system of up to 8 x 9216 rows (square(256) P1: 66 049) is latency-bound on the regular
// path: each CG iteration is three kernels whose cross-block reductions and launch boundaries
// cost ~20 us while the matrix (5.5 MB) sits in L2.  Here one cluster of up to 8 CTAs (the
// portable cluster size; one CTA per SM, 1024 threads each) keeps the vectors in shared memory
// and runs every iteration without leaving the kernel:
//   * CTA r owns the rows [r R, (r+1) R) (R = a multiple of 1024: whole SELL-32 windows);
//     h, q and the Jacobi diagonal of its rows live in its shared memory, x and g in
//     registers (thread t: rows r R + t + 1024 k);
//   * the SpMV (K_a) walks the CTA's SELL-32 chunks (values and 16/32-bit columns stream from
//     L2) and gathers h[col] from the owning CTA's shared memory -- its own, or a neighbour's
//     through distributed shared memory;
//   * each dot product: a block sum per CTA, written to the CTA's shared memory, one
//     barrier.cluster, then every CTA sums the CTAs' partials in rank order -- so all CTAs hold
//     the same bits and take the same branch;
//   * three cluster barriers per iteration (after the (H,AH), (G,CG) and (G,H) partials); the
//     one after (G,H) also publishes the new h to the other CTAs' next SpMV.
// The recurrence is FreeFEM's ConjugueGradient (CG.cpp:196-265) as in ffgpu_solve.cu: the
// rows sum in the same order as the SELL-32 K_a kernel; only the dot products' order differs.
// The iteration count is bounded by itmax; every CTA runs the same number of barriers.
//
// Measured on GB300 (square(256) P1, 532 iterations): 56 us per iteration against 20 us for the
// graph of three kernels on the whole GPU.  ncu: the FP64 pipe of the 8 SMs is 68 % busy.  One
// iteration is ~1 M FP64 operations (SpMV 460 k FMAs, vector updates and dots ~530 k), and
// GB300's FP64 rate (~2 FMA per clock per SM) makes 8 SMs need ~32 us for them: the FP64 work
// has to be spread over all 152 SMs, which a single cluster cannot do.  The path is therefore
// opt-in (FFGPU_CLUSTER_CG=1); the regular path serves every system by default.
#include <cooperative_groups.h>
#include <stdlib.h>

#include "ffgpu_internal.cuh"

namespace cg = cooperative_groups;

namespace ffgpu {

constexpr int kClThreads = 1024;
constexpr int kClMaxCtas = 8;        // portable cluster size
constexpr int kClMaxPass = 9;        // rows per thread (R <= 9216: h, q, dinv = 216 KB of shared memory)

struct ClusterArgs {
    int n, R, ncta;
    SellArgs S;
    const double *val;
    double *x;
    const double *g, *h, *dinv;
    KrylovScalars *ks;
};

// one scalar per CTA -> the cluster's sum, identical bits in every CTA (rank order)
__device__ __forceinline__ double cluster_total(cg::cluster_group &cl, double v, double *part, int slot,
                                                double *bc, int ncta) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double wsum[32];
    v = warp_sum(v);
    if (lane == 0) wsum[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double t = wsum[lane];
        t = warp_sum(t);
        if (lane == 0) part[slot] = t;
    }
    cl.sync();   // every CTA's partial written (release / acquire across the cluster)
    if (warp == 0) {
        double t = 0;
        if (lane < ncta) t = *cl.map_shared_rank(part + slot, lane);
        // fixed tree over ranks: the same order in every CTA
        t = warp_sum(t);
        if (lane == 0) *bc = t;
    }
    __syncthreads();
    return *bc;
}

template <bool C16>
__global__ void __launch_bounds__(kClThreads, 1) cg_cluster(ClusterArgs A) {
    extern __shared__ double sm[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int R = A.R;
    const int row0 = rank * R;
    const int rows = max(0, min(R, A.n - row0));
    double *h_s = sm, *q_s = sm + R, *d_s = sm + 2 * R;
    __shared__ double part[4], bc[4];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int P = R / kClThreads;
    double xr[kClMaxPass], gr[kClMaxPass];
#pragma unroll
    for (int k = 0; k < kClMaxPass; ++k) {
        const int i = t + k * kClThreads;
        xr[k] = gr[k] = 0.0;
        if (k < P && i < rows) {
            xr[k] = A.x[row0 + i];
            gr[k] = A.g[row0 + i];
            h_s[i] = A.h[row0 + i];
            d_s[i] = A.dinv[row0 + i];
        }
    }
    KrylovScalars *ks = A.ks;
    double gcg = ks->gcg, s_gh = ks->s_gh;
    const double eps2 = ks->eps2;
    const int itmax = ks->itmax;
    int iter = 0, conv = 0;
    bool done = ks->done != 0;
    cl.sync();   // h of every CTA in place before the first remote read
    const int c0 = rank * (R / 32), c1 = min(c0 + R / 32, A.S.nchunk);
    while (!done) {
        // ---- K_a: q = A h on this CTA's chunks, (h, q)
        double hq = 0;
        for (int c = c0 + warp; c < c1; c += kClThreads / 32) {
            const int a = __ldg(A.S.perm + (int64_t)c * 32 + lane);
            const int L = __ldg(A.S.len + c);
            const int64_t sr = __ldg(A.S.off + c);
            const int ar = a < 0 ? 0 : a;
            const int64_t ce = sr * 32 + lane;
            double s = 0;
#pragma unroll 8
            for (int j = 0; j < L; ++j) {
                const int64_t e = ce + (int64_t)j * 32;
                const int col = C16 ? ar + (int)__ldg(A.S.col16 + e) : __ldg(A.S.col + e);
                const unsigned off = (unsigned)(col - row0);
                double hv;
                if (off < (unsigned)R) {
                    hv = h_s[off];
                } else {
                    const int owner = col / R;
                    hv = *cl.map_shared_rank(h_s + (col - owner * R), owner);
                }
                s = fma(__ldg(A.val + e), hv, s);
            }
            if (a >= 0) {
                q_s[a - row0] = s;
                hq = fma(h_s[a - row0], s, hq);
            }
        }
        const double s_hq = cluster_total(cl, hq, part, 0, bc + 0, A.ncta);
        const double rho = -s_gh / s_hq;
        // ---- K_b: x += rho h, g += rho q, (g, C g)
        double sg = 0;
#pragma unroll
        for (int k = 0; k < kClMaxPass; ++k) {
            const int i = t + k * kClThreads;
            if (k < P && i < rows) {
                xr[k] = fma(rho, h_s[i], xr[k]);
                gr[k] = fma(rho, q_s[i], gr[k]);
                sg = fma(gr[k], d_s[i] * gr[k], sg);
            }
        }
        const double tot = cluster_total(cl, sg, part, 1, bc + 1, A.ncta);
        const double gamma = tot / gcg;
        gcg = tot;
        ++iter;
        if (tot < eps2) { conv = 1; break; }
        if (iter >= itmax) break;
        // ---- K_c: h = gamma h - C g, (g, h)
        double gh = 0;
#pragma unroll
        for (int k = 0; k < kClMaxPass; ++k) {
            const int i = t + k * kClThreads;
            if (k < P && i < rows) {
                const double hn = gamma * h_s[i] - d_s[i] * gr[k];
                h_s[i] = hn;
                gh = fma(gr[k], hn, gh);
            }
        }
        s_gh = cluster_total(cl, gh, part, 2, bc + 2, A.ncta);
    }
#pragma unroll
    for (int k = 0; k < kClMaxPass; ++k) {
        const int i = t + k * kClThreads;
        if (k < P && i < rows) A.x[row0 + i] = xr[k];
    }
    if (rank == 0 && t == 0 && !ks->done) {
        ks->gcg = gcg;
        ks->iter = iter;
        ks->converged = conv;
        ks->done = 1;
    }
    cl.sync();   // no CTA leaves while another may still read its shared memory
}

// rows per CTA (whole windows of 1024 rows) and CTAs of the cluster for n rows; 0 when the
// system does not fit one cluster
static int cluster_rows(int n, int *ncta) {
    const int w = (n + 1024 * kClMaxCtas - 1) / (1024 * kClMaxCtas);
    if (w < 1 || w > kClMaxPass) return 0;
    const int R = 1024 * w;
    *ncta = (n + R - 1) / R;
    return R;
}

// Whether the cluster CG takes this matrix: FP64 mode, scalar rows, its SELL-32 layout, a
// system that fits one cluster and a cluster the GPU can schedule.  The choice depends on the
// matrix and the device only, never on timings.
bool cluster_cg_fits(ffgpu_matrix *A, int trans) {
    if (A->bs != 1 || A->n > kClMaxCtas * 1024 * kClMaxPass) return false;
    // opt-in (measured slower than the three-kernel graph on GB300, see the file's header)
    const char *e = getenv("FFGPU_CLUSTER_CG");
    if (!e || e[0] != '1') return false;
    int ncta = 0;
    const int R = cluster_rows(A->n, &ncta);
    if (!R) return false;
    void *fn = A->scol16 ? (void *)cg_cluster<true> : (void *)cg_cluster<false>;
    const size_t smem = sizeof(double) * 3 * (size_t)R;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ncta);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ncta;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    (void)trans;
    return nclusters >= 1;
}

// The iteration loop of cg_one for a matrix cluster_cg_fits accepted: x, g, h, dinv and the
// Krylov scalars as cg_init left them (device pointers); x receives the solution.
int cluster_cg_run(ffgpu_matrix *A, int trans, double *x, const double *g, const double *h, cudaStream_t s) {
    FFGPU_TRY(sell_values(A, trans ? kSell64T : kSell64));
    int ncta = 0;
    const int R = cluster_rows(A->n, &ncta);
    FFGPU_CHECK(R > 0, FFGPU_EINVAL, "cluster CG: %d rows do not fit one cluster", A->n);
    ClusterArgs a;
    a.n = A->n;
    a.R = R;
    a.ncta = ncta;
    a.S = sell_args(A);
    a.val = trans ? A->sval_t : A->sval;
    a.x = x;
    a.g = g;
    a.h = h;
    a.dinv = A->diag_inv;
    a.ks = A->ks;
    // the SELL columns may have been built just now (sell_values), after cluster_cg_fits looked
    // at them: the variant launched here gets its shared-memory size set here
    void *fn = A->scol16 ? (void *)cg_cluster<true> : (void *)cg_cluster<false>;
    const size_t smem = sizeof(double) * 3 * (size_t)R;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        set_error("cluster CG: %zu bytes of shared memory refused", smem);
        return kClusterRefused;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ncta);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ncta;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void *args[] = {&a};
    const cudaError_t e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) {
        // the launch was refused (nothing ran): clear the error, the caller takes the
        // regular path
        cudaGetLastError();
        set_error("cluster CG launch refused: %s", cudaGetErrorString(e));
        return kClusterRefused;
    }
    return launch_check(A->ctx, "cg_cluster");
}

}  // namespace ffgpu
