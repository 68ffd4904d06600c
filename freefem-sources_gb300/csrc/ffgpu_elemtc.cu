// ffgpu_elemtc.cu -- P2 element matrices on the tensor cores (tcgen05), exact to FP64 rounding.
//
// FreeFEM forms a P2 element matrix by quadrature (Element_Op, problem.cpp:6063-6132 in 2D,
// :6337-6436 in 3D): sum over the rule's points of w_q op(phi_I) op(phi_J), i.e. B' W B with
// B the basis gradients at the points.  For P2 the gradients are linear in the barycentric
// coordinates, grad phi_I = sum_a lambda_a C_I[a], C_I[a] = sum_b c_{I,a,b} g_b with integer
// c (3, -1, 4; the g_b are the gradients of the barycentric coordinates), and the degree-2
// rules integrate the products exactly, so
//   int_K d_alpha(phi_I) d_beta(phi_J) = m sum_{b,b'} M_{IJ,bb'} g_{b,alpha} g_{b',beta},
//   M_{IJ,bb'} = sum_a c_{I,a,b} c_{J,a,b'} + s_{I,b} s_{J,b'},  s_{I,b} = sum_a c_{I,a,b},
// m = |K| / ((d+1)(d+2)): the element matrices of a whole mesh are ONE product of a constant
// integer matrix M ((I,J) pairs x 16 (b,b')) with the elements' features f_{bb'} = g_b g_b'
// (per (alpha, beta) for [P2]^3 elasticity, the dot over alpha for the scalar P2 stiffness).
//
// GB300 runs FP64 at ~2 FMAs per clock per SM; the FP64 path (ffgpu_assembly.cu, P2Pair) is
// bound there.  Here the product runs on the tensor cores exactly: each feature is rounded to a
// 53-bit fixed-point integer X relative to a power-of-two scale of its element, X is cut into
// five 11-bit digits (exact in fp16), and one tcgen05.mma per digit multiplies the digit tile
// by M (|M| <= 32, sum |M| <= 96 per row: every partial sum is an integer below 2^18, exact in
// the FP32 accumulator).  The epilogue joins the five accumulators into the exact int64
// Y = sum M X, and the FP64 pipe only converts and scales: K = m coef 2^(E-53) Y.  The element
// matrices are therefore the exact contraction of the rounded features (relative error below
// 2^-53 of the element's largest feature), and exactly symmetric.
//
// Tile: the A operand is M (128 rows: the (I <= J) pairs, 55 on tetrahedra, 21 on triangles,
// the rest zero; K = 16), the B operand the digit tiles (N = 48 feature rows per digit: 3
// elasticity elements x 16 rows (9 used) or 48 scalar elements), the accumulators D[pair][row]
// five 48-column blocks of TMEM (256 columns allocated, two CTAs per SM).  Persistent CTAs of
// 128 threads take tiles from a counter; thread 0 issues the five MMAs and commits them to an
// mbarrier; every wait is bounded in time and a timeout is reported through the status word.
#include <cuda_fp16.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcN = 48;                           // MMA N: feature rows per digit per tile
constexpr int kTcDigits = 5;
constexpr int kTcCols = 256;                       // TMEM columns (5 x 48 = 240 used)
constexpr int kTcSliceBytes = kTcN * 16 * 2;       // 48 rows x 16 fp16
constexpr unsigned long long kTcWaitNs = 1000000000ull;   // 1 s
// instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// fp16 (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kTcIdesc = (1u << 4) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a K-major operand tile with 16 fp16 per row in the
// no-swizzle canonical layout: 8 x 8 core matrices of 128 contiguous bytes (a row of a core
// matrix = 8 consecutive k), the two K halves of an 8-row group adjacent (leading byte offset
// 128), 8-row groups 256 bytes apart (stride byte offset)
__device__ __forceinline__ int tile_off(int r, int k) {
    return (r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// shared memory descriptor: start >> 4 (bits 0-13), leading byte offset >> 4 (16-29), stride
// byte offset >> 4 (32-45), descriptor version 1 (46-47), no swizzle (61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// 16 consecutive TMEM columns of this thread's lane, with the wait for the load in the same
// statement (the registers are defined only after tcgen05.wait::ld)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&r)[16]) {
    uint32_t u[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) r[i] = __uint_as_float(u[i]);
}

// the integer c_{I,a,b} of grad phi_I = sum_a lambda_a sum_b c_{I,a,b} g_b (local P2 order:
// vertices, then edges: tetrahedra 01 02 03 12 13 23, triangles edge i opposite vertex i)
template <int DIM>
__device__ int p2c(int I, int a, int b) {
    if (I <= DIM) return b == I ? (a == I ? 3 : -1) : 0;
    const int e = I - DIM - 1;
    int p, q;
    if (DIM == 3) {
        p = e < 3 ? 0 : (e < 5 ? 1 : 2);
        q = e < 3 ? e + 1 : (e == 3 ? 2 : 3);
    } else {
        p = (e + 1) % 3;
        q = (e + 2) % 3;
    }
    return ((a == p && b == q) || (a == q && b == p)) ? 4 : 0;
}

template <int DIM>
__device__ int p2m(int I, int J, int b, int bp) {
    int t = 0, sI = 0, sJ = 0;
    for (int a = 0; a <= DIM; ++a) {
        t += p2c<DIM>(I, a, b) * p2c<DIM>(J, a, bp);
        sI += p2c<DIM>(I, a, b);
        sJ += p2c<DIM>(J, a, bp);
    }
    return t + sI * sJ;
}

// pair t of the upper triangle (I <= J), row by row
__device__ __forceinline__ void pair_of(int t, int nn, int &I, int &J) {
    int i = 0;
    while (t >= nn - i) { t -= nn - i; ++i; }
    I = i;
    J = i + t;
}

// round(f * 2^(53 - E)) for |f| < 2^E, from the bits (integer pipe only)
__device__ __forceinline__ long long fixed53(double f, int E) {
    const long long bits = __double_as_longlong(f);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0;   // zero; subnormals are below 2^-1022 of any element's scale
    const long long mant = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
    const int sh = 1022 + E - ex;
    long long X;
    if (sh <= 0) X = mant;
    else if (sh > 62) X = 0;
    else X = (mant + (1ll << (sh - 1))) >> sh;
    return bits < 0 ? -X : X;
}

// the element's scale: every |g_{b,alpha}| < 2^x; returns x (from the largest magnitude's bits)
template <int DIM>
__device__ __forceinline__ int grad_scale(const double *G) {
    long long mx = 0;
#pragma unroll
    for (int i = 0; i < DIM + 1; ++i)
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const long long v = __double_as_longlong(__ldg(G + 3 * i + d)) & 0x7FFFFFFFFFFFFFFFll;
            mx = v > mx ? v : mx;
        }
    return (int)((mx >> 52) & 0x7FF) - 1022;
}

// the five digits of X into the digit tiles (row n, column k)
__device__ __forceinline__ void put_digits(unsigned char *sb, int n, int k, long long X) {
    const unsigned long long Xa = (unsigned long long)(X < 0 ? -X : X);
    const int off = tile_off(n, k);
#pragma unroll
    for (int s = 0; s < kTcDigits; ++s) {
        const unsigned int D = s == 0 ? (unsigned int)(Xa >> 44) : (unsigned int)((Xa >> (11 * (4 - s))) & 2047u);
        __half h = __ushort2half_rn((unsigned short)D);
        if (X < 0) h = __hneg(h);
        *reinterpret_cast<__half *>(sb + s * kTcSliceBytes + off) = h;
    }
}

__device__ __forceinline__ long long join_digits(const float (&r)[kTcDigits][16], int q) {
    long long y = __float2int_rn(r[0][q]);
#pragma unroll
    for (int s = 1; s < kTcDigits; ++s) y = y * 2048 + __float2int_rn(r[s][q]);
    return y;
}

}  // namespace

// FE 2: scalar P2 stiffness kappa * int grad(phi_I).grad(phi_J) (out[(e*NN + I)*NN + J]);
// FE 3: [P2]^3 elasticity blocks (out[((e*NN + I)*NN + J)*9 + 3c + c'])
template <int DIM, int FE>
__global__ void __launch_bounds__(kTcThreads) elem_tc_kernel(int nt, const double *__restrict__ geo,
                                                             const double *__restrict__ lame, double lam, double mu,
                                                             double *__restrict__ out, int *tile_counter,
                                                             int *status) {
    constexpr int NV = DIM + 1;
    constexpr int NN = DIM == 3 ? 10 : 6;
    constexpr int NP = NN * (NN + 1) / 2;
    constexpr int EPT = FE == 3 ? kTcN / 16 : kTcN;   // elements per tile
    constexpr double mfac = DIM == 3 ? 1.0 / 20.0 : 1.0 / 12.0;
    __shared__ __align__(1024) unsigned char sa[128 * 32];
    __shared__ __align__(1024) unsigned char sb[kTcDigits * kTcSliceBytes];
    __shared__ double coef[EPT][2];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tmem_sh;
    __shared__ int tile_sh, fail_sh;
    const int tid = threadIdx.x, warp = tid >> 5;

    // A operand: row t = pair (I, J), column k = b * NV + b'
    {
        int I = 0, J = 0;
        if (tid < NP) pair_of(tid, NN, I, J);
        for (int k = 0; k < 16; ++k) {
            const int b = k / NV, bp = k % NV;
            const int v = (tid < NP && k < NV * NV) ? p2m<DIM>(I, J, b, bp) : 0;
            *reinterpret_cast<__half *>(sa + tile_off(tid, k)) = __int2half_rn(v);
        }
    }
    for (int i = tid; i < kTcDigits * kTcSliceBytes / 4; i += kTcThreads) reinterpret_cast<uint32_t *>(sb)[i] = 0u;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_sh;
    uint32_t phase = 0;

    for (;;) {
        if (tid == 0) tile_sh = atomicAdd(tile_counter, 1);
        __syncthreads();
        const int e0 = tile_sh * EPT;
        if (e0 >= nt) break;
        // ---- features of the tile's elements, as digits
        if (FE == 3) {
            if (tid < EPT * 9 * NV) {
                const int el = tid / (9 * NV), rem = tid - el * 9 * NV;
                const int ab = rem / NV, b = rem - ab * NV;
                const int al = ab / 3, be = ab - al * 3;
                const int e = e0 + el;
                const int n = el * 16 + ab;
                if (e < nt) {
                    const double *ge = geo + (int64_t)e * kGeoStride;
                    const double *G = ge + 4;
                    const int E = 2 * grad_scale<DIM>(G);
                    const double gb = __ldg(G + 3 * b + al);
#pragma unroll
                    for (int bp = 0; bp < NV; ++bp) put_digits(sb, n, b * NV + bp, fixed53(gb * __ldg(G + 3 * bp + be), E));
                    if (ab == 0 && b == 0) {
                        const double m = __ldg(ge) * mfac * ldexp(1.0, E - 53);
                        coef[el][0] = m * (lame ? __ldg(lame + 2 * (int64_t)e) : lam);
                        coef[el][1] = m * (lame ? __ldg(lame + 2 * (int64_t)e + 1) : mu);
                    }
                } else {
                    for (int bp = 0; bp < NV; ++bp) put_digits(sb, n, b * NV + bp, 0);
                }
            }
        } else {
            for (int task = tid; task < EPT * NV; task += kTcThreads) {
                const int el = task / NV, b = task - el * NV;
                const int e = e0 + el;
                if (e < nt) {
                    const double *ge = geo + (int64_t)e * kGeoStride;
                    const double *G = ge + 4;
                    const int E = 2 * grad_scale<DIM>(G) + 2;   // |sum_alpha g g| < DIM max|g|^2 < 2^E
#pragma unroll
                    for (int bp = 0; bp < NV; ++bp) {
                        double f = 0.0;
#pragma unroll
                        for (int d = 0; d < DIM; ++d) f = fma(__ldg(G + 3 * b + d), __ldg(G + 3 * bp + d), f);
                        put_digits(sb, el, b * NV + bp, fixed53(f, E));
                    }
                    if (b == 0) coef[el][0] = __ldg(ge + 1) * __ldg(ge) * mfac * ldexp(1.0, E - 53);
                } else {
                    for (int bp = 0; bp < NV; ++bp) put_digits(sb, el, b * NV + bp, 0);
                }
            }
        }
        // generic-proxy writes of the operand tiles made visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t da = smem_desc(smem_u32(sa));
#pragma unroll
            for (int s = 0; s < kTcDigits; ++s) {
                const uint64_t db = smem_desc(smem_u32(sb + s * kTcSliceBytes));
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem + s * kTcN),
                    "l"(da), "l"(db), "r"(kTcIdesc), "r"(0)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar))
                         : "memory");
            const unsigned long long t0 = global_ns();
            uint32_t done = 0;
            for (;;) {
                asm volatile(
                    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}\n"
                    : "=r"(done)
                    : "r"(smem_u32(&mbar)), "r"(phase)
                    : "memory");
                if (done || global_ns() - t0 > kTcWaitNs) break;
            }
            fail_sh = !done;
        }
        phase ^= 1u;
        __syncthreads();
        if (fail_sh) {
            if (tid == 0) dev_fail(status, kDevTimeout);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // ---- epilogue: lane t of TMEM = pair t; warps without pairs skip it
        if (warp * 32 < NP) {
            const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
            int I = 0, J = 0;
            const bool act = tid < NP;
            if (act) pair_of(tid, NN, I, J);
            float r[kTcDigits][16];
            if (FE == 3) {
                for (int el = 0; el < EPT; ++el) {
#pragma unroll
                    for (int s = 0; s < kTcDigits; ++s) tmem_ld16(lane_addr + s * kTcN + el * 16, r[s]);
                    const int e = e0 + el;
                    if (!act || e >= nt) continue;
                    long long Y[9];
#pragma unroll
                    for (int q = 0; q < 9; ++q) Y[q] = join_digits(r, q);
                    const long long tr = Y[0] + Y[4] + Y[8];
                    const double l2 = coef[el][0], m2 = coef[el][1];
                    double Yd[9];
#pragma unroll
                    for (int q = 0; q < 9; ++q) Yd[q] = (double)Y[q];
                    double K[9];
#pragma unroll
                    for (int c = 0; c < 3; ++c)
#pragma unroll
                        for (int cp = 0; cp < 3; ++cp) {
                            // lambda P^{c c'} + mu (P^{c' c} + delta tr P)
                            const double q2 = c == cp ? (double)(Y[4 * c] + tr) : Yd[3 * cp + c];
                            K[3 * c + cp] = fma(l2, Yd[3 * c + cp], m2 * q2);
                        }
                    double *oij = out + (((int64_t)e * NN + I) * NN + J) * 9;
#pragma unroll
                    for (int q = 0; q < 9; ++q) oij[q] = K[q];
                    if (I != J) {
                        double *oji = out + (((int64_t)e * NN + J) * NN + I) * 9;
#pragma unroll
                        for (int c = 0; c < 3; ++c)
#pragma unroll
                            for (int cp = 0; cp < 3; ++cp) oji[3 * cp + c] = K[3 * c + cp];
                    }
                }
            } else {
                for (int ch = 0; ch < EPT / 16; ++ch) {
#pragma unroll
                    for (int s = 0; s < kTcDigits; ++s) tmem_ld16(lane_addr + s * kTcN + ch * 16, r[s]);
                    if (!act) continue;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int e = e0 + ch * 16 + j;
                        if (e >= nt) break;
                        const double v = coef[ch * 16 + j][0] * (double)join_digits(r, j);
                        out[((int64_t)e * NN + I) * NN + J] = v;
                        if (I != J) out[((int64_t)e * NN + J) * NN + I] = v;
                    }
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
    }
}

bool elem_tc_enabled() {
    const char *e = getenv("FFGPU_ELEM_TC");
    return !(e && e[0] == '0');
}

int elem_tc_prepare(ffgpu_space *S, const double *geo, double lam, double mu, const double *lame, double **out) {
    *out = nullptr;
    if (!elem_tc_enabled() || !(S->fe == FFGPU_FE_P2 || S->fe == FFGPU_FE_P2VEC3)) return FFGPU_OK;
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    const int bs2 = S->bs * S->bs;
    const size_t bytes = sizeof(double) * (size_t)S->nt * S->nn * S->nn * bs2;
    if (dalloc(ctx, (void **)out, bytes) != cudaSuccess) {
        // no room for the element matrices: the FP64 path forms them inside the row gather
        cudaGetLastError();
        *out = nullptr;
        return FFGPU_OK;
    }
    int *counter = ctx->d_iscratch + 12;
    FFGPU_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s));
    const int ept = S->fe == FFGPU_FE_P2VEC3 ? kTcN / 16 : kTcN;
    const int64_t tiles = ((int64_t)S->nt + ept - 1) / ept;
    const int grid = (int)std::min<int64_t>(2 * kNumSM, tiles);
    if (S->fe == FFGPU_FE_P2VEC3)
        elem_tc_kernel<3, 3><<<grid, kTcThreads, 0, s>>>(S->nt, geo, lame, lam, mu, *out, counter, ctx->d_status);
    else if (S->dim == 3)
        elem_tc_kernel<3, 2><<<grid, kTcThreads, 0, s>>>(S->nt, geo, nullptr, 0.0, 0.0, *out, counter, ctx->d_status);
    else
        elem_tc_kernel<2, 2><<<grid, kTcThreads, 0, s>>>(S->nt, geo, nullptr, 0.0, 0.0, *out, counter, ctx->d_status);
    const int rc = launch_check(ctx, "elem_tc_kernel");
    if (rc) { dfree(ctx, *out); *out = nullptr; }
    return rc;
}

}  // namespace ffgpu
