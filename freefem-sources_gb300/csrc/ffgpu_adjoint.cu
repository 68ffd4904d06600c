// ffgpu_adjoint.cu -- per-element sensitivities of the diffusion problem for the adjoint.
//
// For A(kappa) u = b(f) assembled from  int(kappa grad u.grad v) + int(f v) + on(.., u=g)
// with FreeFEM's tgv rows (A_ii := tgv, b_i := tgv g_i on Dirichlet DOFs; off-diagonal
// entries of those rows are kept, HashMatrix.cpp:1223-1224), and a loss L(u) with adjoint
// state lambda solving A' lambda = dL/du (transpose CG, the A'^-1 path of lgmat.cpp:3219):
//   dL/dkappa_e = - sum_{i,j in e} lambda_i  dA_ij/dkappa_e  u_j
//               = - c_stiff |K| sum_{i,j} lambda_i (grad phi_i . grad phi_j) u_j
//                 with the (i,i) term dropped when i is a tgv row (A_ii = tgv is constant);
//   dL/df_e     =   sum_{i in e, i not tgv} lambda_i int_K phi_i.
// One thread per element reads the cached geometry (barycentric gradients and measure).
#include <string.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

constexpr int kGeo = 16;

template <int DIM>
__global__ void sensitivity_kernel(int nt, const int32_t *__restrict__ nodes, const double *__restrict__ geo,
                                   double c_stiff, const double *__restrict__ u, const double *__restrict__ lam,
                                   const uint8_t *__restrict__ wcl, double *__restrict__ gk,
                                   double *__restrict__ gf) {
    constexpr int NV = DIM + 1;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nt) return;
    const double *ge = geo + (int64_t)e * kGeo;
    const double meas = ge[0];
    const double *G = ge + 4;
    int v[NV];
    double uu[NV], ll[NV];
    bool tg[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        v[i] = nodes[(int64_t)e * NV + i];
        uu[i] = u[v[i]];
        ll[i] = lam[v[i]];
        tg[i] = wcl ? wcl[v[i]] != 0 : false;
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            if (i == j && tg[i]) continue;
            double gg = 0.0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) gg += G[3 * i + d] * G[3 * j + d];
            s += ll[i] * gg * uu[j];
        }
    if (gk) gk[e] = -c_stiff * meas * s;
    if (gf) {
        double t = 0.0;
#pragma unroll
        for (int i = 0; i < NV; ++i)
            if (!tg[i]) t += ll[i];
        gf[e] = t * meas / NV;
    }
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_diffusion_sensitivity(ffgpu_matrix *A, const double *u, const double *lambda, double c_stiff,
                                double *grad_kappa, double *grad_f) {
    FFGPU_CHECK(A && A->space && u && lambda, FFGPU_EINVAL, "ffgpu_diffusion_sensitivity: bad argument");
    ffgpu_space *S = A->space;
    FFGPU_CHECK(S->fe == FFGPU_FE_P1, FFGPU_EINVAL, "sensitivities are provided for P1 diffusion");
    ffgpu_ctx *ctx = A->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    FFGPU_TRY(matrix_prepare_solver(A));   // tgv rows as the solver sees them
    DevIn<double> ud(u, S->ndof, ctx), ld(lambda, S->ndof, ctx);
    DevOut<double> gk(grad_kappa, grad_kappa ? S->nt : 0, ctx, false), gf(grad_f, grad_f ? S->nt : 0, ctx, false);
    FFGPU_TRY(ud.err); FFGPU_TRY(ld.err); FFGPU_TRY(gk.err); FFGPU_TRY(gf.err);
    const uint8_t *wcl = A->ntgv > 0 ? A->wcl : nullptr;
    int grid = (S->nt + 255) / 256;
    if (S->dim == 2)
        sensitivity_kernel<2><<<grid, 256, 0, s>>>(S->nt, S->nodes, A->geo, c_stiff, ud.d, ld.d, wcl, gk.d, gf.d);
    else
        sensitivity_kernel<3><<<grid, 256, 0, s>>>(S->nt, S->nodes, A->geo, c_stiff, ud.d, ld.d, wcl, gk.d, gf.d);
    FFGPU_TRY(launch_check(ctx, "sensitivity"));
    FFGPU_TRY(gk.finish());
    FFGPU_TRY(gf.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

}  // extern "C"
