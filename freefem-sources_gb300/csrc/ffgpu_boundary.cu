// ffgpu_boundary.cu -- boundary terms of a varf: int1d(Th, labels)(...) in 2D and int2d(Th,
// labels)(...) on the boundary faces in 3D (Robin c*u.v into the matrix, Neumann g.v into the
// linear form).
//
// FreeFEM assembles them after the volume terms, boundary element by boundary element
// (AssembleBilinearForm / AssembleLinearForm: problem.cpp:1011-1019, 10722-10735), each on the
// edge/face of its adjacent element (Mesh::BoundaryElement) with the element's own basis
// (Element_Op on an edge / a face: problem.cpp:6222-6262, 6516-6560; Element_rhs:
// problem.cpp:8612-8683, 8517-8580).  On the device:
//   1. bel_elem/bel_face: the adjacent element and its local edge/face (the one opposite that
//      local vertex), found once per space from the vertex -> boundary-element incidence;
//   2. per boundary element the element vector (nn*bs) and the Robin element matrix (nn*nn) of
//      every selected term, one thread per boundary element;
//   3. node -> (boundary element, local node) lists, ascending, which the row kernels of the
//      assembly walk after the volume sum and before on(...), so that every entry receives its
//      boundary contributions in boundary-element order and every tgv variant applies after
//      them, as in FreeFEM.
#include "ffgpu_internal.cuh"

namespace ffgpu {

// local vertices of edge/face f (the one opposite local vertex f): FreeFEM's
// VerticesOfTriangularEdge (fem.hpp:95) and nvfaceTet (Mesh3dn.cpp:72)
__device__ __constant__ int kTriEdge[3][2] = {{1, 2}, {2, 0}, {0, 1}};
__device__ __constant__ int kTetFace[4][3] = {{3, 2, 1}, {0, 2, 3}, {3, 1, 0}, {0, 1, 2}};
__device__ __constant__ int kTetEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

template <int DIM>
__device__ __forceinline__ int face_vertex(int f, int j) {
    return DIM == 2 ? kTriEdge[f][j] : kTetFace[f][j];
}

// pass 0: the smallest element whose edge/face f carries the vertices of boundary element b;
// pass 1: the local edge/face of that element
template <int DIM>
__global__ void badj_elem_kernel(int nt, const int32_t *elems, const int32_t *bv_ptr, const int32_t *bv_elem,
                                 const int32_t *belems, int32_t *bel_elem, int32_t *bel_face, int pass) {
    constexpr int NV = DIM + 1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nt * NV) return;
    const int k = (int)(t / NV), f = (int)(t % NV);
    const int32_t *v = elems + (int64_t)k * NV;
    int fv[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) fv[j] = v[face_vertex<DIM>(f, j)];
    const int a = fv[0];
    for (int p = bv_ptr[a]; p < bv_ptr[a + 1]; ++p) {
        const int b = bv_elem[p];
        const int32_t *bvx = belems + (int64_t)b * DIM;
        bool all = true;
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
            bool in = false;
#pragma unroll
            for (int i = 0; i < DIM; ++i) in |= bvx[j] == fv[i];
            all &= in;
        }
        if (!all) continue;
        if (pass == 0) atomicMin(&bel_elem[b], k);
        else if (bel_elem[b] == k) bel_face[b] = f;
    }
}

// bel_elem starts as kNoElem (every byte 0x7f, above any element index)
constexpr int32_t kNoElem = 0x7f7f7f7f;

__global__ void badj_check_kernel(int nbe, const int32_t *bel_elem, int *status) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbe && bel_elem[b] == kNoElem) dev_fail(status, kDevBadIndex);
}

struct BTermArgs {
    int nbe;
    const int32_t *blabel;
    int nlab;
    const int32_t *labels;
    const int32_t *bel_elem, *bel_face, *elems;
    const double *X;
    const double *robin;   // per boundary element or NULL
    double robin_c;
    int has_robin;
    const double *g;       // per boundary element and component or NULL
    double g0, g1, g2;
    int has_g;
    double *brhs;          // nbe * nn * bs (component-major) or NULL
    double *bmat;          // nbe * nn * nn or NULL
    uint8_t *bsel;         // boundary element carries at least one term
};

// basis values at barycentric point l: P1 = l; P2 = l(2l-1) on vertices, 4 l_a l_b on edges
template <int DIM, int NN>
__device__ __forceinline__ void basis_values(const double *l, double *w) {
    constexpr int NV = DIM + 1;
    if (NN == NV) {
#pragma unroll
        for (int i = 0; i < NV; ++i) w[i] = l[i];
        return;
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) w[i] = l[i] * (2 * l[i] - 1.);
#pragma unroll
    for (int e = 0; e < NN - NV; ++e) {
        const int i0 = DIM == 2 ? kTriEdge[e][0] : kTetEdge[e][0];
        const int i1 = DIM == 2 ? kTriEdge[e][1] : kTetEdge[e][1];
        w[NV + e] = 4. * l[i0] * l[i1];
    }
}

// One thread per element: the element vector of a source given at quadrature points,
// |K| sum_q w_q f_q,c phi_i(lambda_q) (Element_rhs: problem.cpp:7839-7911, 7917-7990)
template <int DIM, int NN, int BS>
__global__ void source_qp_kernel(int nt, int nqp, const double *__restrict__ lam, const double *__restrict__ w,
                                 const double *__restrict__ fqp, const double *__restrict__ geo,
                                 double *__restrict__ fint) {
    constexpr int NV = DIM + 1;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nt) return;
    double s[NN * BS];
#pragma unroll
    for (int i = 0; i < NN * BS; ++i) s[i] = 0.0;
    for (int q = 0; q < nqp; ++q) {
        double l[NV], phi[NN];
#pragma unroll
        for (int i = 0; i < NV; ++i) l[i] = lam[q * NV + i];
        basis_values<DIM, NN>(l, phi);
#pragma unroll
        for (int c = 0; c < BS; ++c) {
            const double wf = w[q] * fqp[(e * nqp + q) * BS + c];
#pragma unroll
            for (int i = 0; i < NN; ++i) s[i * BS + c] += wf * phi[i];
        }
    }
    const double meas = geo[e * kGeoStride];
#pragma unroll
    for (int i = 0; i < NN * BS; ++i) fint[e * NN * BS + i] = meas * s[i];
}

// One thread per element: the mass matrix of a coefficient given at quadrature points,
// |K| sum_q w_q c_q phi_i(lambda_q) phi_j(lambda_q) (Element_Op: problem.cpp:6063-6160, 6337-6437)
template <int DIM, int NN>
__global__ void mass_qp_kernel(int nt, int nqp, const double *__restrict__ lam, const double *__restrict__ w,
                               const double *__restrict__ cqp, const double *__restrict__ geo,
                               double *__restrict__ mloc) {
    constexpr int NV = DIM + 1;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nt) return;
    double m[NN * (NN + 1) / 2];
#pragma unroll
    for (int i = 0; i < NN * (NN + 1) / 2; ++i) m[i] = 0.0;
    for (int q = 0; q < nqp; ++q) {
        double l[NV], phi[NN];
#pragma unroll
        for (int i = 0; i < NV; ++i) l[i] = lam[q * NV + i];
        basis_values<DIM, NN>(l, phi);
        const double wc = w[q] * cqp[e * nqp + q];
        int p = 0;
#pragma unroll
        for (int i = 0; i < NN; ++i)
#pragma unroll
            for (int j = 0; j <= i; ++j) m[p++] += wc * phi[i] * phi[j];
    }
    const double meas = geo[e * kGeoStride];
    double *out = mloc + e * NN * NN;
    int p = 0;
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j, ++p) out[i * NN + j] = out[j * NN + i] = meas * m[p];
}

// One thread per element: the stiffness matrix of a coefficient given at quadrature points,
// |K| sum_q w_q k_q grad phi_i . grad phi_j, with grad lambda_i = G_i from the element geometry
// (P2: grad of l(2l-1) = (4 l - 1) G, of 4 l_a l_b = 4 (l_a G_b + l_b G_a))
template <int DIM, int NN>
__global__ void stiff_qp_kernel(int nt, int nqp, const double *__restrict__ lam, const double *__restrict__ w,
                                const double *__restrict__ kqp, const double *__restrict__ geo,
                                double *__restrict__ kloc) {
    constexpr int NV = DIM + 1;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nt) return;
    const double *ge = geo + e * kGeoStride;
    double G[NV][DIM];
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int d = 0; d < DIM; ++d) G[i][d] = ge[4 + 3 * i + d];
    double m[NN * (NN + 1) / 2];
#pragma unroll
    for (int i = 0; i < NN * (NN + 1) / 2; ++i) m[i] = 0.0;
    for (int q = 0; q < nqp; ++q) {
        double l[NV], g[NN][DIM];
#pragma unroll
        for (int i = 0; i < NV; ++i) l[i] = lam[q * NV + i];
        if (NN == NV) {
#pragma unroll
            for (int i = 0; i < NV; ++i)
#pragma unroll
                for (int d = 0; d < DIM; ++d) g[i][d] = G[i][d];
        } else {
#pragma unroll
            for (int i = 0; i < NV; ++i)
#pragma unroll
                for (int d = 0; d < DIM; ++d) g[i][d] = (4. * l[i] - 1.) * G[i][d];
#pragma unroll
            for (int k = 0; k < NN - NV; ++k) {
                const int a = DIM == 2 ? kTriEdge[k][0] : kTetEdge[k][0];
                const int b = DIM == 2 ? kTriEdge[k][1] : kTetEdge[k][1];
#pragma unroll
                for (int d = 0; d < DIM; ++d) g[NV + k][d] = 4. * (l[a] * G[b][d] + l[b] * G[a][d]);
            }
        }
        const double wk = w[q] * kqp[e * nqp + q];
        int p = 0;
#pragma unroll
        for (int i = 0; i < NN; ++i)
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                double s = 0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) s += g[i][d] * g[j][d];
                m[p++] += wk * s;
            }
    }
    const double meas = ge[0];
    double *out = kloc + e * NN * NN;
    int p = 0;
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j, ++p) out[i * NN + j] = out[j * NN + i] = meas * m[p];
}

// One thread per boundary element: the element vector and Robin matrix of one term.
template <int DIM, int NN, int BS>
__global__ void bterm_kernel(BTermArgs A) {
    constexpr int NV = DIM + 1;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= A.nbe) return;
    if (A.nlab > 0) {
        bool hit = false;
        for (int k = 0; k < A.nlab; ++k) hit |= A.blabel[b] == A.labels[k];
        if (!hit) return;
    }
    A.bsel[b] = 1;
    const int k = A.bel_elem[b], ie = A.bel_face[b];
    const int32_t *v = A.elems + (int64_t)k * NV;
    // quadrature on the edge (Gauss-Legendre, 3 points: QuadratureFormular.cpp:319-343) or the
    // face (T_5, 7 points); points are (s) on the edge, (x, y) on the reference face
    double qx[7], qy[7], qw[7];
    int nq;
    if (DIM == 2) {
        const double g1 = (1 - sqrt(3. / 5.)) / 2;
        qx[0] = 0.5; qw[0] = 8. / 18.;
        qx[1] = g1; qw[1] = 5. / 18.;
        qx[2] = 1 - g1; qw[2] = 5. / 18.;
        nq = 3;
    } else {
        const double s15 = 3.87298334620741688517926539978;
        const double t = 1. / 3., Aw = 0.225;
        const double r = (6 - s15) / 21, s = (9 + 2 * s15) / 21, Bw = (155 - s15) / 1200;
        const double u = (6 + s15) / 21, vv = (9 - 2 * s15) / 21, Cw = (155 + s15) / 1200;
        const double px[7] = {t, r, r, s, u, u, vv}, py[7] = {t, r, s, r, u, vv, u};
        const double pw[7] = {Aw, Bw, Bw, Bw, Cw, Cw, Cw};
#pragma unroll
        for (int q = 0; q < 7; ++q) { qx[q] = px[q]; qy[q] = py[q]; qw[q] = pw[q]; }
        nq = 7;
    }
    double le;
    if (DIM == 2) {
        const double *p1 = A.X + 2 * v[kTriEdge[ie][0]], *p2 = A.X + 2 * v[kTriEdge[ie][1]];
        const double ex = p2[0] - p1[0], ey = p2[1] - p1[1];
        le = sqrt(ex * ex + ey * ey);
    } else {
        const int *f = kTetFace[ie];
        const double *a = A.X + 3 * v[f[0]], *p1 = A.X + 3 * v[f[1]], *p2 = A.X + 3 * v[f[2]];
        const double uu[3] = {p2[0] - a[0], p2[1] - a[1], p2[2] - a[2]};
        const double ww[3] = {p1[0] - a[0], p1[1] - a[1], p1[2] - a[2]};
        const double N[3] = {uu[1] * ww[2] - uu[2] * ww[1], ww[0] * uu[2] - uu[0] * ww[2],
                             uu[0] * ww[1] - uu[1] * ww[0]};
        le = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
    }
    const double c = A.has_robin ? (A.robin ? A.robin[b] : A.robin_c) : 0.0;
    double gc[BS];
#pragma unroll
    for (int cc = 0; cc < BS; ++cc)
        gc[cc] = A.g ? A.g[(int64_t)b * BS + cc] : (cc == 0 ? A.g0 : (cc == 1 ? A.g1 : A.g2));
    double r[NN * BS];
    double m[NN * NN];
#pragma unroll
    for (int i = 0; i < NN * BS; ++i) r[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NN * NN; ++i) m[i] = 0.0;
    for (int q = 0; q < nq; ++q) {
        double l[4], coef;
        if (DIM == 2) {
            coef = le * qw[q];
            const double sa = qx[q], sb = 1 - sa;
            // reference vertices of the edge: (0,0), (1,0), (0,1)
            const int ia = kTriEdge[ie][0], ib = kTriEdge[ie][1];
            const double ax = ia == 1 ? 1.0 : 0.0, ay = ia == 2 ? 1.0 : 0.0;
            const double bx = ib == 1 ? 1.0 : 0.0, by = ib == 2 ? 1.0 : 0.0;
            const double x = ax * sa + bx * sb, y = ay * sa + by * sb;
            l[1] = x; l[2] = y; l[0] = 1 - x - y; l[3] = 0;
        } else {
            coef = le * qw[q] * 0.5;
            const int *f = kTetFace[ie];
            const double x = qx[q], y = qy[q], s = 1 - x - y;
            double pt[3];
#pragma unroll
            for (int cc = 0; cc < 3; ++cc)
                pt[cc] = (f[0] == cc + 1 ? 1.0 : 0.0) * s + (f[1] == cc + 1 ? 1.0 : 0.0) * x +
                         (f[2] == cc + 1 ? 1.0 : 0.0) * y;
            l[1] = pt[0]; l[2] = pt[1]; l[3] = pt[2]; l[0] = 1. - (pt[0] + pt[1] + pt[2]);
        }
        double w[NN];
        basis_values<DIM, NN>(l, w);
        if (A.bmat) {
            const double ccc = c * coef;
#pragma unroll
            for (int i = 0; i < NN; ++i)
#pragma unroll
                for (int j = 0; j < NN; ++j) m[i * NN + j] += ccc * w[i] * w[j];
        }
        if (A.brhs && A.has_g)
#pragma unroll
            for (int cc = 0; cc < BS; ++cc)
#pragma unroll
                for (int i = 0; i < NN; ++i) r[cc * NN + i] += coef * gc[cc] * w[i];
    }
    if (A.bmat && A.has_robin)
        for (int i = 0; i < NN * NN; ++i) A.bmat[(int64_t)b * NN * NN + i] += m[i];
    if (A.brhs && A.has_g)
        for (int i = 0; i < NN * BS; ++i) A.brhs[(int64_t)b * NN * BS + i] += r[i];
}

__global__ void bnode_count_kernel(int nbe, int nn, const uint8_t *bsel, const int32_t *bel_elem,
                                   const int32_t *nodes, int32_t *cnt) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nbe * nn) return;
    const int b = (int)(t / nn), il = (int)(t % nn);
    if (!bsel[b]) return;
    atomicAdd(&cnt[nodes[(int64_t)bel_elem[b] * nn + il]], 1);
}

__global__ void bnode_fill_kernel(int nbe, int nn, const uint8_t *bsel, const int32_t *bel_elem,
                                  const int32_t *nodes, const int32_t *ptr, int32_t *cursor, int32_t *list) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nbe * nn) return;
    const int b = (int)(t / nn), il = (int)(t % nn);
    if (!bsel[b]) return;
    const int node = nodes[(int64_t)bel_elem[b] * nn + il];
    list[ptr[node] + atomicAdd(&cursor[node], 1)] = (int32_t)t;   // t = b * nn + il
}

// per node: its (boundary element, local node) codes in ascending order (short lists)
__global__ void bnode_sort_kernel(int nnodes, const int32_t *ptr, int32_t *list) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nnodes) return;
    const int p0 = ptr[a], p1 = ptr[a + 1];
    for (int i = p0 + 1; i < p1; ++i) {
        const int x = list[i];
        int j = i - 1;
        while (j >= p0 && list[j] > x) { list[j + 1] = list[j]; --j; }
        list[j + 1] = x;
    }
}

static int grid_of(int64_t n, int block) { return (int)((n + block - 1) / block); }

// adjacent element and local edge/face of every boundary element (once per space)
static int boundary_adjacency(ffgpu_space *S) {
    if (S->bel_elem) return FFGPU_OK;
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    if (dalloc(ctx, (void **)&S->bel_elem, sizeof(int32_t) * S->nbe) ||
        dalloc(ctx, (void **)&S->bel_face, sizeof(int32_t) * S->nbe)) {
        dfree(ctx, S->bel_elem); dfree(ctx, S->bel_face);
        S->bel_elem = S->bel_face = nullptr;
        set_error("boundary terms: device allocation failed");
        return FFGPU_ENOMEM;
    }
    FFGPU_CUDA(cudaMemsetAsync(S->bel_elem, 0x7f, sizeof(int32_t) * S->nbe, s));   // kNoElem
    const int64_t m = (int64_t)S->nt * (S->dim + 1);
    for (int pass = 0; pass < 2; ++pass) {
        if (S->dim == 2)
            badj_elem_kernel<2><<<grid_of(m, 256), 256, 0, s>>>(S->nt, S->elems, S->bv_ptr, S->bv_elem, S->belems,
                                                                S->bel_elem, S->bel_face, pass);
        else
            badj_elem_kernel<3><<<grid_of(m, 256), 256, 0, s>>>(S->nt, S->elems, S->bv_ptr, S->bv_elem, S->belems,
                                                                S->bel_elem, S->bel_face, pass);
        FFGPU_TRY(launch_check(ctx, "badj_elem"));
    }
    badj_check_kernel<<<grid_of(S->nbe, 256), 256, 0, s>>>(S->nbe, S->bel_elem, ctx->d_status);
    FFGPU_TRY(launch_check(ctx, "badj_check"));
    const int rc = check_device_status(ctx, "boundary terms (a boundary element has no adjacent element)");
    if (rc) {
        dfree(ctx, S->bel_elem); dfree(ctx, S->bel_face);
        S->bel_elem = S->bel_face = nullptr;
    }
    return rc;
}

template <int DIM, int NN, int BS>
static void launch_bterm(const BTermArgs &a, cudaStream_t s) {
    bterm_kernel<DIM, NN, BS><<<grid_of(a.nbe, 128), 128, 0, s>>>(a);
}

int boundary_prepare(ffgpu_space *S, const ffgpu_varf *v, bool want_rhs, bool want_mat, BoundaryTerms &bt) {
    bt = BoundaryTerms{};
    if (!v || v->nbterms <= 0) return FFGPU_OK;
    FFGPU_CHECK(v->bterms, FFGPU_EINVAL, "varf: nbterms > 0 with NULL bterms");
    FFGPU_CHECK(S->belems, FFGPU_EINVAL, "boundary terms: the space has no boundary elements (ffgpu_space_set_boundary)");
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    bool any_robin = false, any_g = false;
    for (int t = 0; t < v->nbterms; ++t) {
        const ffgpu_bterm &T = v->bterms[t];
        FFGPU_CHECK(T.nlabels >= 0 && T.nlabels <= 64 && (T.nlabels == 0 || T.labels), FFGPU_EINVAL,
                    "boundary term %d: 0..64 labels expected", t);
        any_robin |= T.robin || T.robin_const != 0.0;
        any_g |= T.g || T.g_const[0] != 0.0 || T.g_const[1] != 0.0 || T.g_const[2] != 0.0;
    }
    FFGPU_TRY(boundary_adjacency(S));
    const int nn = S->nn, bsz = S->bs, nbe = S->nbe;
    want_mat = want_mat && any_robin;
    want_rhs = want_rhs && any_g;
    if (!want_mat && !want_rhs) return FFGPU_OK;
    uint8_t *bsel = nullptr;
    int32_t *ptr = nullptr, *list = nullptr, *cnt = nullptr;
    double *brhs = nullptr, *bmat = nullptr;
    auto fail = [&](int rc) {
        dfree(ctx, bsel); dfree(ctx, ptr); dfree(ctx, list); dfree(ctx, cnt);
        dfree(ctx, brhs); dfree(ctx, bmat);
        return rc;
    };
    if (dalloc(ctx, (void **)&bsel, nbe) || dalloc(ctx, (void **)&ptr, sizeof(int32_t) * (S->nnodes + 1)) ||
        dalloc(ctx, (void **)&cnt, sizeof(int32_t) * (S->nnodes + 1)) ||
        dalloc(ctx, (void **)&list, sizeof(int32_t) * (size_t)nbe * nn) ||
        (want_rhs && dalloc(ctx, (void **)&brhs, sizeof(double) * (size_t)nbe * nn * bsz)) ||
        (want_mat && dalloc(ctx, (void **)&bmat, sizeof(double) * (size_t)nbe * nn * nn))) {
        set_error("boundary terms: device allocation failed");
        return fail(FFGPU_ENOMEM);
    }
    cudaMemsetAsync(bsel, 0, nbe, s);
    if (brhs) cudaMemsetAsync(brhs, 0, sizeof(double) * (size_t)nbe * nn * bsz, s);
    if (bmat) cudaMemsetAsync(bmat, 0, sizeof(double) * (size_t)nbe * nn * nn, s);
    for (int t = 0; t < v->nbterms; ++t) {
        const ffgpu_bterm &T = v->bterms[t];
        DevIn<int32_t> lab(T.labels, T.nlabels, ctx);
        DevIn<double> rob(T.robin, T.robin ? nbe : 0, ctx);
        DevIn<double> gg(T.g, T.g ? (size_t)nbe * bsz : 0, ctx);
        if (lab.err || rob.err || gg.err) return fail(lab.err ? lab.err : (rob.err ? rob.err : gg.err));
        BTermArgs a;
        memset(&a, 0, sizeof(a));
        a.nbe = nbe; a.blabel = S->blabel; a.nlab = T.nlabels; a.labels = lab.d;
        a.bel_elem = S->bel_elem; a.bel_face = S->bel_face; a.elems = S->elems; a.X = S->coords;
        a.robin = rob.d; a.robin_c = T.robin_const; a.has_robin = T.robin || T.robin_const != 0.0;
        a.g = gg.d; a.g0 = T.g_const[0]; a.g1 = T.g_const[1]; a.g2 = T.g_const[2];
        a.has_g = T.g || T.g_const[0] != 0.0 || T.g_const[1] != 0.0 || T.g_const[2] != 0.0;
        if (!a.has_robin && !a.has_g) continue;
        a.brhs = brhs; a.bmat = bmat; a.bsel = bsel;
        if (S->dim == 2 && S->fe == FFGPU_FE_P1) launch_bterm<2, 3, 1>(a, s);
        else if (S->dim == 3 && S->fe == FFGPU_FE_P1) launch_bterm<3, 4, 1>(a, s);
        else if (S->dim == 2 && S->fe == FFGPU_FE_P2) launch_bterm<2, 6, 1>(a, s);
        else if (S->dim == 3 && S->fe == FFGPU_FE_P2) launch_bterm<3, 10, 1>(a, s);
        else launch_bterm<3, 10, 3>(a, s);
        const int rc = launch_check(ctx, "bterm_kernel");
        if (rc) return fail(rc);
    }
    const int64_t m = (int64_t)nbe * nn;
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nnodes + 1), s);
    bnode_count_kernel<<<grid_of(m, 256), 256, 0, s>>>(nbe, nn, bsel, S->bel_elem, S->nodes, cnt);
    int rc = launch_check(ctx, "bnode_count");
    if (!rc) rc = device_scan_i32(ctx, cnt, ptr, S->nnodes);
    if (!rc) {
        cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nnodes + 1), s);
        bnode_fill_kernel<<<grid_of(m, 256), 256, 0, s>>>(nbe, nn, bsel, S->bel_elem, S->nodes, ptr, cnt, list);
        rc = launch_check(ctx, "bnode_fill");
    }
    if (!rc) {
        bnode_sort_kernel<<<grid_of(S->nnodes, 256), 256, 0, s>>>(S->nnodes, ptr, list);
        rc = launch_check(ctx, "bnode_sort");
    }
    if (rc) return fail(rc);
    dfree(ctx, cnt);
    dfree(ctx, bsel);
    bt.ptr = ptr; bt.list = list; bt.rhs = brhs; bt.mat = bmat; bt.bel_elem = S->bel_elem;
    return FFGPU_OK;
}

int source_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **fint) {
    *fint = nullptr;
    if (v && v->f_expr) return source_expr_prepare(S, v, geo, fint);
    if (!v || !v->f_qp) return FFGPU_OK;
    FFGPU_CHECK(v->nqp > 0 && v->nqp <= 64 && v->qp_lambda && v->qp_weight, FFGPU_EINVAL,
                "source at quadrature points: 1..64 points with coordinates and weights expected (nqp %d)", v->nqp);
    ffgpu_ctx *ctx = S->ctx;
    const int nv = S->dim + 1, nn = S->nn, bs = S->bs;
    DevIn<double> lam(v->qp_lambda, (size_t)v->nqp * nv, ctx), w(v->qp_weight, v->nqp, ctx);
    DevIn<double> fq(v->f_qp, (size_t)S->nt * v->nqp * bs, ctx);
    FFGPU_TRY(lam.err); FFGPU_TRY(w.err); FFGPU_TRY(fq.err);
    FFGPU_CUDA(dalloc(ctx, (void **)fint, sizeof(double) * (size_t)S->nt * nn * bs));
    void (*k)(int, int, const double *, const double *, const double *, const double *, double *) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = source_qp_kernel<2, 3, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = source_qp_kernel<3, 4, 1>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = source_qp_kernel<2, 6, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = source_qp_kernel<3, 10, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2VEC3) k = source_qp_kernel<3, 10, 3>;
    FFGPU_CHECK(k, FFGPU_EINVAL, "source at quadrature points: unsupported element");
    k<<<(int)((S->nt + 127) / 128), 128, 0, ctx->stream>>>(S->nt, v->nqp, lam.d, w.d, fq.d, geo, *fint);
    const int rc = launch_check(ctx, "source_qp");
    if (rc) { dfree(ctx, *fint); *fint = nullptr; }
    return rc;
}

int mass_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **mloc) {
    *mloc = nullptr;
    if (!v || !v->mass_qp) return FFGPU_OK;
    FFGPU_CHECK(v->form == FFGPU_FORM_DIFFUSION && S->bs == 1, FFGPU_EINVAL,
                "a mass coefficient at quadrature points needs the scalar diffusion form");
    FFGPU_CHECK(v->nqp > 0 && v->nqp <= 64 && v->qp_lambda && v->qp_weight, FFGPU_EINVAL,
                "mass at quadrature points: 1..64 points with coordinates and weights expected (nqp %d)", v->nqp);
    ffgpu_ctx *ctx = S->ctx;
    const int nv = S->dim + 1, nn = S->nn;
    DevIn<double> lam(v->qp_lambda, (size_t)v->nqp * nv, ctx), w(v->qp_weight, v->nqp, ctx);
    DevIn<double> cq(v->mass_qp, (size_t)S->nt * v->nqp, ctx);
    FFGPU_TRY(lam.err); FFGPU_TRY(w.err); FFGPU_TRY(cq.err);
    FFGPU_CUDA(dalloc(ctx, (void **)mloc, sizeof(double) * (size_t)S->nt * nn * nn));
    void (*k)(int, int, const double *, const double *, const double *, const double *, double *) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = mass_qp_kernel<2, 3>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = mass_qp_kernel<3, 4>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = mass_qp_kernel<2, 6>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = mass_qp_kernel<3, 10>;
    FFGPU_CHECK(k, FFGPU_EINVAL, "mass at quadrature points: unsupported element");
    k<<<(int)((S->nt + 127) / 128), 128, 0, ctx->stream>>>(S->nt, v->nqp, lam.d, w.d, cq.d, geo, *mloc);
    const int rc = launch_check(ctx, "mass_qp");
    if (rc) { dfree(ctx, *mloc); *mloc = nullptr; }
    return rc;
}

int stiff_prepare(ffgpu_space *S, const ffgpu_varf *v, const double *geo, double **kloc) {
    *kloc = nullptr;
    if (!v || !v->stiff_qp) return FFGPU_OK;
    FFGPU_CHECK(v->form == FFGPU_FORM_DIFFUSION && S->bs == 1, FFGPU_EINVAL,
                "a stiffness coefficient at quadrature points needs the scalar diffusion form");
    FFGPU_CHECK(v->nqp > 0 && v->nqp <= 64 && v->qp_lambda && v->qp_weight, FFGPU_EINVAL,
                "stiffness at quadrature points: 1..64 points with coordinates and weights expected (nqp %d)", v->nqp);
    ffgpu_ctx *ctx = S->ctx;
    const int nv = S->dim + 1, nn = S->nn;
    DevIn<double> lam(v->qp_lambda, (size_t)v->nqp * nv, ctx), w(v->qp_weight, v->nqp, ctx);
    DevIn<double> kq(v->stiff_qp, (size_t)S->nt * v->nqp, ctx);
    FFGPU_TRY(lam.err); FFGPU_TRY(w.err); FFGPU_TRY(kq.err);
    FFGPU_CUDA(dalloc(ctx, (void **)kloc, sizeof(double) * (size_t)S->nt * nn * nn));
    void (*k)(int, int, const double *, const double *, const double *, const double *, double *) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = stiff_qp_kernel<2, 3>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = stiff_qp_kernel<3, 4>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = stiff_qp_kernel<2, 6>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = stiff_qp_kernel<3, 10>;
    FFGPU_CHECK(k, FFGPU_EINVAL, "stiffness at quadrature points: unsupported element");
    k<<<(int)((S->nt + 127) / 128), 128, 0, ctx->stream>>>(S->nt, v->nqp, lam.d, w.d, kq.d, geo, *kloc);
    const int rc = launch_check(ctx, "stiff_qp");
    if (rc) { dfree(ctx, *kloc); *kloc = nullptr; }
    return rc;
}

void boundary_release(ffgpu_space *S, BoundaryTerms &bt) {
    ffgpu_ctx *ctx = S->ctx;
    if (bt.ptr) dfree(ctx, (void *)bt.ptr);
    if (bt.list) dfree(ctx, (void *)bt.list);
    if (bt.rhs) dfree(ctx, (void *)bt.rhs);
    if (bt.mat) dfree(ctx, (void *)bt.mat);
    bt = BoundaryTerms{};
}

}  // namespace ffgpu
