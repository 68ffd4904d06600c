// ffgpu_mesh.cu -- FreeFEM's structured meshes and its P2 node numbering, built on the device.
//
// square(nx, ny) (Carre_, lgmesh.cpp:1229-1384) and cube(nx, ny, nz) (BuildCube,
// msh3.cpp:7879-8132) on the unit square/cube, in FreeFEM's vertex, element and boundary-element
// order, so that the numbering and the sparsity pattern built from them are FreeFEM's:
//   square: vertex (i, j) -> i + (nx+1) j at (i/nx, j/ny); square (i, j) -> triangles
//           (i0, i1, i2), (i0, i2, i3); boundary edges bottom, right, top, left (labels 1..4);
//   cube:   vertex (i, j, k) -> i + (nx+1) j + (nx+1)(ny+1) k at (i/nx, j/ny, k/nz) (as
//           0 + (1/nx) i); hexahedra in (i, j, k) order, 6 tetrahedra each; boundary faces in
//           element order, local face order (the face opposite vertex f), each labelled by the
//           cube face it lies on (x=0: 4, x=1: 2, y=0: 1, y=1: 3, z=0: 5, z=1: 6).
// P2 on tetrahedra (GenericMesh::BuildDFNumbering, GenericMesh.hpp:1878-1929): the element slots
// k*10 + i (4 vertices, then the edges 01 02 03 12 13 23) are visited in order and a node is
// numbered when first met.  On the device: the first slot of every vertex and edge comes from
// the ascending vertex -> element incidence (its first element holding the vertex / both
// endpoints); slots that are their own first slot are numbered by an exclusive scan.
#include "ffgpu_internal.cuh"

namespace ffgpu {

__device__ __constant__ int kHex6Tets[6][4] = {{4, 0, 6, 7}, {0, 4, 5, 7}, {1, 0, 5, 7},
                                                {0, 1, 3, 7}, {2, 0, 3, 7}, {0, 2, 6, 7}};
__device__ __constant__ int kMeshTetFace[4][3] = {{3, 2, 1}, {0, 2, 3}, {3, 1, 0}, {0, 1, 2}};
__device__ __constant__ int kCubeBitLabel[6] = {4, 2, 1, 3, 5, 6};
__device__ __constant__ int kMeshTetEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

struct CubeDims {
    int nx, ny, nz;
    __device__ __forceinline__ int64_t nv() const { return (int64_t)(nx + 1) * (ny + 1) * (nz + 1); }
    __device__ __forceinline__ int vbits(int p) const {
        const int nj = nx + 1, nk = nj * (ny + 1);
        const int i = p % nj, j = (p / nj) % (ny + 1), k = p / nk;
        return (i == 0) + 2 * (i == nx) + 4 * (j == 0) + 8 * (j == ny) + 16 * (k == 0) + 32 * (k == nz);
    }
};

__global__ void cube_vertices_kernel(CubeDims D, double *X) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= D.nv()) return;
    const int nj = D.nx + 1, nk = nj * (D.ny + 1);
    const int i = (int)(p % nj), j = (int)((p / nj) % (D.ny + 1)), k = (int)(p / nk);
    const double xd = 1.0 / D.nx, yd = 1.0 / D.ny, zd = 1.0 / D.nz;
    X[3 * p] = 0.0 + xd * i;
    X[3 * p + 1] = 0.0 + yd * j;
    X[3 * p + 2] = 0.0 + zd * k;
}

__device__ __forceinline__ void cube_tet(const CubeDims &D, int64_t t, int v[4]) {
    const int64_t h = t / 6;
    const int q = (int)(t % 6);
    const int nj = D.nx + 1, nk = nj * (D.ny + 1);
    const int hi = (int)(h % D.nx), hj = (int)((h / D.nx) % D.ny), hk = (int)(h / ((int64_t)D.nx * D.ny));
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int c = kHex6Tets[q][m];
        const int a = c & 1, b = (c >> 1) & 1, cc = c >> 2;
        v[m] = (hi + a) + nj * (hj + b) + nk * (hk + cc);
    }
}

__global__ void cube_tets_kernel(CubeDims D, int64_t nt, int32_t *E) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int v[4];
    cube_tet(D, t, v);
#pragma unroll
    for (int m = 0; m < 4; ++m) E[4 * t + m] = v[m];
}

// bit b of the cube face a tetrahedron face lies on, or -1
__device__ __forceinline__ int cube_face_bit(const CubeDims &D, const int v[4], int f) {
    const int common = D.vbits(v[kMeshTetFace[f][0]]) & D.vbits(v[kMeshTetFace[f][1]]) & D.vbits(v[kMeshTetFace[f][2]]);
    if (common == 0 || (common & (common - 1))) return -1;
    return __ffs(common) - 1;
}

__global__ void cube_bcount_kernel(CubeDims D, int64_t nt, int32_t *flag) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nt * 4) return;
    int v[4];
    cube_tet(D, s / 4, v);
    flag[s] = cube_face_bit(D, v, (int)(s % 4)) >= 0;
}

__global__ void cube_bfill_kernel(CubeDims D, int64_t nt, const int32_t *pos, int32_t *BE, int32_t *BL) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nt * 4) return;
    int v[4];
    cube_tet(D, s / 4, v);
    const int f = (int)(s % 4);
    const int b = cube_face_bit(D, v, f);
    if (b < 0) return;
    const int64_t e = pos[s];
#pragma unroll
    for (int j = 0; j < 3; ++j) BE[3 * e + j] = v[kMeshTetFace[f][j]];
    BL[e] = kCubeBitLabel[b];
}

__global__ void square_kernel(int nx, int ny, double *X, int32_t *E, int32_t *BE, int32_t *BL) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int nx1 = nx + 1;
    const int64_t nv = (int64_t)nx1 * (ny + 1), ns = (int64_t)nx * ny, nbe = 2 * (int64_t)(nx + ny);
    if (t < nv) {
        const int i = (int)(t % nx1), j = (int)(t / nx1);
        X[2 * t] = (double)i / nx;
        X[2 * t + 1] = (double)j / ny;
    }
    if (t < ns) {
        const int ii = (int)(t % nx), jj = (int)(t / nx);
        const int i0 = ii + jj * nx1, i1 = i0 + 1, i2 = i1 + nx1, i3 = i2 - 1;
        int32_t *a = E + 6 * t;
        a[0] = i0; a[1] = i1; a[2] = i2;
        a[3] = i0; a[4] = i2; a[5] = i3;
    }
    if (t < nbe) {
        int p, q, lab;
        if (t < nx) { p = (int)t; q = p + 1; lab = 1; }
        else if (t < nx + ny) { const int jb = (int)(t - nx); p = nx + jb * nx1; q = p + nx1; lab = 2; }
        else if (t < 2 * nx + ny) { const int ib = (int)(t - nx - ny); p = ib + ny * nx1; q = p + 1; lab = 3; }
        else { const int jb = (int)(t - 2 * nx - ny); p = jb * nx1; q = p + nx1; lab = 4; }
        BE[2 * t] = p; BE[2 * t + 1] = q;
        BL[t] = lab;
    }
}

// ---------------------------------------------------------------- P2 numbering (tetrahedra)
__global__ void vcount_kernel(int64_t n, const int32_t *E, int32_t *cnt) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s < n) atomicAdd(&cnt[E[s]], 1);
}

__global__ void vfill_kernel(int64_t n, const int32_t *E, const int32_t *ptr, int32_t *cur, int32_t *list) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int v = E[s];
    list[ptr[v] + atomicAdd(&cur[v], 1)] = (int32_t)(s / 4);
}

__global__ void vsort_kernel(int nv, const int32_t *ptr, int32_t *list) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int p0 = ptr[v], p1 = ptr[v + 1];
    for (int i = p0 + 1; i < p1; ++i) {
        const int x = list[i];
        int j = i - 1;
        while (j >= p0 && list[j] > x) { list[j + 1] = list[j]; --j; }
        list[j + 1] = x;
    }
}

// first slot of the node in slot s, and whether s is it
__global__ void p2_first_kernel(int64_t nt, const int32_t *E, const int32_t *ptr, const int32_t *list,
                                int32_t *first, int32_t *primary, int *status) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nt * 10) return;
    const int64_t k = s / 10;
    const int i = (int)(s % 10);
    const int32_t *v = E + 4 * k;
    int64_t fs = -1;
    if (i < 4) {
        const int a = v[i];
        const int k0 = list[ptr[a]];
        const int32_t *w = E + 4 * (int64_t)k0;
        for (int m = 0; m < 4; ++m)
            if (w[m] == a) { fs = (int64_t)k0 * 10 + m; break; }
    } else {
        const int a = v[kMeshTetEdge[i - 4][0]], b = v[kMeshTetEdge[i - 4][1]];
        for (int p = ptr[a]; p < ptr[a + 1] && fs < 0; ++p) {
            const int k1 = list[p];
            const int32_t *w = E + 4 * (int64_t)k1;
            for (int e = 0; e < 6; ++e) {
                const int x = w[kMeshTetEdge[e][0]], y = w[kMeshTetEdge[e][1]];
                if ((x == a && y == b) || (x == b && y == a)) { fs = (int64_t)k1 * 10 + 4 + e; break; }
            }
        }
    }
    if (fs < 0 || fs > s) { dev_fail(status, kDevBadIndex); fs = s; }
    first[s] = (int32_t)fs;
    primary[s] = fs == s;
}

__global__ void p2_assign_kernel(int64_t n, const int32_t *first, const int32_t *rank, int32_t *nodes) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s < n) nodes[s] = rank[first[s]];
}

static int grid_n(int64_t n, int b) { return (int)((n + b - 1) / b); }

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_mesh_sizes(int dim, int nx, int ny, int nz, int *nv, int *nt, int *nbe) {
    FFGPU_CHECK(nv && nt && nbe && nx >= 1 && ny >= 1 && (dim == 2 || (dim == 3 && nz >= 1)), FFGPU_EINVAL,
                "ffgpu_mesh_sizes: bad argument");
    int64_t v, t, b;
    if (dim == 2) {
        v = (int64_t)(nx + 1) * (ny + 1); t = 2 * (int64_t)nx * ny; b = 2 * (int64_t)(nx + ny);
    } else {
        v = (int64_t)(nx + 1) * (ny + 1) * (nz + 1); t = 6 * (int64_t)nx * ny * nz;
        b = 4 * ((int64_t)nx * ny + (int64_t)ny * nz + (int64_t)nx * nz);
    }
    FFGPU_CHECK(t * (dim + 1) < INT32_MAX && v < INT32_MAX, FFGPU_EINVAL, "mesh too large for 32-bit indices");
    *nv = (int)v; *nt = (int)t; *nbe = (int)b;
    return FFGPU_OK;
}

int ffgpu_mesh_build(ffgpu_ctx *ctx, int dim, int nx, int ny, int nz, double *coords, int32_t *elems,
                     int32_t *belems, int32_t *blabel) {
    FFGPU_CHECK(ctx && coords && elems && belems && blabel, FFGPU_EINVAL, "ffgpu_mesh_build: NULL argument");
    int nv, nt, nbe;
    FFGPU_TRY(ffgpu_mesh_sizes(dim, nx, ny, nz, &nv, &nt, &nbe));
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevOut<double> X(coords, (size_t)nv * dim, ctx, false);
    DevOut<int32_t> E(elems, (size_t)nt * (dim + 1), ctx, false);
    DevOut<int32_t> BE(belems, (size_t)nbe * dim, ctx, false);
    DevOut<int32_t> BL(blabel, (size_t)nbe, ctx, false);
    FFGPU_TRY(X.err); FFGPU_TRY(E.err); FFGPU_TRY(BE.err); FFGPU_TRY(BL.err);
    if (dim == 2) {
        const int64_t m = std::max<int64_t>(nv, std::max<int64_t>((int64_t)nx * ny, nbe));
        square_kernel<<<grid_n(m, 256), 256, 0, s>>>(nx, ny, X.d, E.d, BE.d, BL.d);
        FFGPU_TRY(launch_check(ctx, "square_kernel"));
    } else {
        const CubeDims D{nx, ny, nz};
        cube_vertices_kernel<<<grid_n(nv, 256), 256, 0, s>>>(D, X.d);
        FFGPU_TRY(launch_check(ctx, "cube_vertices"));
        cube_tets_kernel<<<grid_n(nt, 256), 256, 0, s>>>(D, nt, E.d);
        FFGPU_TRY(launch_check(ctx, "cube_tets"));
        int32_t *flag = nullptr, *pos = nullptr;
        const int64_t ns = (int64_t)nt * 4;
        if (dalloc(ctx, (void **)&flag, sizeof(int32_t) * (ns + 1)) ||
            dalloc(ctx, (void **)&pos, sizeof(int32_t) * (ns + 1))) {
            dfree(ctx, flag);
            set_error("ffgpu_mesh_build: device allocation failed");
            return FFGPU_ENOMEM;
        }
        cube_bcount_kernel<<<grid_n(ns, 256), 256, 0, s>>>(D, nt, flag);
        int rc = launch_check(ctx, "cube_bcount");
        if (!rc) rc = device_scan_i32(ctx, flag, pos, (int)ns);
        if (!rc) {
            int total = 0;
            cudaMemcpyAsync(&total, pos + ns, sizeof(int), cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            if (total != nbe) { set_error("cube: %d boundary faces found, %d expected", total, nbe); rc = FFGPU_EMESH; }
        }
        if (!rc) {
            cube_bfill_kernel<<<grid_n(ns, 256), 256, 0, s>>>(D, nt, pos, BE.d, BL.d);
            rc = launch_check(ctx, "cube_bfill");
        }
        dfree(ctx, flag);
        dfree(ctx, pos);
        FFGPU_TRY(rc);
    }
    FFGPU_TRY(X.finish()); FFGPU_TRY(E.finish()); FFGPU_TRY(BE.finish()); FFGPU_TRY(BL.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

int ffgpu_number_p2(ffgpu_ctx *ctx, int nv, int nt, const int32_t *elems, int32_t *nodes, int *nnodes) {
    FFGPU_CHECK(ctx && elems && nodes && nnodes && nv > 0 && nt > 0, FFGPU_EINVAL, "ffgpu_number_p2: bad argument");
    FFGPU_CHECK((int64_t)nt * 10 < INT32_MAX, FFGPU_EINVAL, "ffgpu_number_p2: mesh too large");
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevIn<int32_t> E(elems, (size_t)nt * 4, ctx);
    DevOut<int32_t> N(nodes, (size_t)nt * 10, ctx, false);
    FFGPU_TRY(E.err); FFGPU_TRY(N.err);
    const int64_t n4 = (int64_t)nt * 4, n10 = (int64_t)nt * 10;
    int32_t *cnt = nullptr, *ptr = nullptr, *list = nullptr, *first = nullptr, *prim = nullptr, *rank = nullptr;
    int rc = FFGPU_OK;
    if (dalloc(ctx, (void **)&cnt, sizeof(int32_t) * (nv + 1)) ||
        dalloc(ctx, (void **)&ptr, sizeof(int32_t) * (nv + 1)) ||
        dalloc(ctx, (void **)&list, sizeof(int32_t) * n4) ||
        dalloc(ctx, (void **)&first, sizeof(int32_t) * n10) ||
        dalloc(ctx, (void **)&prim, sizeof(int32_t) * (n10 + 1)) ||
        dalloc(ctx, (void **)&rank, sizeof(int32_t) * (n10 + 1))) {
        set_error("ffgpu_number_p2: device allocation failed");
        rc = FFGPU_ENOMEM;
    }
    // element vertex indices are checked first: every incidence index below depends on them
    if (!rc) {
        check_elems_kernel<<<grid_n(n4, 256), 256, 0, s>>>(E.d, n4, nv, ctx->d_status);
        rc = launch_check(ctx, "check_elems");
        if (!rc) rc = check_device_status(ctx, "ffgpu_number_p2");
    }
    if (!rc) {
        cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nv + 1), s);
        vcount_kernel<<<grid_n(n4, 256), 256, 0, s>>>(n4, E.d, cnt);
        rc = launch_check(ctx, "vcount");
    }
    if (!rc) rc = device_scan_i32(ctx, cnt, ptr, nv);
    if (!rc) {
        cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nv + 1), s);
        vfill_kernel<<<grid_n(n4, 256), 256, 0, s>>>(n4, E.d, ptr, cnt, list);
        rc = launch_check(ctx, "vfill");
    }
    if (!rc) {
        vsort_kernel<<<grid_n(nv, 256), 256, 0, s>>>(nv, ptr, list);
        rc = launch_check(ctx, "vsort");
    }
    if (!rc) {
        p2_first_kernel<<<grid_n(n10, 256), 256, 0, s>>>(nt, E.d, ptr, list, first, prim, ctx->d_status);
        rc = launch_check(ctx, "p2_first");
        if (!rc) rc = check_device_status(ctx, "ffgpu_number_p2 (inconsistent mesh)");
    }
    if (!rc) rc = device_scan_i32(ctx, prim, rank, (int)n10);
    if (!rc) {
        p2_assign_kernel<<<grid_n(n10, 256), 256, 0, s>>>(n10, first, rank, N.d);
        rc = launch_check(ctx, "p2_assign");
    }
    int total = 0;
    if (!rc && cudaMemcpyAsync(&total, rank + n10, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = FFGPU_ECUDA;
    if (!rc) rc = N.finish();
    dfree(ctx, cnt); dfree(ctx, ptr); dfree(ctx, list);
    dfree(ctx, first); dfree(ctx, prim); dfree(ctx, rank);
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) { set_error("ffgpu_number_p2 failed"); rc = FFGPU_ECUDA; }
    if (!rc) *nnodes = total;
    return rc;
}

}  // extern "C"
