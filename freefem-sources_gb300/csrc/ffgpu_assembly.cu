// ffgpu_assembly.cu -- mesh/FE-space upload, symbolic pattern and numeric assembly.
//
// Design (GB300): FreeFEM walks elements and scatters each element matrix into a hash
// matrix (problem.cpp:1096-1103, HashMatrix.cpp:1295-1332).  Here every matrix row is
// owned by one warp, which gathers the contributions of the elements incident to its node:
//   pass 1 (count):  gather the nodes of the incident elements, sort, unique -> row degree;
//   scan:            row pointer;
//   pass 2 (fill):   same gather -> sorted column list, then add the element-matrix rows of
//                    the incident elements in ascending element order (the reference's
//                    summation order), apply tgv, write the row once, coalesced.
// No atomics and no colouring are needed on the value path: each value is written once and
// no read-modify-write of the matrix happens.  The element geometry (barycentric gradients
// and measure) is computed once per element and cached (16 doubles per element).
// For [P2]^3 the pattern is stored as 3x3 blocks (DOF = 3*node + c, FESpacen.hpp:582),
// which is the same (i,j) set as FreeFEM's MatriceMorse and 2/3 of the index traffic.
#include <string.h>

#include "ffgpu_internal.cuh"

namespace ffgpu {

// ------------------------------------------------------------------ small device utils
template <typename T>
__device__ void warp_bitonic_sort(T *s, int P) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                int ixj = i ^ j;
                if (ixj > i) {
                    bool up = (i & k) == 0;
                    T a = s[i], b = s[ixj];
                    if ((a > b) == up) { s[i] = b; s[ixj] = a; }
                }
            }
            __syncwarp();
        }
}

__device__ __forceinline__ int pow2_ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// binary search of v in the sorted list s[0..n)
__device__ __forceinline__ int find_sorted(const int *s, int n, int v) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int w = s[mid];
        if (w == v) return mid;
        if (w < v) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// ------------------------------------------------------------------ space construction
__global__ void build_nodes_kernel(const int32_t *dof, int nt, int ndofK, int nn, int bs,
                                   int ndof, int32_t *nodes, int *status) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nt * nn) return;
    int k = (int)(t / nn), i = (int)(t % nn);
    const int32_t *d = dof + (int64_t)k * ndofK;
    int v0 = d[i];
    if (v0 < 0 || v0 >= ndof) { dev_fail(status, kDevBadIndex); nodes[t] = 0; return; }
    if (bs == 1) { nodes[t] = v0; return; }
    int node = v0 / bs;
    bool ok = (v0 % bs) == 0;
    for (int c = 1; c < bs; ++c) ok = ok && d[c * nn + i] == bs * node + c;
    if (!ok) dev_fail(status, kDevBadDofLayout);
    nodes[t] = node;
}

__global__ void check_elems_kernel(const int32_t *elems, int64_t m, int nv, int *status) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < m && (elems[t] < 0 || elems[t] >= nv)) dev_fail(status, kDevBadIndex);
}

__global__ void inc_count_kernel(const int32_t *nodes, int64_t m, int32_t *cnt) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < m) atomicAdd(&cnt[nodes[t]], 1);
}

__global__ void inc_fill_kernel(const int32_t *nodes, int64_t m, int nn, const int32_t *ptr,
                                int32_t *cursor, int32_t *inc_elem, uint8_t *inc_loc) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= m) return;
    int a = nodes[t];
    int pos = ptr[a] + atomicAdd(&cursor[a], 1);
    inc_elem[pos] = (int32_t)(t / nn);
    inc_loc[pos] = (uint8_t)(t % nn);
}

// sort each node's incidence list by element number (the reference's element order)
__global__ void inc_sort_kernel(const int32_t *ptr, int nnodes, int max_inc, int32_t *inc_elem,
                                uint8_t *inc_loc) {
    extern __shared__ long long sh_inc[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int P = pow2_ceil(max_inc);
    long long *s = sh_inc + (int64_t)w * P;
    for (int a = blockIdx.x * (blockDim.x >> 5) + w; a < nnodes; a += gridDim.x * (blockDim.x >> 5)) {
        int b = ptr[a], e = ptr[a + 1], n = e - b;
        for (int i = lane; i < P; i += 32)
            s[i] = i < n ? (((long long)inc_elem[b + i]) << 8) | inc_loc[b + i] : 0x7fffffffffffffffLL;
        __syncwarp();
        warp_bitonic_sort(s, P);
        for (int i = lane; i < n; i += 32) {
            inc_elem[b + i] = (int32_t)(s[i] >> 8);
            inc_loc[b + i] = (uint8_t)(s[i] & 0xff);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ geometry
// meas and barycentric gradients: Triangle::H (fem.hpp:321-324), Tet::Gradlambda
// (Mesh3dn.hpp:126-136), tet volume det(AB,AC,AD)/6 (Mesh3dn.hpp:70)
__global__ void geometry_kernel(const double *X, const int32_t *elems, int nt, int dim,
                                const double *kappa, double c_stiff, double *geo) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
    double *g = geo + (int64_t)k * kGeoStride;
    double G[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double meas;
    if (dim == 2) {
        const int32_t *v = elems + 3 * (int64_t)k;
        double P[3][2];
        for (int i = 0; i < 3; ++i) { P[i][0] = X[2 * (int64_t)v[i]]; P[i][1] = X[2 * (int64_t)v[i] + 1]; }
        double area = ((P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[1][1] - P[0][1]) * (P[2][0] - P[0][0])) * 0.5;
        for (int i = 0; i < 3; ++i) {
            int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            double ex = P[i2][0] - P[i1][0], ey = P[i2][1] - P[i1][1];
            G[i][0] = -ey / (2 * area);
            G[i][1] = ex / (2 * area);
        }
        meas = area;
    } else {
        const int32_t *v = elems + 4 * (int64_t)k;
        double A[3], V[3][3];
        for (int d = 0; d < 3; ++d) A[d] = X[3 * (int64_t)v[0] + d];
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) V[i][d] = X[3 * (int64_t)v[i + 1] + d] - A[d];
        double c23[3] = {V[1][1] * V[2][2] - V[1][2] * V[2][1], V[1][2] * V[2][0] - V[1][0] * V[2][2],
                         V[1][0] * V[2][1] - V[1][1] * V[2][0]};
        double c31[3] = {V[2][1] * V[0][2] - V[2][2] * V[0][1], V[2][2] * V[0][0] - V[2][0] * V[0][2],
                         V[2][0] * V[0][1] - V[2][1] * V[0][0]};
        double c12[3] = {V[0][1] * V[1][2] - V[0][2] * V[1][1], V[0][2] * V[1][0] - V[0][0] * V[1][2],
                         V[0][0] * V[1][1] - V[0][1] * V[1][0]};
        double vol = (V[0][0] * c23[0] + V[0][1] * c23[1] + V[0][2] * c23[2]) / 6.;
        double det1 = 1. / (6. * vol);
        for (int d = 0; d < 3; ++d) {
            G[1][d] = c23[d] * det1;
            G[2][d] = c31[d] * det1;
            G[3][d] = c12[d] * det1;
            G[0][d] = -G[1][d] - G[2][d] - G[3][d];
        }
        meas = vol;
    }
    g[0] = meas;
    g[1] = (kappa ? kappa[k] : 1.0) * c_stiff;
    g[2] = 0; g[3] = 0;
    for (int i = 0; i < 4; ++i)
        for (int d = 0; d < 3; ++d) g[4 + 3 * i + d] = G[i][d];
}

// ------------------------------------------------------------------ element entries
// P2 gradients are linear: grad(phi_i) = sum_a lambda_a C_i[a], with
//   vertex i: C_i[i] = 3 g_i, C_i[a != i] = -g_i            (grad = (4 lambda_i - 1) g_i)
//   edge (p,q): C_i[p] = 4 g_q, C_i[q] = 4 g_p, else 0      (grad = 4(lambda_p g_q + lambda_q g_p))
// (P012_3d.cpp:199-277; 2D: FESpace.cpp:1219-1300 with edge i opposite vertex i), and
//   int_K lambda_a lambda_b = |K| (1 + delta_ab) / ((d+1)(d+2)),
// so int_K d_alpha(phi_i) d_beta(phi_j) = m (sum_a C_i[a].al C_j[a].be + S_i.al S_j.be),
// m = |K|/((d+1)(d+2)), S_i = sum_a C_i[a].  This integrates the degree-2 integrand
// exactly, as FreeFEM's default rules (T_5, Tet_5) do.
struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 v3(const double *p) { return V3{__ldg(p), __ldg(p + 1), __ldg(p + 2)}; }
__device__ __forceinline__ V3 operator*(double a, V3 v) { return V3{a * v.x, a * v.y, a * v.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double comp(V3 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }

// local edge e -> vertices (p,q): tets {01,02,03,12,13,23}, triangles edge i opposite vertex i
template <int DIM>
__device__ __forceinline__ void edge_vertices(int e, int &p, int &q) {
    if (DIM == 3) {
        p = e < 3 ? 0 : (e < 5 ? 1 : 2);
        q = e < 3 ? e + 1 : (e == 3 ? 2 : 3);
    } else {
        p = (e + 1) % 3;
        q = (e + 2) % 3;
    }
}

// One P2 basis function J in the two-gradient form used below, with no divergent branches:
//   C_J[a] = c1(a) g_p1 + c2(a) g_p2,   S_J = sum_a C_J[a] = d1 g_p1 + d2 g_p2
//   vertex j:   p1 = p2 = j, c1(a) = (a == j ? 3 : -1), c2 = 0,  d1 = 3 - dim, d2 = 0
//   edge (r,s): p1 = s, p2 = r, c1(a) = 4 [a == r], c2(a) = 4 [a == s], d1 = d2 = 4
// (grad(phi_j) = (4 lambda_j - 1) g_j and grad(4 lambda_r lambda_s) = 4 (lambda_r g_s + lambda_s g_r)).
template <int DIM>
struct P2Basis {
    int p1, p2;
    bool vtx;
    __device__ __forceinline__ explicit P2Basis(int J) {
        vtx = J <= DIM;
        int r = 0, s = 0;
        edge_vertices<DIM>(vtx ? 0 : J - DIM - 1, r, s);
        p1 = vtx ? J : s;
        p2 = vtx ? J : r;
    }
    __device__ __forceinline__ double c1(int a) const {
        return vtx ? (a == p1 ? 3.0 : -1.0) : (a == p2 ? 4.0 : 0.0);
    }
    __device__ __forceinline__ double c2(int a) const { return vtx ? 0.0 : (a == p1 ? 4.0 : 0.0); }
    __device__ __forceinline__ double d1() const { return vtx ? 3.0 - DIM : 4.0; }
    __device__ __forceinline__ double d2() const { return vtx ? 0.0 : 4.0; }
};

// P2 mass matrix of the element, int_K phi_i phi_j = |K| kP2Mass*[i][j] / den (exact integrals
// of the degree-4 products of the vertex functions l(2l-1) and edge functions 4 l_p l_q,
// int_K l^a = |K| d! prod a_i! / (d + |a|)!), local order as the P2 basis above
__device__ __constant__ signed char kP2Mass2[6][6] = {{6, -1, -1, -4, 0, 0},  {-1, 6, -1, 0, -4, 0},
                                                     {-1, -1, 6, 0, 0, -4},  {-4, 0, 0, 32, 16, 16},
                                                     {0, -4, 0, 16, 32, 16}, {0, 0, -4, 16, 16, 32}};
__device__ __constant__ signed char kP2Mass3[10][10] = {
    {6, 1, 1, 1, -4, -4, -4, -6, -6, -6},   {1, 6, 1, 1, -4, -6, -6, -4, -4, -6},
    {1, 1, 6, 1, -6, -4, -6, -4, -6, -4},   {1, 1, 1, 6, -6, -6, -4, -6, -4, -4},
    {-4, -4, -6, -6, 32, 16, 16, 16, 16, 8}, {-4, -6, -4, -6, 16, 32, 16, 16, 8, 16},
    {-4, -6, -6, -4, 16, 16, 32, 8, 16, 16}, {-6, -4, -4, -6, 16, 16, 8, 32, 16, 16},
    {-6, -4, -6, -4, 16, 8, 16, 16, 32, 16}, {-6, -6, -4, -4, 8, 16, 16, 16, 16, 32}};

template <int DIM>
__device__ __forceinline__ double p2_mass(int i, int j) {
    return DIM == 3 ? kP2Mass3[i][j] * (1.0 / 420.0) : kP2Mass2[i][j] * (1.0 / 180.0);
}

// The 3x3 matrix (1/m) int_K d_a(phi_I) d_b(phi_J) = sum_c C_I[c]_a C_J[c]_b + S_I,a S_J,b as a sum
// of at most three outer products u_k (x) w_k:
//   I vertex i:   u = g_i,  w = 4 C_J[i] - (d-2) S_J                    (rank 1)
//   I edge (p,q): 4 g_q (x) C_J[p] + 4 g_p (x) C_J[q] + S_I (x) S_J    (rank 3)
// The I type is the same on every lane of a warp (a row's node is either a vertex or an edge
// of all its elements); the J side is evaluated without branches.
template <int DIM>
struct P2Pair {
    V3 u0, w0, u1, w1, u2, w2;
    bool vertex;
    __device__ __forceinline__ P2Pair(const double *G, int I, int Jidx) {
        const P2Basis<DIM> J(Jidx);
        const V3 g1 = v3(G + 3 * J.p1), g2 = v3(G + 3 * J.p2);
        vertex = I <= DIM;
        if (vertex) {
            u0 = v3(G + 3 * I);
            // 4 C_J[i] - (d-2) S_J, with the coefficients selected, not branched on
            const double a1 = 4.0 * J.c1(I) - (DIM - 2) * J.d1(), a2 = 4.0 * J.c2(I) - (DIM - 2) * J.d2();
            w0 = a1 * g1 + a2 * g2;
            u1 = w1 = u2 = w2 = V3{0.0, 0.0, 0.0};
        } else {
            int p, q;
            edge_vertices<DIM>(I - DIM - 1, p, q);
            const V3 gp = v3(G + 3 * p), gq = v3(G + 3 * q);
            u0 = 4.0 * gq; w0 = J.c1(p) * g1 + J.c2(p) * g2;
            u1 = 4.0 * gp; w1 = J.c1(q) * g1 + J.c2(q) * g2;
            u2 = 4.0 * (gp + gq); w2 = J.d1() * g1 + J.d2() * g2;
        }
    }
    __device__ __forceinline__ double g(int a, int b) const {
        double t = comp(u0, a) * comp(w0, b);
        if (!vertex) t += comp(u1, a) * comp(w1, b) + comp(u2, a) * comp(w2, b);
        return t;
    }
    __device__ __forceinline__ double trace() const {
        double t = u0.x * w0.x + u0.y * w0.y + u0.z * w0.z;
        if (!vertex) t += u1.x * w1.x + u1.y * w1.y + u1.z * w1.z + u2.x * w2.x + u2.y * w2.y + u2.z * w2.z;
        return t;
    }
};

// int_K phi_i for the linear form with a constant source on the element
template <int DIM, int ORDER>
__device__ __forceinline__ double basis_integral(double meas, int i) {
    if (ORDER == 1) return meas / (DIM + 1);
    if (DIM == 3) return i < 4 ? -meas / 20.0 : meas / 5.0;
    return i < 3 ? 0.0 : meas / 3.0;
}

// ------------------------------------------------------------------ row gather (both passes)
// Register path for rows with at most 32 distinct neighbours: the candidates are read 32 at
// a time, duplicates inside a batch are merged with __match_any_sync, the new ones are
// appended to a list held one entry per lane, and the list is sorted by a 32-lane bitonic
// network on shuffles.  Returns the degree, or -1 when the row has more than 32 neighbours.
__device__ int gather_row_small(int b, int m, const int32_t *inc_elem, const int32_t *nodes, int nn, int *s) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    int u = 0, mine = 0x7fffffff;
    for (int p0 = 0; p0 < m; p0 += 32) {
        const int p = p0 + lane;
        int v = 0x7fffffff;
        if (p < m) {
            const int t = p / nn, i = p - t * nn;
            v = nodes[(int64_t)inc_elem[b + t] * nn + i];
        }
        const unsigned grp = __match_any_sync(full, v);
        bool fresh = v != 0x7fffffff && lane == __ffs(grp) - 1;
        for (int L = 0; L < u; ++L) fresh &= __shfl_sync(full, mine, L) != v;
        const unsigned bal = __ballot_sync(full, fresh);
        const int cnt = __popc(bal);
        if (u + cnt > 32) return -1;
        if (fresh) s[u + __popc(bal & ((1u << lane) - 1u))] = v;
        __syncwarp();
        if (lane >= u && lane < u + cnt) mine = s[lane];
        __syncwarp();
        u += cnt;
    }
    // ascending bitonic sort of one value per lane (unused lanes hold INT_MAX)
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int o = __shfl_xor_sync(full, mine, j);
            const bool lower = (lane & j) == 0, up = (lane & k) == 0;
            mine = (lower == up) ? min(mine, o) : max(mine, o);
        }
    if (lane < u) s[lane] = mine;
    __syncwarp();
    return u;
}

// Gathers the candidate neighbour nodes of node a into s, sorts and compacts them in
// place; returns the row degree (or -1 on overflow).
__device__ int gather_row(int a, const int32_t *inc_ptr, const int32_t *inc_elem,
                          const int32_t *nodes, int nn, int *s, int *status) {
    const int lane = threadIdx.x & 31;
    int b = inc_ptr[a], e = inc_ptr[a + 1];
    int m = (e - b) * nn;
    if (m > kCandMax) { if (lane == 0) dev_fail(status, kDevCandOverflow); return -1; }
    if (nn <= 4) {
        const int u = gather_row_small(b, m, inc_elem, nodes, nn, s);
        if (u >= 0) return u;
    }
    int P = pow2_ceil(max(m, 32));
    for (int p = lane; p < P; p += 32) {
        int v = 0x7fffffff;
        if (p < m) {
            int t = p / nn, i = p - t * nn;
            v = nodes[(int64_t)inc_elem[b + t] * nn + i];
        }
        s[p] = v;
    }
    __syncwarp();
    warp_bitonic_sort(s, P);
    int count = 0, prev = (int)0x80000000;
    for (int c = 0; c < P; c += 32) {
        int v = s[c + lane];
        int vp = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0) vp = prev;
        bool f = (v != 0x7fffffff) && (v != vp);
        unsigned bal = __ballot_sync(0xffffffffu, f);
        prev = __shfl_sync(0xffffffffu, v, 31);
        __syncwarp();
        if (f) s[count + __popc(bal & ((1u << lane) - 1u))] = v;
        count += __popc(bal);
        __syncwarp();
    }
    return count;
}

__global__ void row_count_kernel(int nnodes, const int32_t *inc_ptr, const int32_t *inc_elem,
                                 const int32_t *nodes, int nn, int32_t *deg, int *status) {
    __shared__ int sh[4][kCandMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int a = blockIdx.x * 4 + w; a < nnodes; a += gridDim.x * 4) {
        int d = gather_row(a, inc_ptr, inc_elem, nodes, nn, sh[w], status);
        if (lane == 0) deg[a] = d < 0 ? 0 : d;
        __syncwarp();
    }
}

// ------------------------------------------------------------------ fill + numeric pass
struct FillArgs {
    int nnodes, nt;
    const int32_t *inc_ptr, *inc_elem;
    const uint8_t *inc_loc;
    const int32_t *nodes;
    const double *geo;
    const int32_t *browptr;
    int32_t *bcol;            // NULL: numeric only (pattern already built)
    const int32_t *pcol;      // numeric only: the stored pattern, read instead of re-gathering rows
    int32_t *diagpos;         // block index of the diagonal block, written with the pattern
    double *val;              // NULL: no matrix (linear form only)
    double *rhs;              // NULL: no linear form
    const double *fP0;        // nt*bs or NULL
    const double *fint;       // element vectors of a source at quadrature points, or NULL
    const double *mloc;       // element mass matrices of a coefficient at quadrature points, or NULL
    const double *kloc;       // element stiffness matrices of a coefficient at quadrature points, or NULL
    const double *tloc;       // element matrices of the general volume terms (ffgpu_varf.terms), or NULL
    const double *lame;       // per-element (lambda, mu) of the elasticity form, or NULL
    const double *eloc;       // [P2]^3 element blocks from the tensor cores (ffgpu_elemtc.cu), or NULL
    double f0, f1, f2;
    double c_mass;
    double lam, mu;           // elasticity
    const uint8_t *onbc;
    const double *g;
    double tgv;
    int max_deg;
    int *status;
    // boundary terms (NULL bptr: none): node -> codes b*NN + il, element vectors / matrices
    const int32_t *bptr, *blist, *bel_elem;
    const double *brhs, *bmat;
};

// FE: 1 = P1 scalar, 2 = P2 scalar, 3 = [P2]^3 elasticity
template <int DIM, int FE>
__global__ void __launch_bounds__(128) row_fill_kernel(FillArgs A) {
    constexpr int nvk = DIM + 1;
    constexpr int NN = FE == 1 ? nvk : (DIM == 3 ? 10 : 6);
    constexpr int BS = FE == 3 ? 3 : 1;
    constexpr int BS2 = BS * BS;
    // lanes = slot * NN + lb: SLOTS incident elements per step, each lane one block (la, lb).
    // Every slot accumulates into its own copy of the row (acc[slot][k][q]) so that one step
    // is one full-warp FP64 add; the copies are summed in slot order at the end.  Entries are
    // therefore formed as sum_s (sum of the slot's elements in element order): deterministic,
    // and the same association rhs_kernel uses for the linear form.
    constexpr int SLOTS = 32 / NN;
    extern __shared__ __align__(16) unsigned char sh_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    int *cols = (int *)sh_raw + w * kCandMax;
    double *acc = (double *)((int *)sh_raw + warps * kCandMax) + (int64_t)w * SLOTS * A.max_deg * BS2;
    const double mfac = DIM == 3 ? 1.0 / 20.0 : 1.0 / 12.0;
    const bool has_mass = A.c_mass != 0.0 && !A.mloc;

    for (int a = blockIdx.x * warps + w; a < A.nnodes; a += gridDim.x * warps) {
        int deg;
        if (A.pcol) {
            // the row's sorted columns as the pattern pass stored them
            const int64_t r0 = A.browptr[a];
            deg = (int)(A.browptr[a + 1] - r0);
            if (deg > kCandMax) { if (lane == 0) dev_fail(A.status, kDevCandOverflow); continue; }
            for (int r = lane; r < deg; r += 32) cols[r] = A.pcol[r0 + r];
            __syncwarp();
        } else {
            deg = gather_row(a, A.inc_ptr, A.inc_elem, A.nodes, NN, cols, A.status);
        }
        if (deg < 0) continue;
        if (deg > A.max_deg) { if (lane == 0) dev_fail(A.status, kDevDegOverflow); continue; }
        const int64_t rb = A.browptr[a];
        if (A.bcol)
            for (int r = lane; r < deg; r += 32) A.bcol[rb + r] = cols[r];
        const int span = deg * BS2;   // one slot copy
        for (int q = lane; q < SLOTS * span; q += 32) acc[q] = 0.0;
        double racc = 0.0;   // rhs partial of slot `lane / NN`, component `lane % NN` (< BS)
        __syncwarp();
        const int ib = A.inc_ptr[a], ie = A.inc_ptr[a + 1];
        for (int t0 = ib; t0 < ie; t0 += SLOTS) {
            // ---- element contributions of this step
            const int slot = lane / NN;
            const int lb = lane - slot * NN;
            const int t = t0 + slot;
            const bool act = slot < SLOTS && t < ie;
            int rank = -1;
            double v[BS2];
#pragma unroll
            for (int q = 0; q < BS2; ++q) v[q] = 0.0;
            if (act) {
                const int e = A.inc_elem[t];
                const int la = A.inc_loc[t];
                const double *ge = A.geo + (int64_t)e * kGeoStride;
                const double meas = __ldg(ge), kap = __ldg(ge + 1);
                const double *G = ge + 4;
                const int nb = A.nodes[(int64_t)e * NN + lb];
                rank = find_sorted(cols, deg, nb);
                if (FE == 1) {
                    double s = 0;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) s += __ldg(G + 3 * la + d) * __ldg(G + 3 * lb + d);
                    double val = A.kloc ? A.kloc[((int64_t)e * NN + la) * NN + lb] : kap * meas * s;
                    if (has_mass) val += A.c_mass * meas * mfac * (la == lb ? 2.0 : 1.0);
                    if (A.mloc) val += A.mloc[((int64_t)e * NN + la) * NN + lb];
                    if (A.tloc) val += A.tloc[((int64_t)e * NN + la) * NN + lb];
                    v[0] = val;
                } else if (FE == 2) {
                    const double m = meas * mfac;
                    v[0] = A.kloc ? A.kloc[((int64_t)e * NN + la) * NN + lb] : kap * m * P2Pair<DIM>(G, la, lb).trace();
                    if (has_mass) v[0] += A.c_mass * meas * p2_mass<DIM>(la, lb);
                    if (A.mloc) v[0] += A.mloc[((int64_t)e * NN + la) * NN + lb];
                    if (A.tloc) v[0] += A.tloc[((int64_t)e * NN + la) * NN + lb];
                } else if (A.eloc) {
                    const double *eb = A.eloc + (((int64_t)e * NN + la) * NN + lb) * BS2;
#pragma unroll
                    for (int q = 0; q < BS2; ++q) v[q] = __ldg(eb + q);
                } else {
                    const P2Pair<DIM> P(G, la, lb);
                    const double m = meas * mfac;
                    {
                        const double tr = P.trace();
                        const double lam = A.lame ? __ldg(A.lame + 2 * (int64_t)e) : A.lam;
                        const double mu = A.lame ? __ldg(A.lame + 2 * (int64_t)e + 1) : A.mu;
#pragma unroll
                        for (int c = 0; c < 3; ++c)
#pragma unroll
                            for (int cp = 0; cp < 3; ++cp) {
                                double x = lam * P.g(c, cp) + mu * P.g(cp, c);
                                if (cp == c) x += mu * tr;
                                v[3 * c + cp] = m * x;
                            }
                    }
                }
                if (rank < 0) dev_fail(A.status, kDevNotFound);
            }
            // ---- accumulate: each slot into its own copy, no two lanes on one entry
            if (act && rank >= 0) {
#pragma unroll
                for (int q = 0; q < BS2; ++q) acc[slot * span + rank * BS2 + q] += v[q];
            }
            // ---- linear form: lane (slot, c < BS) adds its element's share to component c
            if (A.rhs && act && lb < BS) {
                const int ee = A.inc_elem[t], ll = A.inc_loc[t];
                const double meas = A.geo[(int64_t)ee * kGeoStride];
                const double f = A.fP0 ? A.fP0[(int64_t)ee * BS + lb] : (lb == 0 ? A.f0 : (lb == 1 ? A.f1 : A.f2));
                // explicit roundings: the linear-form-only kernel forms the same sums bit for bit
                const double add = A.fint ? A.fint[((int64_t)ee * NN + ll) * BS + lb]
                                          : __dmul_rn(__dmul_rn(meas, f), FE == 1 ? 1.0 / (DIM + 1)
                                                                                  : basis_integral<DIM, 2>(1.0, ll));
                racc = __dadd_rn(racc, add);
            }
            __syncwarp();
        }
        // ---- sum the slot copies (slot order); slots no element reached hold zeros and are
        // skipped (a row with ie - ib < SLOTS incident elements fills only that many)
        const int nsl = min(SLOTS, ie - ib);
        for (int q = lane; q < span; q += 32) {
            double t = acc[q];
            for (int sl = 1; sl < nsl; ++sl) t += acc[sl * span + q];
            acc[q] = t;
        }
        {
            double r = 0.0;
            for (int sl = 0; sl < max(nsl, 1); ++sl) {
                const double p = __shfl_sync(0xffffffffu, racc, sl * NN + (lane < BS ? lane : 0));
                r = sl == 0 ? p : r + p;
            }
            racc = r;   // lanes < BS: component `lane`
        }
        __syncwarp();
        // ---- boundary terms, boundary element by boundary element, after the volume sum
        if (A.bptr) {
            const int p1 = A.bptr[a + 1];
            for (int p = A.bptr[a]; p < p1; ++p) {
                const int code = A.blist[p];
                const int bb = code / NN, il = code - bb * NN;
                if (A.bmat && A.val && lane < NN) {
                    const int cn = A.nodes[(int64_t)A.bel_elem[bb] * NN + lane];
                    const int rk = find_sorted(cols, deg, cn);
                    const double m = A.bmat[((int64_t)bb * NN + il) * NN + lane];
                    if (rk < 0) dev_fail(A.status, kDevNotFound);
                    else
#pragma unroll
                        for (int c = 0; c < BS; ++c) acc[rk * BS2 + c * BS + c] += m;
                }
                if (A.brhs && A.rhs && lane < BS) racc += A.brhs[((int64_t)bb * BS + lane) * NN + il];
                __syncwarp();
            }
        }
        // ---- Dirichlet rows (tgv > 0): diagonal := tgv, rhs := tgv * g
        int self = find_sorted(cols, deg, a);
        if (self < 0) { if (lane == 0) dev_fail(A.status, kDevNotFound); continue; }
        if (A.bcol && lane == 0) A.diagpos[a] = (int32_t)(rb + self);
        if (lane < BS) {
            int64_t dof = (int64_t)a * BS + lane;
            bool on = A.onbc && A.onbc[dof];
            if (on && A.tgv > 0) {
                if (A.val) acc[self * BS2 + lane * BS + lane] = A.tgv;
                racc = A.tgv * (A.g ? A.g[dof] : 0.0);
            } else if (on) {
                racc = A.g ? A.g[dof] : 0.0;   // tgv < 0: b_i = g_i (tgv1 = 1, problem.cpp:9937)
            }
            if (A.rhs) A.rhs[dof] = racc;
        }
        __syncwarp();
        // tgv < 0 (HashMatrix::SetBC, HashMatrix.cpp:1195-1238): Dirichlet rows get a unit
        // diagonal (0 when tgv <= -10) and, except for -3/-30, zero off-diagonals; for
        // -2/-20/-3/-30 the Dirichlet columns are zeroed too (the diagonal also for -20/-30).
        if (A.val && A.onbc && A.tgv < 0) {
            const double tgv = A.tgv;
            const bool keep_row = fabs(tgv + 3.0) < 1e-10 || fabs(tgv + 30.0) < 1e-10;
            const bool zero_col = fabs(tgv + 2.0) < 1e-10 || fabs(tgv + 20.0) < 1e-10 || fabs(tgv + 3.0) < 1e-10 ||
                                  fabs(tgv + 30.0) < 1e-10;
            for (int q = lane; q < deg * BS2; q += 32) {
                const int k = q / BS2, r = (q % BS2) / BS, cp = q % BS;
                const int col = cols[k];
                const bool diag = col == a && r == cp;
                double v = acc[q];
                if (A.onbc[(int64_t)a * BS + r]) v = diag ? (tgv < -9.0 ? 0.0 : 1.0) : (keep_row ? v : 0.0);
                if (zero_col && A.onbc[(int64_t)col * BS + cp] && (!diag || tgv < -19.0)) v = 0.0;
                acc[q] = v;
            }
            __syncwarp();
        }
        if (A.val)
            for (int q = lane; q < deg * BS2; q += 32) A.val[rb * BS2 + q] = acc[q];
        __syncwarp();
    }
}

// linear form only (real[int] b = a(0,Vh)): per node, sum over incident elements
template <int DIM, int FE>
__global__ void rhs_kernel(int nnodes, const int32_t *inc_ptr, const int32_t *inc_elem,
                           const uint8_t *inc_loc, const double *geo, const double *fP0,
                           const double *fint, double f0, double f1, double f2, const uint8_t *onbc,
                           const double *g,
                           double tgv, double *rhs, const int32_t *bptr, const int32_t *blist,
                           const double *brhs) {
    constexpr int BS = FE == 3 ? 3 : 1;
    // same association as the fill kernel's fused linear form: element p of the node goes to
    // partial p % SLOTS, partials summed in order
    constexpr int NN = FE == 1 ? DIM + 1 : (DIM == 3 ? 10 : 6);
    constexpr int SLOTS = 32 / NN;
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nnodes * BS) return;
    int a = (int)(t / BS), c = (int)(t % BS);
    double part[SLOTS];
#pragma unroll
    for (int sl = 0; sl < SLOTS; ++sl) part[sl] = 0.0;
    const int ib = inc_ptr[a], ie = inc_ptr[a + 1];
    for (int p0 = ib; p0 < ie; p0 += SLOTS) {
#pragma unroll
        for (int sl = 0; sl < SLOTS; ++sl) {
            const int p = p0 + sl;
            if (p < ie) {
                int e = inc_elem[p], l = inc_loc[p];
                double meas = geo[(int64_t)e * kGeoStride];
                double f = fP0 ? fP0[(int64_t)e * BS + c] : (c == 0 ? f0 : (c == 1 ? f1 : f2));
                const double add = fint ? fint[((int64_t)e * NN + l) * BS + c]
                                        : __dmul_rn(__dmul_rn(meas, f), FE == 1 ? 1.0 / (DIM + 1)
                                                                                : basis_integral<DIM, 2>(1.0, l));
                part[sl] = __dadd_rn(part[sl], add);
            }
        }
    }
    double s = part[0];
#pragma unroll
    for (int sl = 1; sl < SLOTS; ++sl) s += part[sl];
    if (bptr)   // boundary terms, in boundary-element order, after the volume terms
        for (int p = bptr[a]; p < bptr[a + 1]; ++p) {
            const int code = blist[p];
            const int bb = code / NN, il = code - bb * NN;
            s += brhs[((int64_t)bb * BS + c) * NN + il];
        }
    if (onbc && onbc[t]) s = (tgv > 0 ? tgv : 1.0) * (g ? g[t] : 0.0);
    rhs[t] = s;
}

// ------------------------------------------------------------------ CSR export
__global__ void export_csr_kernel(int nb, int bs, const int32_t *browptr, const int32_t *bcol,
                                  const double *val, int32_t *rowptr, int32_t *col, double *out) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nb) return;
    int64_t b0 = browptr[a], deg = browptr[a + 1] - b0;
    for (int c = 0; c < bs; ++c) {
        int64_t r0 = b0 * bs * bs + c * bs * deg;
        rowptr[(int64_t)a * bs + c] = (int32_t)r0;
        for (int64_t k = 0; k < deg; ++k)
            for (int cp = 0; cp < bs; ++cp) {
                col[r0 + k * bs + cp] = bs * bcol[b0 + k] + cp;
                out[r0 + k * bs + cp] = val[(b0 + k) * bs * bs + c * bs + cp];
            }
    }
    if (a == nb - 1) rowptr[(int64_t)nb * bs] = (int32_t)((int64_t)browptr[nb] * bs * bs);
}

// ------------------------------------------------------------------ on(labels): DOF marking
// AssembleBC (problem.cpp:9881-10034) marks the DOFs of the boundary elements carrying one of
// the labels.  On the device: (1) vertices of the selected boundary elements, (2) vertex nodes
// of those vertices, (3) edge nodes whose two endpoints lie on one common selected boundary
// element (scanning the vertex -> boundary-element incidence of one endpoint).
__device__ __forceinline__ bool label_selected(int lab, int nlabels, const int32_t *labels) {
    for (int k = 0; k < nlabels; ++k)
        if (labels[k] == lab) return true;
    return false;
}

__global__ void bmark_vertices_kernel(int nbe, int bdim, const int32_t *belems, const int32_t *blabel,
                                      int nlabels, const int32_t *labels, uint8_t *vmark) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbe || !label_selected(blabel[b], nlabels, labels)) return;
    for (int k = 0; k < bdim; ++k) vmark[belems[(int64_t)b * bdim + k]] = 1;
}

__device__ __forceinline__ void mark_node(uint8_t *onbc, int node, int bs, int comp_mask) {
    for (int c = 0; c < bs; ++c)
        if (comp_mask == 0 || (comp_mask >> c) & 1) onbc[(int64_t)node * bs + c] = 1;
}

template <int DIM>
__global__ void bmark_nodes_kernel(int nt, int nn, const int32_t *elems, const int32_t *nodes, const uint8_t *vmark,
                                   const int32_t *bv_ptr, const int32_t *bv_elem, const int32_t *belems,
                                   const int32_t *blabel, int nlabels, const int32_t *labels, int bs,
                                   int comp_mask, uint8_t *onbc) {
    constexpr int NV = DIM + 1;
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nt * nn) return;
    int e = (int)(t / nn), i = (int)(t % nn);
    const int32_t *v = elems + (int64_t)e * NV;
    if (i < NV) {
        if (vmark[v[i]]) mark_node(onbc, nodes[t], bs, comp_mask);
        return;
    }
    int p, q;
    edge_vertices<DIM>(i - NV, p, q);
    int a = v[p], b = v[q];
    if (!vmark[a] || !vmark[b]) return;
    for (int k = bv_ptr[a]; k < bv_ptr[a + 1]; ++k) {
        int f = bv_elem[k];
        if (!label_selected(blabel[f], nlabels, labels)) continue;
        const int32_t *fv = belems + (int64_t)f * DIM;
        bool has_b = false;
        for (int j = 0; j < DIM; ++j) has_b |= fv[j] == b;
        if (has_b) { mark_node(onbc, nodes[t], bs, comp_mask); return; }
    }
}

__global__ void bcount_kernel(int nbe, int bdim, const int32_t *belems, int32_t *cnt) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < (int64_t)nbe * bdim) atomicAdd(&cnt[belems[t]], 1);
}

__global__ void bfill_kernel(int nbe, int bdim, const int32_t *belems, const int32_t *ptr, int32_t *cursor,
                             int32_t *out) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nbe * bdim) return;
    int v = belems[t];
    out[ptr[v] + atomicAdd(&cursor[v], 1)] = (int32_t)(t / bdim);
}

__global__ void row_degree_kernel(int n, const int32_t *rp, int32_t *deg) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) deg[a] = rp[a + 1] - rp[a];
}

// diagonal block of each row of a sorted CSR (-1 if absent)
__global__ void diagpos_kernel(int n, const int32_t *rp, const int32_t *col, int32_t *pos) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int lo = rp[a], hi = rp[a + 1] - 1, p = -1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int c = col[mid];
        if (c == a) { p = mid; break; }
        if (c < a) lo = mid + 1; else hi = mid - 1;
    }
    pos[a] = p;
}

static int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

int space_bc_mask_device(ffgpu_space *S, int nlabels, const int32_t *labels, int comp_mask, uint8_t *onbc) {
    FFGPU_CHECK(S->belems, FFGPU_EINVAL, "on(labels): the space has no boundary elements (ffgpu_space_set_boundary)");
    FFGPU_CHECK(nlabels > 0 && nlabels <= 64 && labels, FFGPU_EINVAL, "on(labels): 1..64 labels expected");
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    DevIn<int32_t> lab(labels, nlabels, ctx);
    FFGPU_TRY(lab.err);
    FFGPU_CUDA(cudaMemsetAsync(S->vmark, 0, S->nv, s));
    FFGPU_CUDA(cudaMemsetAsync(onbc, 0, S->ndof, s));
    bmark_vertices_kernel<<<grid_for(S->nbe, 256), 256, 0, s>>>(S->nbe, S->dim, S->belems, S->blabel, nlabels,
                                                                 lab.d, S->vmark);
    FFGPU_TRY(launch_check(ctx, "bmark_vertices"));
    int64_t m = (int64_t)S->nt * S->nn;
    if (S->dim == 2)
        bmark_nodes_kernel<2><<<grid_for(m, 256), 256, 0, s>>>(S->nt, S->nn, S->elems, S->nodes, S->vmark, S->bv_ptr,
                                                               S->bv_elem, S->belems, S->blabel, nlabels, lab.d,
                                                               S->bs, comp_mask, onbc);
    else
        bmark_nodes_kernel<3><<<grid_for(m, 256), 256, 0, s>>>(S->nt, S->nn, S->elems, S->nodes, S->vmark, S->bv_ptr,
                                                               S->bv_elem, S->belems, S->blabel, nlabels, lab.d,
                                                               S->bs, comp_mask, onbc);
    return launch_check(ctx, "bmark_nodes");
}

}  // namespace ffgpu

using namespace ffgpu;

// ------------------------------------------------------------------ helpers on the host
static int fill_launch(ffgpu_space *S, FillArgs &fa) {
    ffgpu_ctx *ctx = S->ctx;
    const int warps = 4;
    int bs2 = S->bs * S->bs;
    const int nn = S->nn, slots = 32 / nn;
    size_t smem = (size_t)warps * kCandMax * sizeof(int) + (size_t)warps * slots * fa.max_deg * bs2 * sizeof(double);
    int grid = min(kNumSM * 16, max(1, (S->nnodes + warps - 1) / warps));
    void (*kern)(FillArgs) = nullptr;
    if (S->dim == 2 && S->fe == FFGPU_FE_P1) kern = row_fill_kernel<2, 1>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P1) kern = row_fill_kernel<3, 1>;
    if (S->dim == 2 && S->fe == FFGPU_FE_P2) kern = row_fill_kernel<2, 2>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2) kern = row_fill_kernel<3, 2>;
    if (S->dim == 3 && S->fe == FFGPU_FE_P2VEC3) kern = row_fill_kernel<3, 3>;
    FFGPU_CHECK(kern, FFGPU_EINVAL, "unsupported element (dim %d, fe %d)", S->dim, S->fe);
    FFGPU_CHECK(smem <= 200 * 1024, FFGPU_EMESH, "row degree %d too large for shared memory", fa.max_deg);
    FFGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, warps * 32, smem, ctx->stream>>>(fa);
    return launch_check(ctx, "row_fill_kernel");
}

static int varf_check(const ffgpu_space *S, const ffgpu_varf *v) {
    FFGPU_CHECK(v, FFGPU_EINVAL, "varf is NULL");
    if (v->form == FFGPU_FORM_ELASTICITY)
        FFGPU_CHECK(S->fe == FFGPU_FE_P2VEC3, FFGPU_EINVAL, "elasticity needs the [P2,P2,P2] space");
    else
        FFGPU_CHECK(v->form == FFGPU_FORM_DIFFUSION && S->fe != FFGPU_FE_P2VEC3, FFGPU_EINVAL,
                    "unsupported form %d for this space", v->form);
    return FFGPU_OK;
}

static int run_geometry(ffgpu_space *S, const ffgpu_varf *v, double *geo) {
    ffgpu_ctx *ctx = S->ctx;
    DevIn<double> kap(v->kappa, v->kappa ? S->nt : 0, ctx);
    FFGPU_TRY(kap.err);
    double cs = v->form == FFGPU_FORM_DIFFUSION ? v->c_stiff : 1.0;
    geometry_kernel<<<grid_for(S->nt, 256), 256, 0, ctx->stream>>>(S->coords, S->elems, S->nt, S->dim,
                                                                   kap.d, cs, geo);
    return launch_check(ctx, "geometry_kernel");
}

static int numeric_pass(ffgpu_matrix *M, const ffgpu_varf *v, const ffgpu_bc *bc, double *rhs,
                        bool build_cols) {
    ffgpu_space *S = M->space;
    ffgpu_ctx *ctx = S->ctx;
    FFGPU_TRY(varf_check(S, v));
    FFGPU_TRY(run_geometry(S, v, M->geo));
    int bs = S->bs;
    DevIn<double> fP0(v->f, v->f ? (size_t)S->nt * bs : 0, ctx);
    DevIn<uint8_t> onbc(bc ? bc->onbc : nullptr, bc && bc->onbc ? S->ndof : 0, ctx);
    DevIn<double> gv(bc ? bc->g : nullptr, bc && bc->g ? S->ndof : 0, ctx);
    DevOut<double> rh(rhs, rhs ? S->ndof : 0, ctx, false);
    FFGPU_TRY(fP0.err); FFGPU_TRY(onbc.err); FFGPU_TRY(gv.err); FFGPU_TRY(rh.err);
    const uint8_t *mask = onbc.d;
    if (bc && !bc->onbc && bc->nlabels > 0) {
        if (!M->bcmask) FFGPU_CUDA(dalloc(ctx, (void **)&M->bcmask, S->ndof));
        FFGPU_TRY(space_bc_mask_device(S, bc->nlabels, bc->labels, bc->comp_mask, M->bcmask));
        mask = M->bcmask;
    }
    FillArgs fa;
    memset(&fa, 0, sizeof(fa));
    fa.nnodes = S->nnodes; fa.nt = S->nt;
    fa.inc_ptr = S->inc_ptr; fa.inc_elem = S->inc_elem; fa.inc_loc = S->inc_loc;
    fa.nodes = S->nodes; fa.geo = M->geo; fa.browptr = M->browptr;
    fa.bcol = build_cols ? M->bcol : nullptr;
    fa.pcol = build_cols ? nullptr : M->bcol;
    fa.diagpos = M->diagpos;
    fa.val = M->val; fa.rhs = rh.d; fa.fP0 = fP0.d;
    fa.f0 = v->f_const[0]; fa.f1 = v->f_const[1]; fa.f2 = v->f_const[2];
    fa.c_mass = v->form == FFGPU_FORM_DIFFUSION ? v->c_mass : 0.0;
    if (v->form == FFGPU_FORM_ELASTICITY) {
        fa.mu = v->E / (2 * (1 + v->nu));
        fa.lam = v->E * v->nu / ((1 + v->nu) * (1 - 2 * v->nu));
    }
    fa.onbc = mask; fa.g = gv.d; fa.tgv = bc ? bc->tgv : 0.0;
    fa.max_deg = M->max_deg; fa.status = ctx->d_status;
    DevIn<double> lame(v->form == FFGPU_FORM_ELASTICITY ? v->lame : nullptr, (size_t)S->nt * 2, ctx);
    FFGPU_TRY(lame.err);
    fa.lame = lame.d;
    double *fint = nullptr, *mloc = nullptr;
    if (rh.d) FFGPU_TRY(source_prepare(S, v, M->geo, &fint));
    double *kloc = nullptr, *tloc = nullptr;
    int frc = mass_prepare(S, v, M->geo, &mloc);
    if (!frc) frc = stiff_prepare(S, v, M->geo, &kloc);
    if (!frc) frc = terms_prepare(S, v, M->geo, &tloc);
    // P2 stiffness / [P2]^3 elasticity with an element-constant coefficient: the element
    // matrices from the tensor cores (a coefficient at the rule's points keeps its own path)
    double *eloc = nullptr;
    if (!frc && !kloc && (S->fe == FFGPU_FE_P2VEC3 || (S->fe == FFGPU_FE_P2 && v->c_stiff != 0.0)))
        frc = elem_tc_prepare(S, M->geo, fa.lam, fa.mu, lame.d, &eloc);
    if (frc) { dfree(ctx, fint); dfree(ctx, mloc); dfree(ctx, kloc); dfree(ctx, tloc); return frc; }
    fa.fint = fint;
    fa.mloc = mloc;
    fa.kloc = S->fe == FFGPU_FE_P2 && eloc ? eloc : kloc;
    fa.eloc = S->fe == FFGPU_FE_P2VEC3 ? eloc : nullptr;
    fa.tloc = tloc;
    BoundaryTerms bt;
    frc = boundary_prepare(S, v, rh.d != nullptr, true, bt);
    if (!frc) {
        fa.bptr = bt.ptr; fa.blist = bt.list; fa.bel_elem = bt.bel_elem; fa.brhs = bt.rhs; fa.bmat = bt.mat;
        frc = fill_launch(S, fa);
        boundary_release(S, bt);
    }
    dfree(ctx, fint);
    dfree(ctx, mloc);
    dfree(ctx, kloc);
    dfree(ctx, tloc);
    dfree(ctx, eloc);
    FFGPU_TRY(frc);
    FFGPU_TRY(check_device_status(ctx, "assembly"));
    FFGPU_TRY(rh.finish());
    // the solver data of a previous numeric state are stale; so is a cached CG graph, which
    // holds the addresses of the derived value arrays
    M->ntgv = -1;
    if (M->val_t) { dfree(ctx, M->val_t); M->val_t = nullptr; }
    if (M->val32) { dfree(ctx, M->val32); M->val32 = nullptr; }
    if (M->valx) { dfree(ctx, M->valx); M->valx = nullptr; }
    if (M->valx_t) { dfree(ctx, M->valx_t); M->valx_t = nullptr; }
    sell_release_values(M);
    direct_invalidate(M);
    if (M->cg_exec) { cudaGraphExecDestroy(M->cg_exec); M->cg_exec = nullptr; }
    return FFGPU_OK;
}

extern "C" {

int ffgpu_space_create(ffgpu_ctx *ctx, int dim, int nv, const double *coords, int nt,
                       const int32_t *elems, int fe, int ndofK, const int32_t *dof, int ndof,
                       ffgpu_space **out) {
    FFGPU_CHECK(ctx && out && coords && elems && (dof || fe == FFGPU_FE_P1), FFGPU_EINVAL,
                "ffgpu_space_create: NULL argument");
    FFGPU_CHECK(dof || ndof == nv, FFGPU_EINVAL,
                "ffgpu_space_create: P1 without a DOF table needs ndof == nv (got %d, nv %d)", ndof, nv);
    FFGPU_CHECK(dim == 2 || dim == 3, FFGPU_EINVAL, "dim must be 2 or 3");
    FFGPU_CHECK(nv > 0 && nt > 0 && ndof > 0, FFGPU_EINVAL, "empty mesh or space");
    int nvk = dim + 1, nn, bs;
    if (fe == FFGPU_FE_P1) { nn = nvk; bs = 1; }
    else if (fe == FFGPU_FE_P2) { nn = dim == 3 ? 10 : 6; bs = 1; }
    else if (fe == FFGPU_FE_P2VEC3) { FFGPU_CHECK(dim == 3, FFGPU_EINVAL, "[P2]^3 needs dim 3"); nn = 10; bs = 3; }
    else { set_error("unknown finite element %d", fe); return FFGPU_EINVAL; }
    FFGPU_CHECK(ndofK == nn * bs, FFGPU_EINVAL, "ndofK %d does not match the element (%d)", ndofK, nn * bs);
    FFGPU_CHECK(ndof % bs == 0, FFGPU_EINVAL, "ndof %d not a multiple of %d", ndof, bs);
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    ffgpu_space *S = new ffgpu_space();
    memset(S, 0, sizeof(*S));
    S->ctx = ctx; S->dim = dim; S->nvk = nvk; S->nv = nv; S->nt = nt; S->fe = fe; S->nn = nn;
    S->bs = bs; S->ndofK = ndofK; S->ndof = ndof; S->nnodes = ndof / bs;
    int64_t m = (int64_t)nt * nn;
    int rc = FFGPU_OK;
    int32_t *cnt = nullptr;
    {
        DevIn<int32_t> D(dof, dof ? (size_t)nt * ndofK : 0, ctx);   // NULL (P1): the vertices
        if (D.err) { rc = D.err; goto fail; }
        if (dalloc(ctx, (void **)&S->coords, sizeof(double) * nv * dim) ||
            dalloc(ctx, (void **)&S->elems, sizeof(int32_t) * nt * nvk) ||
            dalloc(ctx, (void **)&S->nodes, sizeof(int32_t) * m) ||
            dalloc(ctx, (void **)&S->inc_ptr, sizeof(int32_t) * (S->nnodes + 1)) ||
            dalloc(ctx, (void **)&S->inc_elem, sizeof(int32_t) * m) ||
            dalloc(ctx, (void **)&S->inc_loc, m) ||
            dalloc(ctx, (void **)&cnt, sizeof(int32_t) * (S->nnodes + 1))) {
            set_error("ffgpu_space_create: device allocation failed");
            rc = FFGPU_ENOMEM; goto fail;
        }
        // host or device arrays, copied straight into the space's own buffers
        if (cudaMemcpyAsync(S->coords, coords, sizeof(double) * nv * dim, cudaMemcpyDefault, s) ||
            cudaMemcpyAsync(S->elems, elems, sizeof(int32_t) * nt * nvk, cudaMemcpyDefault, s)) {
            set_error("ffgpu_space_create: copy of the mesh failed");
            rc = FFGPU_ECUDA; goto fail;
        }
        check_elems_kernel<<<grid_for((int64_t)nt * nvk, 256), 256, 0, s>>>(S->elems, (int64_t)nt * nvk, nv, ctx->d_status);
        if ((rc = launch_check(ctx, "check_elems"))) goto fail;
        build_nodes_kernel<<<grid_for(m, 256), 256, 0, s>>>(dof ? D.d : S->elems, nt, ndofK, nn, bs, ndof,
                                                            S->nodes, ctx->d_status);
        if ((rc = launch_check(ctx, "build_nodes"))) goto fail;
        if ((rc = check_device_status(ctx, "ffgpu_space_create"))) goto fail;
    }
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nnodes + 1), s);
    inc_count_kernel<<<grid_for(m, 256), 256, 0, s>>>(S->nodes, m, cnt);
    if ((rc = launch_check(ctx, "inc_count"))) goto fail;
    if ((rc = device_max_i32(ctx, cnt, S->nnodes, &S->max_inc))) goto fail;
    if ((rc = device_scan_i32(ctx, cnt, S->inc_ptr, S->nnodes))) goto fail;
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nnodes + 1), s);
    inc_fill_kernel<<<grid_for(m, 256), 256, 0, s>>>(S->nodes, m, nn, S->inc_ptr, cnt, S->inc_elem, S->inc_loc);
    if ((rc = launch_check(ctx, "inc_fill"))) goto fail;
    {
        int P = 1;
        while (P < S->max_inc) P <<= 1;
        size_t smem = (size_t)4 * P * sizeof(long long);
        if (smem > 200 * 1024 || (int64_t)S->max_inc * nn > kCandMax) {
            set_error("node valence %d too high (at most %d candidate neighbours)", S->max_inc, kCandMax);
            rc = FFGPU_EMESH; goto fail;
        }
        cudaFuncSetAttribute(inc_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        inc_sort_kernel<<<min(kNumSM * 8, max(1, (S->nnodes + 3) / 4)), 128, smem, s>>>(
            S->inc_ptr, S->nnodes, S->max_inc, S->inc_elem, S->inc_loc);
        if ((rc = launch_check(ctx, "inc_sort"))) goto fail;
    }
    dfree(ctx, cnt);
    cnt = nullptr;
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        set_error("ffgpu_space_create: %s", cudaGetErrorString(cudaGetLastError()));
        rc = FFGPU_ECUDA; goto fail;
    }
    *out = S;
    return FFGPU_OK;
fail:
    if (cnt) dfree(ctx, cnt);
    ffgpu_space_destroy(S);
    return rc;
}

int ffgpu_space_destroy(ffgpu_space *S) {
    if (!S) return FFGPU_OK;
    cudaStreamSynchronize(S->ctx->stream);
    dfree(S->ctx, S->coords); dfree(S->ctx, S->elems); dfree(S->ctx, S->nodes);
    dfree(S->ctx, S->inc_ptr); dfree(S->ctx, S->inc_elem); dfree(S->ctx, S->inc_loc);
    dfree(S->ctx, S->belems); dfree(S->ctx, S->blabel); dfree(S->ctx, S->bv_ptr); dfree(S->ctx, S->bv_elem); dfree(S->ctx, S->vmark);
    dfree(S->ctx, S->bel_elem); dfree(S->ctx, S->bel_face);
    delete S;
    return FFGPU_OK;
}

int ffgpu_space_set_boundary(ffgpu_space *S, int nbe, const int32_t *belems, const int32_t *blabel) {
    FFGPU_CHECK(S && nbe > 0 && belems && blabel, FFGPU_EINVAL, "ffgpu_space_set_boundary: bad argument");
    ffgpu_ctx *ctx = S->ctx;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int bdim = S->dim;   // vertices per boundary element
    dfree(ctx, S->belems); dfree(ctx, S->blabel); dfree(ctx, S->bv_ptr); dfree(ctx, S->bv_elem); dfree(ctx, S->vmark);
    dfree(ctx, S->bel_elem); dfree(ctx, S->bel_face);
    S->belems = S->blabel = S->bv_ptr = S->bv_elem = S->bel_elem = S->bel_face = nullptr;
    S->vmark = nullptr;
    S->nbe = nbe;
    int32_t *cnt = nullptr;
    if (dalloc(ctx, (void **)&S->belems, sizeof(int32_t) * nbe * bdim) ||
        dalloc(ctx, (void **)&S->blabel, sizeof(int32_t) * nbe) ||
        dalloc(ctx, (void **)&S->bv_ptr, sizeof(int32_t) * (S->nv + 1)) ||
        dalloc(ctx, (void **)&S->bv_elem, sizeof(int32_t) * nbe * bdim) ||
        dalloc(ctx, (void **)&S->vmark, S->nv) ||
        dalloc(ctx, (void **)&cnt, sizeof(int32_t) * (S->nv + 1))) {
        set_error("ffgpu_space_set_boundary: device allocation failed");
        dfree(ctx, cnt);
        return FFGPU_ENOMEM;
    }
    FFGPU_CUDA(cudaMemcpyAsync(S->belems, belems, sizeof(int32_t) * nbe * bdim, cudaMemcpyDefault, s));
    FFGPU_CUDA(cudaMemcpyAsync(S->blabel, blabel, sizeof(int32_t) * nbe, cudaMemcpyDefault, s));
    check_elems_kernel<<<grid_for((int64_t)nbe * bdim, 256), 256, 0, s>>>(S->belems, (int64_t)nbe * bdim, S->nv,
                                                                           ctx->d_status);
    FFGPU_TRY(launch_check(ctx, "check_belems"));
    int rc = check_device_status(ctx, "ffgpu_space_set_boundary");
    if (!rc) {
        cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nv + 1), s);
        bcount_kernel<<<grid_for((int64_t)nbe * bdim, 256), 256, 0, s>>>(nbe, bdim, S->belems, cnt);
        rc = launch_check(ctx, "bcount");
    }
    if (!rc) rc = device_scan_i32(ctx, cnt, S->bv_ptr, S->nv);
    if (!rc) {
        cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (S->nv + 1), s);
        bfill_kernel<<<grid_for((int64_t)nbe * bdim, 256), 256, 0, s>>>(nbe, bdim, S->belems, S->bv_ptr, cnt,
                                                                         S->bv_elem);
        rc = launch_check(ctx, "bfill");
    }
    dfree(ctx, cnt);
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) { set_error("ffgpu_space_set_boundary failed"); rc = FFGPU_ECUDA; }
    return rc;
}

int ffgpu_space_bc_mask(ffgpu_space *S, int nlabels, const int32_t *labels, int comp_mask, uint8_t *onbc) {
    FFGPU_CHECK(S && onbc, FFGPU_EINVAL, "ffgpu_space_bc_mask: NULL argument");
    cudaStream_t s = S->ctx->stream;
    FFGPU_CUDA(cudaSetDevice(S->ctx->device));
    DevOut<uint8_t> m(onbc, S->ndof, S->ctx, false);
    FFGPU_TRY(m.err);
    FFGPU_TRY(space_bc_mask_device(S, nlabels, labels, comp_mask, m.d));
    FFGPU_TRY(m.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

int ffgpu_matrix_assemble(ffgpu_space *S, const ffgpu_varf *v, const ffgpu_bc *bc, double *rhs,
                          ffgpu_matrix **out) {
    FFGPU_CHECK(S && out, FFGPU_EINVAL, "ffgpu_matrix_assemble: NULL argument");
    FFGPU_TRY(varf_check(S, v));
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    ffgpu_matrix *M = new ffgpu_matrix();
    memset(M, 0, sizeof(*M));
    M->ctx = ctx; M->space = S; M->bs = S->bs; M->nb = S->nnodes; M->n = S->ndof;
    M->ntgv = -1; M->csr_lanes = 0;
    int rc = FFGPU_OK;
    int32_t *deg = nullptr;
    if (dalloc(ctx, (void **)&M->browptr, sizeof(int32_t) * (M->nb + 1)) ||
        dalloc(ctx, (void **)&deg, sizeof(int32_t) * (M->nb + 1)) ||
        dalloc(ctx, (void **)&M->geo, sizeof(double) * kGeoStride * S->nt)) {
        set_error("ffgpu_matrix_assemble: device allocation failed");
        rc = FFGPU_ENOMEM; goto fail;
    }
    // symbolic: row degrees, row pointer
    row_count_kernel<<<min(kNumSM * 16, max(1, (M->nb + 3) / 4)), 128, 0, s>>>(
        M->nb, S->inc_ptr, S->inc_elem, S->nodes, S->nn, deg, ctx->d_status);
    if ((rc = launch_check(ctx, "row_count"))) goto fail;
    if ((rc = check_device_status(ctx, "pattern"))) goto fail;
    if ((rc = device_max_i32(ctx, deg, M->nb, &M->max_deg))) goto fail;
    if ((rc = device_scan_i32(ctx, deg, M->browptr, M->nb))) goto fail;
    // SpMV row order: block rows grouped by degree so that the lanes of a warp share trip counts
    if (dalloc(ctx, (void **)&M->rowperm, sizeof(int32_t) * M->nb)) {
        set_error("ffgpu_matrix_assemble: device allocation failed");
        rc = FFGPU_ENOMEM; goto fail;
    }
    if ((rc = device_order_by_key_desc(ctx, deg, M->nb, M->max_deg, M->rowperm))) goto fail;
    {
        int32_t nnzb = 0;
        cudaMemcpyAsync(&nnzb, M->browptr + M->nb, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        M->nnzb = nnzb;
        M->nnz = M->nnzb * M->bs * M->bs;
    }
    dfree(ctx, deg);
    deg = nullptr;
    if (dalloc(ctx, (void **)&M->bcol, sizeof(int32_t) * M->nnzb) ||
        dalloc(ctx, (void **)&M->diagpos, sizeof(int32_t) * M->nb) ||
        dalloc(ctx, (void **)&M->val, sizeof(double) * M->nnz)) {
        set_error("ffgpu_matrix_assemble: allocation of %lld values failed", (long long)M->nnz);
        rc = FFGPU_ENOMEM; goto fail;
    }
    if ((rc = numeric_pass(M, v, bc, rhs, true))) goto fail;
    *out = M;
    return FFGPU_OK;
fail:
    if (deg) dfree(ctx, deg);
    ffgpu_matrix_destroy(M);
    return rc;
}

int ffgpu_matrix_reassemble(ffgpu_matrix *M, const ffgpu_varf *v, const ffgpu_bc *bc, double *rhs) {
    FFGPU_CHECK(M && M->space, FFGPU_EINVAL, "ffgpu_matrix_reassemble: matrix has no FE space");
    FFGPU_CUDA(cudaSetDevice(M->ctx->device));
    return numeric_pass(M, v, bc, rhs, false);
}

int ffgpu_rhs_assemble(ffgpu_space *S, const ffgpu_varf *v, const ffgpu_bc *bc, double *rhs) {
    FFGPU_CHECK(S && v && rhs, FFGPU_EINVAL, "ffgpu_rhs_assemble: NULL argument");
    FFGPU_TRY(varf_check(S, v));
    ffgpu_ctx *ctx = S->ctx;
    cudaStream_t s = ctx->stream;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    double *geo = nullptr;
    FFGPU_CUDA(dalloc(ctx, (void **)&geo, sizeof(double) * kGeoStride * S->nt));
    int rc = run_geometry(S, v, geo);
    {
        DevIn<double> fP0(v->f, v->f ? (size_t)S->nt * S->bs : 0, ctx);
        DevIn<uint8_t> onbc(bc ? bc->onbc : nullptr, bc && bc->onbc ? S->ndof : 0, ctx);
        DevIn<double> gv(bc ? bc->g : nullptr, bc && bc->g ? S->ndof : 0, ctx);
        DevOut<double> rh(rhs, S->ndof, ctx, false);
        if (!rc) rc = fP0.err ? fP0.err : (onbc.err ? onbc.err : (gv.err ? gv.err : rh.err));
        uint8_t *lmask = nullptr;
        const uint8_t *mask = onbc.d;
        if (!rc && bc && !bc->onbc && bc->nlabels > 0) {
            if (dalloc(ctx, (void **)&lmask, S->ndof) != cudaSuccess) rc = FFGPU_ENOMEM;
            if (!rc) rc = space_bc_mask_device(S, bc->nlabels, bc->labels, bc->comp_mask, lmask);
            mask = lmask;
        }
        BoundaryTerms bt;
        double *fint = nullptr;
        if (!rc) rc = source_prepare(S, v, geo, &fint);
        if (!rc) rc = boundary_prepare(S, v, true, false, bt);
        if (!rc) {
            void (*k)(int, const int32_t *, const int32_t *, const uint8_t *, const double *,
                      const double *, const double *, double, double, double, const uint8_t *,
                      const double *, double, double *, const int32_t *, const int32_t *,
                      const double *) = nullptr;
            if (S->dim == 2 && S->fe == FFGPU_FE_P1) k = rhs_kernel<2, 1>;
            if (S->dim == 3 && S->fe == FFGPU_FE_P1) k = rhs_kernel<3, 1>;
            if (S->dim == 2 && S->fe == FFGPU_FE_P2) k = rhs_kernel<2, 2>;
            if (S->dim == 3 && S->fe == FFGPU_FE_P2) k = rhs_kernel<3, 2>;
            if (S->dim == 3 && S->fe == FFGPU_FE_P2VEC3) k = rhs_kernel<3, 3>;
            k<<<grid_for((int64_t)S->ndof, 256), 256, 0, s>>>(
                S->nnodes, S->inc_ptr, S->inc_elem, S->inc_loc, geo, fP0.d, fint, v->f_const[0],
                v->f_const[1], v->f_const[2], mask, gv.d, bc ? bc->tgv : 0.0, rh.d, bt.ptr, bt.list, bt.rhs);
            rc = launch_check(ctx, "rhs_kernel");
        }
        boundary_release(S, bt);
        dfree(ctx, fint);
        if (!rc) rc = rh.finish();
        if (lmask) dfree(ctx, lmask);
    }
    dfree(ctx, geo);
    cudaStreamSynchronize(s);
    return rc;
}

int ffgpu_matrix_from_csr(ffgpu_ctx *ctx, int n, int64_t nnz, const int32_t *rowptr,
                          const int32_t *col, const double *val, ffgpu_matrix **out) {
    FFGPU_CHECK(ctx && out && rowptr && col && val && n > 0 && nnz > 0, FFGPU_EINVAL,
                "ffgpu_matrix_from_csr: bad argument");
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    ffgpu_matrix *M = new ffgpu_matrix();
    memset(M, 0, sizeof(*M));
    M->ctx = ctx; M->bs = 1; M->nb = n; M->n = n; M->nnzb = nnz; M->nnz = nnz; M->ntgv = -1;
    if (dalloc(ctx, (void **)&M->browptr, sizeof(int32_t) * (n + 1)) ||
        dalloc(ctx, (void **)&M->bcol, sizeof(int32_t) * nnz) ||
        dalloc(ctx, (void **)&M->diagpos, sizeof(int32_t) * n) ||
        dalloc(ctx, (void **)&M->val, sizeof(double) * nnz)) {
        set_error("ffgpu_matrix_from_csr: device allocation failed");
        ffgpu_matrix_destroy(M);
        return FFGPU_ENOMEM;
    }
    cudaMemcpyAsync(M->browptr, rowptr, sizeof(int32_t) * (n + 1), cudaMemcpyDefault, s);
    cudaMemcpyAsync(M->bcol, col, sizeof(int32_t) * nnz, cudaMemcpyDefault, s);
    cudaMemcpyAsync(M->val, val, sizeof(double) * nnz, cudaMemcpyDefault, s);
    {
        int32_t first = -1, last = -1;
        cudaMemcpyAsync(&first, M->browptr, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&last, M->browptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        FFGPU_CUDA(cudaStreamSynchronize(s));
        if (first != 0 || last != nnz) {
            set_error("rowptr inconsistent with nnz");
            ffgpu_matrix_destroy(M);
            return FFGPU_EINVAL;
        }
        int32_t *deg = nullptr;
        FFGPU_CUDA(dalloc(ctx, (void **)&deg, sizeof(int32_t) * n));
        row_degree_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, M->browptr, deg);
        int rc = launch_check(ctx, "row_degree");
        if (!rc) rc = device_max_i32(ctx, deg, n, &M->max_deg);
        if (!rc && dalloc(ctx, (void **)&M->rowperm, sizeof(int32_t) * n)) { set_error("allocation failed"); rc = FFGPU_ENOMEM; }
        if (!rc) rc = device_order_by_key_desc(ctx, deg, n, M->max_deg, M->rowperm);
        dfree(ctx, deg);
        if (rc) { ffgpu_matrix_destroy(M); return rc; }
    }
    diagpos_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, M->browptr, M->bcol, M->diagpos);
    FFGPU_TRY(launch_check(ctx, "diagpos"));
    FFGPU_CUDA(cudaStreamSynchronize(s));
    *out = M;
    return FFGPU_OK;
}

int ffgpu_matrix_destroy(ffgpu_matrix *M) {
    if (!M) return FFGPU_OK;
    cudaStreamSynchronize(M->ctx->stream);
    if (M->cg_exec) cudaGraphExecDestroy(M->cg_exec);
    direct_release(M);
    dfree(M->ctx, M->browptr); dfree(M->ctx, M->bcol); dfree(M->ctx, M->diagpos); dfree(M->ctx, M->rowperm); dfree(M->ctx, M->val);
    dfree(M->ctx, M->geo); dfree(M->ctx, M->bcmask);
    dfree(M->ctx, M->diag_inv); dfree(M->ctx, M->wcl); dfree(M->ctx, M->vec); dfree(M->ctx, M->val_t);
    dfree(M->ctx, M->val32); dfree(M->ctx, M->valx); dfree(M->ctx, M->valx_t); dfree(M->ctx, M->hx); dfree(M->ctx, M->ks);
    sell_release(M);
    delete M;
    return FFGPU_OK;
}

int ffgpu_matrix_info(const ffgpu_matrix *M, int *n, int64_t *nnz, int *bs) {
    FFGPU_CHECK(M, FFGPU_EINVAL, "ffgpu_matrix_info: NULL matrix");
    if (n) *n = M->n;
    if (nnz) *nnz = M->nnz;
    if (bs) *bs = M->bs;
    return FFGPU_OK;
}

int ffgpu_matrix_csr(const ffgpu_matrix *M, int32_t *rowptr, int32_t *col, double *val) {
    FFGPU_CHECK(M && rowptr && col && val, FFGPU_EINVAL, "ffgpu_matrix_csr: NULL argument");
    ffgpu_ctx *ctx = M->ctx;
    cudaStream_t s = ctx->stream;
    FFGPU_CUDA(cudaSetDevice(ctx->device));
    DevOut<int32_t> rp(rowptr, M->n + 1, ctx, false);
    DevOut<int32_t> cl(col, M->nnz, ctx, false);
    DevOut<double> vl(val, M->nnz, ctx, false);
    FFGPU_TRY(rp.err); FFGPU_TRY(cl.err); FFGPU_TRY(vl.err);
    export_csr_kernel<<<grid_for(M->nb, 128), 128, 0, s>>>(M->nb, M->bs, M->browptr, M->bcol, M->val,
                                                            rp.d, cl.d, vl.d);
    FFGPU_TRY(launch_check(ctx, "export_csr"));
    FFGPU_TRY(rp.finish()); FFGPU_TRY(cl.finish()); FFGPU_TRY(vl.finish());
    FFGPU_CUDA(cudaStreamSynchronize(s));
    return FFGPU_OK;
}

}  // extern "C"
