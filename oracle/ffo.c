/*
 * ffo.c -- CPU oracle for the FreeFEM assemble-and-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the algorithm FreeFEM 4.15
 * runs for `matrix A = a(Vh,Vh,solver=CG)`, `real[int] b = a(0,Vh)` and `u[] = A^-1*b`.
 * It is the checker of the CUDA path (tests, smoke(), bench cpu_baseline) and is never
 * linked into, or called by, the product library.
 *
 * Restated reference pieces (file:line within FreeFEM-sources):
 *   HashMatrix insert-or-find, hash (i+j*n)%nhash ......... src/femlib/HashMatrix.hpp:157-183,322-362
 *   element matrix += into the hash matrix (full type) .... src/femlib/HashMatrix.cpp:1295-1332
 *   COO SpMV in insertion order, transpose = swap i/j ..... src/femlib/HashMatrix.cpp:1087-1154
 *   SetBC with tgv > 0 (diag := tgv, row kept) ............ src/femlib/HashMatrix.cpp:1195-1238
 *   gettgv (largest diagonal, count, ratio 1e6) ........... src/femlib/HashMatrix.cpp:1341-1371
 *   Jacobi preconditioner, x0 = b/tgv on tgv rows ......... src/femlib/VirtualSolverCG.hpp:27-99
 *   ConjugueGradient ...................................... src/femlib/CG.cpp:196-265
 *   fgmres (right preconditioned, MGS, Givens) ............ src/femlib/CG.cpp:348-517
 *   Element_Op full (quadrature loop, c*coef*w_i*w_j) ..... src/fflib/problem.cpp:6063-6160 / 6337-6437
 *   Element_rhs (coef*c*w_i) .............................. src/fflib/problem.cpp:7839-7911
 *   P1 2D gradients Triangle::H ........................... src/femlib/fem.hpp:321-324
 *   Tet::Gradlambda, tet volume ........................... src/femlib/Mesh3dn.hpp:70,126-136
 *   P2 3D basis and gradients ............................. src/femlib/P012_3d.cpp:199-277
 *   P2 2D basis (edge i opposite vertex i) ................ src/femlib/FESpace.cpp:1219-1300
 *   3D node numbering by first encounter .................. src/femlib/GenericMesh.hpp:1711-1954
 *   quadrature rules T_2, T_5, Tet_2, Tet_5 ............... src/femlib/QuadratureFormular.cpp:151-188,712-743
 *   Sortij / CSR (row then column order) .................. src/femlib/HashMatrix.cpp:671-682,870-876
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ hash matrix */
typedef struct {
    int n;
    int64_t nnz, nnzmax, nhash;
    int *i, *j;
    double *a;
    int64_t *next, *head;
} ffo_hm;

static void hm_grow(ffo_hm *A) {
    int64_t nm = A->nnzmax * 2 + 16;
    A->i = (int *)realloc(A->i, nm * sizeof(int));
    A->j = (int *)realloc(A->j, nm * sizeof(int));
    A->a = (double *)realloc(A->a, nm * sizeof(double));
    A->next = (int64_t *)realloc(A->next, nm * sizeof(int64_t));
    A->nnzmax = nm;
    /* rehash with a larger table (HashMatrix::Increaze / ReHash) */
    int64_t nh = A->n * (int64_t)(nm / A->n < 50 ? (nm / A->n > 1 ? nm / A->n : 1) : 50);
    if (nh > A->nhash) {
        free(A->head);
        A->nhash = nh;
        A->head = (int64_t *)malloc(nh * sizeof(int64_t));
        for (int64_t h = 0; h < nh; ++h) A->head[h] = -1;
        for (int64_t k = 0; k < A->nnz; ++k) {
            int64_t h = ((int64_t)A->i[k] + (int64_t)A->j[k] * A->n) % A->nhash;
            A->next[k] = A->head[h];
            A->head[h] = k;
        }
    }
}

void *ffo_hm_new(int n) {
    ffo_hm *A = (ffo_hm *)calloc(1, sizeof(ffo_hm));
    A->n = n;
    A->nnzmax = 0;
    A->nhash = n > 0 ? n : 1;
    A->head = (int64_t *)malloc(A->nhash * sizeof(int64_t));
    for (int64_t h = 0; h < A->nhash; ++h) A->head[h] = -1;
    hm_grow(A);
    return A;
}

void ffo_hm_free(void *p) {
    ffo_hm *A = (ffo_hm *)p;
    if (!A) return;
    free(A->i); free(A->j); free(A->a); free(A->next); free(A->head); free(A);
}

static double *hm_find(const ffo_hm *A, int ii, int jj) {
    int64_t h = ((int64_t)ii + (int64_t)jj * A->n) % A->nhash;
    for (int64_t k = A->head[h]; k != -1; k = A->next[k])
        if (A->i[k] == ii && A->j[k] == jj) return A->a + k;
    return 0;
}

/* insert-or-find: a new entry is appended (insertion order defines the COO order) */
static double *hm_npij(ffo_hm *A, int ii, int jj) {
    double *p = hm_find(A, ii, jj);
    if (p) return p;
    if (A->nnz == A->nnzmax) hm_grow(A);
    int64_t h = ((int64_t)ii + (int64_t)jj * A->n) % A->nhash;
    int64_t k = A->nnz++;
    A->i[k] = ii; A->j[k] = jj; A->a[k] = 0.0;
    A->next[k] = A->head[h];
    A->head[h] = k;
    return A->a + k;
}

int64_t ffo_hm_nnz(const void *p) { return ((const ffo_hm *)p)->nnz; }

void ffo_hm_coo(const void *p, int *I, int *J, double *V) {
    const ffo_hm *A = (const ffo_hm *)p;
    memcpy(I, A->i, A->nnz * sizeof(int));
    memcpy(J, A->j, A->nnz * sizeof(int));
    memcpy(V, A->a, A->nnz * sizeof(double));
}

/* Sortij + Buildp: row-major sorted CSR (counting sort by row, then by column) */
void ffo_hm_csr(const void *p, int *rowptr, int *col, double *val) {
    const ffo_hm *A = (const ffo_hm *)p;
    int n = A->n;
    int64_t nnz = A->nnz;
    int64_t *cnt = (int64_t *)calloc(n + 1, sizeof(int64_t));
    for (int64_t k = 0; k < nnz; ++k) cnt[A->i[k] + 1]++;
    for (int r = 0; r < n; ++r) cnt[r + 1] += cnt[r];
    int64_t *pos = (int64_t *)malloc((n + 1) * sizeof(int64_t));
    memcpy(pos, cnt, (n + 1) * sizeof(int64_t));
    for (int64_t k = 0; k < nnz; ++k) {
        int64_t q = pos[A->i[k]]++;
        col[q] = A->j[k];
        val[q] = A->a[k];
    }
    for (int r = 0; r < n; ++r) {
        rowptr[r] = (int)cnt[r];
        /* insertion sort of the row by column (rows are short) */
        for (int64_t a = cnt[r] + 1; a < cnt[r + 1]; ++a) {
            int c = col[a]; double v = val[a]; int64_t b = a - 1;
            while (b >= cnt[r] && col[b] > c) { col[b + 1] = col[b]; val[b + 1] = val[b]; --b; }
            col[b + 1] = c; val[b + 1] = v;
        }
    }
    rowptr[n] = (int)nnz;
    free(cnt); free(pos);
}

/* ------------------------------------------------------------------ quadrature */
/* rule ids: 2 = T_2 (qf2pT), 5 = T_5 (qf5pT, 2D default); 102 = Tet_2, 105 = Tet_5 (3D default).
 * Points are barycentric (lambda_1, lambda_2[, lambda_3]); weights are relative to the
 * element measure (coef = |K| * w_q). */
static int quad_rule(int id, double *P, double *W) {
    if (id == 2) {
        const double p[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};
        for (int q = 0; q < 3; ++q) { P[2 * q] = p[q][0]; P[2 * q + 1] = p[q][1]; W[q] = 1. / 3.; }
        return 3;
    }
    if (id == 5) {
        const double s15 = 3.87298334620741688517926539978;
        const double t = 1. / 3., A = 0.225;
        const double r = (6 - s15) / 21, s = (9 + 2 * s15) / 21, B = (155 - s15) / 1200;
        const double u = (6 + s15) / 21, v = (9 - 2 * s15) / 21, C = (155 + s15) / 1200;
        const double p[7][2] = {{t, t}, {r, r}, {r, s}, {s, r}, {u, u}, {u, v}, {v, u}};
        const double w[7] = {A, B, B, B, C, C, C};
        for (int q = 0; q < 7; ++q) { P[2 * q] = p[q][0]; P[2 * q + 1] = p[q][1]; W[q] = w[q]; }
        return 7;
    }
    if (id == 102) {
        const double a = 0.58541019662496845446137605030968, b = 0.138196601125010515179541316563436;
        const double p[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
        for (int q = 0; q < 4; ++q) { for (int d = 0; d < 3; ++d) P[3 * q + d] = p[q][d]; W[q] = 0.25; }
        return 4;
    }
    if (id == 105) {
        /* 14-point degree-5 rule on the tetrahedron (three orbits: 4 + 4 + 6 points) */
        const double a1 = 0.7217942490673263207930282587889082, b1 = 0.0927352503108912264023239137370306;
        const double a2 = 0.067342242210098170607962798709629, b2 = 0.310885919263300609797345733763457;
        const double a3 = 0.454496295874350350508119473720660, b3 = 0.045503704125649649491880526279339;
        const double w1 = 0.0122488405193936582572850342477212 * 6.;
        const double w2 = 0.0187813209530026417998642753888810 * 6.;
        const double w3 = 7.09100346284691107301157135337624E-3 * 6.;
        const double p[14][3] = {{a1, b1, b1}, {b1, a1, b1}, {b1, b1, a1}, {b1, b1, b1},
                                 {a2, b2, b2}, {b2, a2, b2}, {b2, b2, a2}, {b2, b2, b2},
                                 {a3, a3, b3}, {a3, b3, a3}, {b3, a3, a3}, {b3, b3, a3},
                                 {b3, a3, b3}, {a3, b3, b3}};
        const double w[14] = {w1, w1, w1, w1, w2, w2, w2, w2, w3, w3, w3, w3, w3, w3};
        for (int q = 0; q < 14; ++q) { for (int d = 0; d < 3; ++d) P[3 * q + d] = p[q][d]; W[q] = w[q]; }
        return 14;
    }
    return 0;
}

/* the points (reference coordinates, dim per point) and weights of rule `id`; returns nq */
int ffo_quad_points(int id, double *P, double *W) { return quad_rule(id, P, W); }

/* ------------------------------------------------------------------ basis */
static const int tet_edge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
static const int tri_edge[3][2] = {{1, 2}, {2, 0}, {0, 1}};

/* geometry: barycentric gradients G[d+1][3] and measure */
static double geom(int dim, const double *X, const int *v, double G[4][3]) {
    if (dim == 2) {
        const double *A = X + 2 * v[0], *B = X + 2 * v[1], *C = X + 2 * v[2];
        double area = ((B[0] - A[0]) * (C[1] - A[1]) - (B[1] - A[1]) * (C[0] - A[0])) * 0.5;
        const double *P[3] = {A, B, C};
        for (int i = 0; i < 3; ++i) {
            const double *p1 = P[(i + 1) % 3], *p2 = P[(i + 2) % 3];
            double ex = p2[0] - p1[0], ey = p2[1] - p1[1];          /* Edge(i) */
            G[i][0] = -ey / (2 * area); G[i][1] = ex / (2 * area); G[i][2] = 0;
        }
        return area;
    } else {
        const double *A = X + 3 * v[0], *B = X + 3 * v[1], *C = X + 3 * v[2], *D = X + 3 * v[3];
        double V1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
        double V2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        double V3[3] = {D[0] - A[0], D[1] - A[1], D[2] - A[2]};
        double c23[3] = {V2[1] * V3[2] - V2[2] * V3[1], V2[2] * V3[0] - V2[0] * V3[2], V2[0] * V3[1] - V2[1] * V3[0]};
        double c31[3] = {V3[1] * V1[2] - V3[2] * V1[1], V3[2] * V1[0] - V3[0] * V1[2], V3[0] * V1[1] - V3[1] * V1[0]};
        double c12[3] = {V1[1] * V2[2] - V1[2] * V2[1], V1[2] * V2[0] - V1[0] * V2[2], V1[0] * V2[1] - V1[1] * V2[0]};
        double vol = (V1[0] * c23[0] + V1[1] * c23[1] + V1[2] * c23[2]) / 6.;
        double det1 = 1. / (6. * vol);
        for (int d = 0; d < 3; ++d) {
            G[1][d] = c23[d] * det1; G[2][d] = c31[d] * det1; G[3][d] = c12[d] * det1;
            G[0][d] = -G[1][d] - G[2][d] - G[3][d];
        }
        return vol;
    }
}

/* scalar basis values and gradients at barycentric point l[] */
static int basis(int dim, int order, const double *l, double G[4][3], double *w, double dw[][3]) {
    int nv = dim + 1;
    if (order == 1) {
        for (int i = 0; i < nv; ++i) { w[i] = l[i]; for (int d = 0; d < 3; ++d) dw[i][d] = G[i][d]; }
        return nv;
    }
    int k = 0;
    for (int i = 0; i < nv; ++i, ++k) {
        w[k] = l[i] * (2 * l[i] - 1.);
        for (int d = 0; d < 3; ++d) dw[k][d] = G[i][d] * (4 * l[i] - 1);
    }
    int ne = dim == 2 ? 3 : 6;
    for (int e = 0; e < ne; ++e, ++k) {
        int i0 = dim == 2 ? tri_edge[e][0] : tet_edge[e][0];
        int i1 = dim == 2 ? tri_edge[e][1] : tet_edge[e][1];
        w[k] = 4. * l[i0] * l[i1];
        for (int d = 0; d < 3; ++d) dw[k][d] = 4 * (G[i1][d] * l[i0] + G[i0][d] * l[i1]);
    }
    return k;
}

/* ------------------------------------------------------------------ assembly
 * form: 0 = sum_d coef*dx_d(u)dx_d(v) (+ mass_c0*u*v)      (P1/P2 scalar)
 *       1 = linear elasticity lambda div u div v + 2 mu eps(u):eps(v)  (P2 vector, 3D)
 * fe:   1 = P1, 2 = P2 scalar, 3 = [P2,P2,P2] (local DOF = comp*10 + node)
 * coef: P0 coefficient per element or NULL (then c0 = 1 multiplies the stiffness)
 * kqp:  or the stiffness coefficient at the rule's points, kqp[k*nq + q] (replaces coef)
 * mass: constant coefficient of u*v (0 = none), or mqp: its values at the rule's points,
 *       mqp[k*nq + q] (a coefficient that is any function of the point, as Element_Op takes it)
 */
typedef struct {
    int dim, nt, ndofK, fe, form, quad;
    const double *X;
    const int *elems, *dof;
    const double *coef;
    double E, nu, mass;
    const double *mqp;
    const double *kqp;   /* stiffness coefficient at the rule's points (replaces coef), or NULL */
    const double *lame;  /* elasticity: per-element (lambda, mu) (replaces E, nu), or NULL */
} ffo_form;

static void elem_matrix(const ffo_form *F, int k, double *M /* ndofK^2, row = test */) {
    int dim = F->dim, nv = dim + 1;
    double G[4][3] = {{0}};
    const int *v = F->elems + (int64_t)k * nv;
    double mes = geom(dim, F->X, v, G);
    double P[14 * 3], W[14];
    int nq = quad_rule(F->quad, P, W);
    int nd = F->ndofK;
    memset(M, 0, sizeof(double) * nd * nd);
    int order = F->fe == 1 ? 1 : 2;
    double w[10], dw[10][3];
    for (int q = 0; q < nq; ++q) {
        double l[4];
        if (dim == 2) { l[1] = P[2 * q]; l[2] = P[2 * q + 1]; l[0] = 1. - l[1] - l[2]; }
        else { l[1] = P[3 * q]; l[2] = P[3 * q + 1]; l[3] = P[3 * q + 2]; l[0] = 1. - (l[1] + l[2] + l[3]); }
        double coef = mes * W[q];
        int nb = basis(dim, order, l, G, w, dw);
        if (F->form == 0) {
            double c = F->kqp ? F->kqp[(int64_t)k * nq + q] : (F->coef ? F->coef[k] : 1.0);
            /* one term per derivative, as the varf lists them: dx(u)*dx(v) + dy(u)*dy(v) [+ dz] */
            for (int d = 0; d < dim; ++d) {
                double ccc = c * coef;
                for (int i = 0; i < nb; ++i)
                    for (int j = 0; j < nb; ++j) M[i * nd + j] += ccc * dw[i][d] * dw[j][d];
            }
            if (F->mass != 0.0 || F->mqp) {
                double ccc = (F->mqp ? F->mqp[(int64_t)k * nq + q] : F->mass) * coef;
                for (int i = 0; i < nb; ++i)
                    for (int j = 0; j < nb; ++j) M[i * nd + j] += ccc * w[i] * w[j];
            }
        } else {
            /* elasticity terms ((trial comp, d), (test comp, d')) with coefficients:
             *   lambda * dc'(u_c') dc(v_c)                     for all c, c'
             *   2mu * dc(u_c) dc(v_c)                          for all c
             *   2mu/2 * (dq u_p + dp u_q)(dq v_p + dp v_q)     for p < q     */
            double E = F->E, nu = F->nu;
            double mu = E / (2 * (1 + nu)), lam = E * nu / ((1 + nu) * (1 - 2 * nu));
            if (F->lame) { lam = F->lame[2 * (int64_t)k]; mu = F->lame[2 * (int64_t)k + 1]; }
            double s2 = sqrt(2.), is2 = 1. / s2;
            double half = 2. * mu * is2 * is2;
            for (int ci = 0; ci < 3; ++ci)      /* test component, derivative ci */
                for (int cj = 0; cj < 3; ++cj) {/* trial component, derivative cj */
                    double ccc = lam * coef;
                    for (int i = 0; i < 10; ++i)
                        for (int j = 0; j < 10; ++j)
                            M[(ci * 10 + i) * nd + cj * 10 + j] += ccc * dw[i][ci] * dw[j][cj];
                }
            for (int c = 0; c < 3; ++c) {
                double ccc = 2. * mu * coef;
                for (int i = 0; i < 10; ++i)
                    for (int j = 0; j < 10; ++j)
                        M[(c * 10 + i) * nd + c * 10 + j] += ccc * dw[i][c] * dw[j][c];
            }
            const int pr[3][2] = {{1, 2}, {0, 2}, {0, 1}};
            for (int s = 0; s < 3; ++s) {
                int p = pr[s][0], qq = pr[s][1];
                /* strain component (dq u_p + dp u_q): (comp p, deriv q) and (comp q, deriv p) */
                int tc[2] = {p, qq}, td[2] = {qq, p};
                double ccc = half * coef;
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int i = 0; i < 10; ++i)
                            for (int j = 0; j < 10; ++j)
                                M[(tc[a] * 10 + i) * nd + tc[b] * 10 + j] += ccc * dw[i][td[a]] * dw[j][td[b]];
            }
        }
    }
}

/* assemble the bilinear form into the hash matrix, element by element (insertion order) */
int ffo_assemble(void *hm, int dim, int nt, const double *X, const int *elems, int ndofK,
                 const int *dof, int fe, int form, int quad, const double *coef, double E,
                 double nu, double mass, const double *mqp, const double *kqp, const double *lame) {
    ffo_hm *A = (ffo_hm *)hm;
    ffo_form F = {dim, nt, ndofK, fe, form, quad, X, elems, dof, coef, E, nu, mass, mqp, kqp, lame};
    double *M = (double *)malloc(sizeof(double) * ndofK * ndofK);
    for (int k = 0; k < nt; ++k) {
        elem_matrix(&F, k, M);
        const int *d = dof + (int64_t)k * ndofK;
        for (int il = 0; il < ndofK; ++il)
            for (int jl = 0; jl < ndofK; ++jl) *hm_npij(A, d[il], d[jl]) += M[il * ndofK + jl];
    }
    free(M);
    return 0;
}

/* element matrices only (for the per-element sensitivity of the adjoint) */
void ffo_element_matrix(int dim, const double *X, const int *elems, int k, int ndofK, int fe,
                        int form, int quad, const double *coef, double E, double nu,
                        double mass, double *M) {
    ffo_form F = {dim, 0, ndofK, fe, form, quad, X, elems, 0, coef, E, nu, mass, 0, 0, 0};
    elem_matrix(&F, k, M);
}

/* linear form: b[dof] += |K| w_q f_c phi_i  (f P0 per element and component, or constant) */
/* fqp (or NULL): the source at the rule's points, fqp[(k*nq + q)*ncomp + c], in place of
 * fP0 / fconst -- a source that is any function of the coordinates, as Element_rhs takes it
 * (problem.cpp:7839-7911, 7917-7990) */
int ffo_rhs(double *b, int dim, int nt, const double *X, const int *elems, int ndofK,
            const int *dof, int fe, int quad, const double *fP0, int ncomp, const double *fconst,
            const double *fqp) {
    int nv = dim + 1, order = fe == 1 ? 1 : 2;
    double P[14 * 3], W[14];
    int nq = quad_rule(quad, P, W);
    for (int k = 0; k < nt; ++k) {
        double G[4][3] = {{0}};
        const int *v = elems + (int64_t)k * nv;
        double mes = geom(dim, X, v, G);
        const int *d = dof + (int64_t)k * ndofK;
        for (int q = 0; q < nq; ++q) {
            double l[4], w[10], dw[10][3];
            if (dim == 2) { l[1] = P[2 * q]; l[2] = P[2 * q + 1]; l[0] = 1. - l[1] - l[2]; }
            else { l[1] = P[3 * q]; l[2] = P[3 * q + 1]; l[3] = P[3 * q + 2]; l[0] = 1. - (l[1] + l[2] + l[3]); }
            double coef = mes * W[q];
            int nb = basis(dim, order, l, G, w, dw);
            for (int c = 0; c < ncomp; ++c) {
                double fc = fqp ? fqp[((int64_t)k * nq + q) * ncomp + c]
                                : (fP0 ? fP0[(int64_t)k * ncomp + c] : fconst[c]);
                if (fc == 0.0 && !fP0 && !fqp) continue;
                for (int i = 0; i < nb; ++i) b[d[c * nb + i]] += coef * fc * w[i];
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ boundary terms
 * One varf term on the boundary elements e whose label is one of labels[0..nlabels) (every
 * boundary element when nlabels == 0), integrated on the edge/face bel_face[e] (the one
 * opposite that local vertex) of the adjacent element bel_elem[e], in boundary-element order
 * (the bedges / be(k) loops of AssembleBilinearForm and AssembleLinearForm,
 * problem.cpp:1011-1019, 10722-10735):
 *   hm != NULL: element matrix M(i,j) = sum_q (c coef_q) w_i w_j over every local i, j of the
 *               element, per component for [P2,P2,P2], then A += M (Element_Op on an edge,
 *               problem.cpp:6222-6262; on a face, problem.cpp:6516-6560);
 *   b  != NULL: b(i) += coef_q g_c w_i for component c (Element_rhs on an edge,
 *               problem.cpp:8612-8683; on a face, problem.cpp:8517-8580).
 * 2D: 3-point Gauss-Legendre on the edge (QF_GaussLegendre3, QuadratureFormular.cpp:319-343),
 *     coef = |E| a_q with E = Edge(ie), point PA s + PB (1 - s) where PA, PB are the reference
 *     vertices VerticesOfTriangularEdge[ie] (fem.hpp:95,112).
 * 3D: the 7-point T_5 rule on the face, coef = 0.5 |N| a_q with N = (P_f0 P_f2) x (P_f0 P_f1),
 *     point KHat[f0] (1-x-y) + KHat[f1] x + KHat[f2] y, f = nvfaceTet[ie] (GenericMesh.hpp:272,
 *     Mesh3dn.hpp:76, Mesh3dn.cpp:72).
 * c (Robin coefficient) and g (source): per boundary element (nbe, resp. nbe*ncomp) or NULL,
 * then the constants cconst / gconst[c]. */
static const int tet_face[4][3] = {{3, 2, 1}, {0, 2, 3}, {3, 1, 0}, {0, 1, 2}};

int ffo_bterm(void *hm, double *b, int dim, const double *X, const int *elems, int ndofK,
              const int *dof, int fe, int nbe, const int *bel_elem, const int *bel_face,
              const int *blabel, int nlabels, const int *labels, const double *cP, double cconst,
              const double *gP, int ncomp, const double *gconst) {
    ffo_hm *A = (ffo_hm *)hm;
    const int nv = dim + 1, order = fe == 1 ? 1 : 2, ncp = fe == 3 ? 3 : 1;
    double P[14 * 3], W[14];
    int nq;
    if (dim == 2) {
        const double g1 = (1 - sqrt(3. / 5.)) / 2;
        P[0] = 0.5; W[0] = 8. / 18.;
        P[1] = g1; W[1] = 5. / 18.;
        P[2] = 1 - g1; W[2] = 5. / 18.;
        nq = 3;
    } else {
        nq = quad_rule(5, P, W);
    }
    const double hat2[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    const double hat3[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double *M = hm ? (double *)malloc(sizeof(double) * ndofK * ndofK) : NULL;
    for (int e = 0; e < nbe; ++e) {
        if (nlabels > 0) {
            int hit = 0;
            for (int k = 0; k < nlabels; ++k) hit |= blabel[e] == labels[k];
            if (!hit) continue;
        }
        const int k = bel_elem[e], ie = bel_face[e];
        const int *v = elems + (int64_t)k * nv;
        const int *d = dof + (int64_t)k * ndofK;
        double G[4][3] = {{0}};
        if (M) memset(M, 0, sizeof(double) * ndofK * ndofK);
        for (int q = 0; q < nq; ++q) {
            double l[4], coef;
            if (dim == 2) {
                const double *p1 = X + 2 * v[tri_edge[ie][0]], *p2 = X + 2 * v[tri_edge[ie][1]];
                const double ex = p2[0] - p1[0], ey = p2[1] - p1[1];
                const double le = sqrt(ex * ex + ey * ey);
                coef = le * W[q];
                const double sa = P[q], sb = 1 - sa;
                const double *PA = hat2[tri_edge[ie][0]], *PB = hat2[tri_edge[ie][1]];
                const double x = PA[0] * sa + PB[0] * sb, y = PA[1] * sa + PB[1] * sb;
                l[1] = x; l[2] = y; l[0] = 1 - x - y;
            } else {
                const int *f = tet_face[ie];
                const double *a = X + 3 * v[f[0]], *p1 = X + 3 * v[f[1]], *p2 = X + 3 * v[f[2]];
                const double u[3] = {p2[0] - a[0], p2[1] - a[1], p2[2] - a[2]};
                const double w[3] = {p1[0] - a[0], p1[1] - a[1], p1[2] - a[2]};
                const double N[3] = {u[1] * w[2] - u[2] * w[1], w[0] * u[2] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
                const double le = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
                coef = le * W[q] * 0.5;
                const double x = P[2 * q], y = P[2 * q + 1], s = 1 - x - y;
                double pt[3];
                for (int c = 0; c < 3; ++c) pt[c] = hat3[f[0]][c] * s + hat3[f[1]][c] * x + hat3[f[2]][c] * y;
                l[1] = pt[0]; l[2] = pt[1]; l[3] = pt[2]; l[0] = 1. - (pt[0] + pt[1] + pt[2]);
            }
            double w[10], dw[10][3];
            const int nb = basis(dim, order, l, G, w, dw);
            if (M) {
                const double c = cP ? cP[e] : cconst;
                for (int cp = 0; cp < ncp; ++cp) {
                    const double ccc = c * coef;
                    for (int i = 0; i < nb; ++i)
                        for (int j = 0; j < nb; ++j) M[(cp * nb + i) * ndofK + cp * nb + j] += ccc * w[i] * w[j];
                }
            }
            if (b)
                for (int i = 0; i < nb; ++i)
                    for (int c = 0; c < ncomp; ++c) {
                        const double gc = gP ? gP[(int64_t)e * ncomp + c] : gconst[c];
                        if (gc == 0.0 && !gP) continue;
                        b[d[c * nb + i]] += coef * gc * w[i];
                    }
        }
        if (M)
            for (int il = 0; il < ndofK; ++il)
                for (int jl = 0; jl < ndofK; ++jl) *hm_npij(A, d[il], d[jl]) += M[il * ndofK + jl];
    }
    free(M);
    (void)nv;
    return 0;
}

/* SetBC (HashMatrix.cpp:1195-1238) with the rhs of AssembleBC (problem.cpp:9937,10020):
 *   tgv > 0: diagonal := tgv on marked rows, b_i = tgv g_i;
 *   tgv < 0: b_i = g_i; marked rows get diagonal 1 (0 if tgv <= -10) and zero off-diagonals
 *            (rows kept for -3/-30); for -2/-20/-3/-30 the marked columns are zeroed too,
 *            the diagonal included for -20/-30. */
void ffo_setbc(void *hm, double *b, const char *onbc, const double *g, double tgv) {
    ffo_hm *A = (ffo_hm *)hm;
    for (int i = 0; i < A->n; ++i)
        if (onbc[i]) {
            if (tgv > 0) *hm_npij(A, i, i) = tgv;
            else hm_npij(A, i, i);
            if (b) b[i] = (tgv > 0 ? tgv : 1.0) * (g ? g[i] : 0.0);
        }
    if (tgv >= 0) return;
    int keep_row = fabs(tgv + 3.0) < 1e-10 || fabs(tgv + 30.0) < 1e-10;
    int zero_col = fabs(tgv + 2.0) < 1e-10 || fabs(tgv + 20.0) < 1e-10 || keep_row;
    for (int64_t k = 0; k < A->nnz; ++k) {
        int ii = A->i[k], jj = A->j[k];
        if (onbc[ii]) {
            if (jj == ii) A->a[k] = tgv < -9.0 ? 0.0 : 1.0;
            else if (!keep_row) A->a[k] = 0.0;
        }
    }
    if (zero_col)
        for (int64_t k = 0; k < A->nnz; ++k) {
            int ii = A->i[k], jj = A->j[k];
            if (onbc[jj] && (ii != jj || tgv < -19.0)) A->a[k] = 0.0;
        }
}

/* ------------------------------------------------------------------ solvers */
static void spmv_add(const ffo_hm *A, const double *x, double *y, int trans) {
    const int *ii = trans ? A->j : A->i, *jj = trans ? A->i : A->j;
    for (int64_t k = 0; k < A->nnz; ++k) y[ii[k]] += A->a[k] * x[jj[k]];
}
static void matmul(const ffo_hm *A, const double *x, double *y, int trans) {
    memset(y, 0, sizeof(double) * A->n);
    spmv_add(A, x, y, trans);
}
static double dot(int n, const double *x, const double *y) {
    double s = 0; for (int i = 0; i < n; ++i) s += x[i] * y[i]; return s;
}

/* HMatVirtPrecon: diag1 = 1/A_ii (1 if |A_ii|^2 < 1e-60); tgv rows = diag equal to the
 * largest diagonal when it beats the second largest distinct diagonal by >= 1e6 */
static double *jacobi(const ffo_hm *A, char *wcl, int *ntgv) {
    int n = A->n;
    double *d = (double *)malloc(sizeof(double) * n);
    double ttgv = 0, max1 = 0; int nt = 0;
    for (int i = 0; i < n; ++i) {
        double *p = hm_find(A, i, i);
        d[i] = p ? *p : 0.0;
        if (p) {
            double a = *p;
            if (a > ttgv) { max1 = ttgv; ttgv = a; nt = 1; }
            else if (a == ttgv) ++nt;
            else if (a > max1) max1 = a;
        }
    }
    if (max1 * 1e6 > ttgv) { ttgv = 0; nt = 0; }
    if (ntgv) *ntgv = nt;
    double tgve = ttgv > 0 ? ttgv : 1e200;
    for (int i = 0; i < n; ++i) {
        if (wcl) wcl[i] = nt ? (d[i] == tgve) : 0;
        d[i] = (d[i] * d[i] < 1e-60) ? 1.0 : 1.0 / d[i];
    }
    return d;
}

/* Jacobi PCG of CG.cpp:196-265 with SolverCG::dosolver's x0 = b/tgv on tgv rows.
 * returns 1 converged, 2 converged at start, 0 not converged; *iters as nbitermax */
int ffo_cg(const void *hm, const double *b, double *x, double eps, int itmax, int trans,
           double tgv, int *iters, double *gcg_out) {
    const ffo_hm *A = (const ffo_hm *)hm;
    int n = A->n;
    char *wcl = (char *)malloc(n);
    int ntgv = 0;
    double *D = jacobi(A, wcl, &ntgv);
    if (ntgv) for (int i = 0; i < n; ++i) if (wcl[i]) x[i] = b[i] / tgv;
    if (itmax <= 0) itmax = n;
    double *G = (double *)malloc(sizeof(double) * n), *CG = (double *)malloc(sizeof(double) * n);
    double *H = (double *)malloc(sizeof(double) * n);
    matmul(A, x, G, trans);
    for (int i = 0; i < n; ++i) G[i] -= b[i];                 /* G = Ax - b */
    for (int i = 0; i < n; ++i) CG[i] = D[i] * G[i];
    double gCg = dot(n, G, CG), gCgp, eps2 = eps * eps;
    for (int i = 0; i < n; ++i) H[i] = -CG[i];
    if (eps > 0) eps2 *= gCg;
    int ret = 0, it = 0;
    if (gCg < 1e-30) { ret = 2; it = 0; }
    else
        for (int iter = 1; iter <= itmax; ++iter) {
            gCgp = gCg;
            matmul(A, H, CG, trans);                          /* AH shares CG */
            double rho = -dot(n, G, H) / dot(n, H, CG);
            for (int i = 0; i < n; ++i) x[i] += rho * H[i];
            for (int i = 0; i < n; ++i) G[i] += rho * CG[i];
            for (int i = 0; i < n; ++i) CG[i] = D[i] * G[i];
            gCg = dot(n, G, CG);
            double gamma = gCg / gCgp;
            for (int i = 0; i < n; ++i) H[i] = gamma * H[i] - CG[i];
            it = iter;
            if (gCg < eps2) { ret = 1; break; }
        }
    if (iters) *iters = it;
    if (gcg_out) { gcg_out[0] = gCg; gcg_out[1] = eps2; }
    free(G); free(CG); free(H); free(D); free(wcl);
    return ret;
}

/* fgmres of CG.cpp:348-517 (right Jacobi preconditioner, restart nbkrylov) */
int ffo_fgmres(const void *hm, const double *b, double *px, double eps, int nbitermx,
               int nbkrylov, int trans, double tgv, int *iters, double *relres_out) {
    const ffo_hm *A = (const ffo_hm *)hm;
    int n = A->n, m = nbkrylov;
    char *wcl = (char *)malloc(n);
    int ntgv = 0;
    double *D = jacobi(A, wcl, &ntgv);
    if (ntgv) for (int i = 0; i < n; ++i) if (wcl[i]) px[i] = b[i] / tgv;
    if (nbitermx <= 0) nbitermx = n;
    double *rot0 = (double *)malloc(sizeof(double) * (m + 2)), *rot1 = (double *)malloc(sizeof(double) * (m + 2));
    double *g = (double *)malloc(sizeof(double) * (m + 1)), *g1 = (double *)malloc(sizeof(double) * (m + 1));
    double *Hn = (double *)calloc((size_t)(m + 2) * (m + 1), sizeof(double));
#define HN(i, j) Hn[(size_t)(i) * (m + 1) + (j)]
    double *V = (double *)malloc(sizeof(double) * (size_t)n * (m + 1));
    double *Vp = (double *)malloc(sizeof(double) * (size_t)n * (m + 1));
    double *wi = (double *)malloc(sizeof(double) * n), *vi = (double *)malloc(sizeof(double) * n);
    double *ri = (double *)malloc(sizeof(double) * n), *x0 = (double *)malloc(sizeof(double) * n);
    double *uni = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) wi[i] = (ntgv && wcl[i]) ? 0.0 : b[i];
    double normb = sqrt(dot(n, wi, wi));
    memcpy(uni, px, sizeof(double) * n);
    int noconv = 1, iter = 0;
    double relres = 1e100;
    while (noconv) {
        memcpy(x0, uni, sizeof(double) * n);
        matmul(A, uni, ri, trans);
        for (int i = 0; i < n; ++i) ri[i] = -(ri[i] - b[i]);
        g[0] = sqrt(dot(n, ri, ri));
        if (normb < 1.e-20 || eps < 0) normb = 1.;
        for (int i = 0; i < n; ++i) V[i] = (1. / g[0]) * ri[i];
        int it;
        for (it = 0; it < m; it++, iter++) {
            double *Vit = V + (size_t)it * n, *Vpit = Vp + (size_t)it * n;
            for (int i = 0; i < n; ++i) vi[i] = D[i] * Vit[i];
            memcpy(Vpit, vi, sizeof(double) * n);
            matmul(A, vi, wi, trans);
            for (int i = 0; i <= it; i++) {
                double *Vi_ = V + (size_t)i * n;
                HN(i, it) = dot(n, wi, Vi_);
                double c = -HN(i, it);
                for (int r = 0; r < n; ++r) wi[r] += c * Vi_[r];
            }
            double aux = HN(it + 1, it) = sqrt(dot(n, wi, wi));
            double *Vn = V + (size_t)(it + 1) * n;
            for (int r = 0; r < n; ++r) Vn[r] = (1. / aux) * wi[r];
            for (int i = 0; i < it; i++) {
                double aa = rot0[i] * HN(i, it) + rot1[i] * HN(i + 1, it);
                double bb = -rot1[i] * HN(i, it) + rot0[i] * HN(i + 1, it);
                HN(i, it) = aa; HN(i + 1, it) = bb;
            }
            double sq = sqrt(HN(it, it) * HN(it, it) + HN(it + 1, it) * HN(it + 1, it));
            rot0[it] = HN(it, it) / sq;
            rot1[it] = HN(it + 1, it) / sq;
            HN(it, it) = rot0[it] * HN(it, it) + rot1[it] * HN(it + 1, it);
            HN(it + 1, it) = 0.;
            g[it + 1] = -rot1[it] * g[it];
            g[it] = rot0[it] * g[it];
            relres = fabs(g[it + 1]);
            if (relres / normb < fabs(eps)) { noconv = 0; break; }
            if (it > nbitermx) break;
        }
        if (it > m - 1) it = m - 1;
        double *y = (double *)malloc(sizeof(double) * (it + 1));
        for (int i = it; i >= 0; i--) {
            g1[i] = g[i];
            for (int j = i + 1; j < it + 1; j++) g1[i] = g1[i] - HN(i, j) * y[j];
            y[i] = g1[i] / HN(i, i);
        }
        memset(wi, 0, sizeof(double) * n);
        for (int i = 0; i < it + 1; i++) {
            double *Vpi = Vp + (size_t)i * n;
            for (int r = 0; r < n; ++r) wi[r] += y[i] * Vpi[r];
        }
        free(y);
        for (int r = 0; r < n; ++r) uni[r] = wi[r] + x0[r];
        memcpy(px, uni, sizeof(double) * n);
        if (!noconv) break;
        if (iter > nbitermx) break;
    }
#undef HN
    if (iters) *iters = iter;
    if (relres_out) *relres_out = relres / normb;
    free(rot0); free(rot1); free(g); free(g1); free(Hn); free(V); free(Vp);
    free(wi); free(vi); free(ri); free(x0); free(uni); free(D); free(wcl);
    return !noconv;
}

void ffo_matmul(const void *hm, const double *x, double *y, int trans) {
    matmul((const ffo_hm *)hm, x, y, trans);
}

/* ------------------------------------------------------------------ numbering */
/* first-encounter node numbering over elements: nkeys = vertex keys then edge keys
 * (tet edge order {01,02,03,12,13,23}; triangle edge i opposite vertex i).
 * node_tab[k*nn + i] = node number; returns the node count. */
int ffo_number_nodes(int dim, int nv, int nt, const int *elems, int with_vertices,
                     int with_edges, int *node_tab) {
    int nvk = dim + 1, ne = dim == 2 ? 3 : 6;
    int nn = (with_vertices ? nvk : 0) + (with_edges ? ne : 0);
    int64_t cap = 1;
    while (cap < 4 * (int64_t)nt * nn + 16) cap <<= 1;
    uint64_t *keys = (uint64_t *)malloc(cap * sizeof(uint64_t));
    int *vals = (int *)malloc(cap * sizeof(int));
    for (int64_t h = 0; h < cap; ++h) keys[h] = UINT64_MAX;
    int count = 0;
    for (int k = 0; k < nt; ++k) {
        const int *v = elems + (int64_t)k * nvk;
        int m = 0;
        for (int t = 0; t < nn; ++t) {
            uint64_t a, b;
            if (with_vertices && t < nvk) { a = (uint64_t)v[t]; b = 0xffffffffu; }
            else {
                int e = t - (with_vertices ? nvk : 0);
                int i0 = dim == 2 ? tri_edge[e][0] : tet_edge[e][0];
                int i1 = dim == 2 ? tri_edge[e][1] : tet_edge[e][1];
                a = (uint64_t)v[i0]; b = (uint64_t)v[i1];
                if (b < a) { uint64_t s = a; a = b; b = s; }
            }
            uint64_t key = (a << 32) | b;
            uint64_t h = (key * 0x9E3779B97F4A7C15ull) & (cap - 1);
            while (keys[h] != UINT64_MAX && keys[h] != key) h = (h + 1) & (cap - 1);
            if (keys[h] == UINT64_MAX) { keys[h] = key; vals[h] = count++; }
            node_tab[(int64_t)k * nn + m++] = vals[h];
        }
    }
    free(keys); free(vals);
    return count;
}
