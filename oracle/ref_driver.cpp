// ref_driver.cpp -- extern "C" driver around FreeFEM's own HashMatrix and Krylov solvers.
//
// TEST INFRASTRUCTURE ONLY.  Linked with src/femlib/HashMatrix.cpp, src/femlib/CG.cpp and
// src/femlib/gibbs.cpp compiled unmodified from the FreeFEM sources (recipe: oracle/Makefile, target `ref`);
// the result lives in oracle/_ref/ and is never shipped.  It pins the C restatement in
// oracle/ffo.c: same hash-matrix pattern and COO order, same SetBC, same CG and fgmres.
//
// The Jacobi preconditioner and the x0 = b/tgv initialisation restate HMatVirtPrecon and
// SolverCG::dosolver (src/femlib/VirtualSolverCG.hpp:27-99,169-190), whose header pulls
// in the interpreter; everything else below calls reference code directly.
#include <cmath>
#include <cstring>
#include <iostream>
#include <vector>
#include "HashMatrix.hpp"
#include "CG.hpp"

long verbosity = 0;
long mpirank = 0;
void ShowDebugStack() {}

typedef HashMatrix<int, double> HM;

struct RefMat : CGMatVirt<int, double> {
  HM *A; int t;
  RefMat(HM *AA, int trans) : CGMatVirt<int, double>(AA->n), A(AA), t(trans) {}
  double *addmatmul(double *x, double *Ax) const { return A->addMatMul(x, Ax, t); }
};

struct RefJacobi : CGMatVirt<int, double> {
  double *d; int *wcl; double tgv; int ntgv;
  RefJacobi(HM *A, double ttgv) : CGMatVirt<int, double>(A->n), d(new double[A->n]), wcl(0), tgv(ttgv), ntgv(0) {
    int n = A->n, ntgv1 = 0;
    double tgvm = A->gettgv(&ntgv1);
    if (ntgv1) {
      wcl = new int[n];
      double tgve = tgvm <= 0 ? 1e200 : tgvm;
      for (int i = 0; i < n; ++i) ntgv += (wcl[i] = ((*A)(i, i) == tgve));
    }
    for (int i = 0; i < n; ++i) d[i] = (*A)(i, i);
    for (int i = 0; i < n; ++i) d[i] = (std::norm(d[i]) < 1e-60) ? 1. : 1. / d[i];
  }
  ~RefJacobi() { delete[] d; delete[] wcl; }
  double *addmatmul(double *x, double *Ax) const {
    for (int i = 0; i < this->n; ++i) Ax[i] += d[i] * x[i];
    return Ax;
  }
  void SetInitWithBC(double *rhs, double *x) const {
    if (wcl) for (int i = 0; i < this->n; ++i) if (wcl[i]) x[i] = rhs[i] / tgv;
  }
};

// FreeFEM's Gibbs renumbering (src/femlib/gibbs.cpp:209, `integer` = long there).
int gibbsa_(long *n, long *ptvois, long *vois, long *r, long *m, long *nv, long *nx, long *ny, long *nn,
            long *w1, long *w2, long *pfold, long *pfnew, long *impre, long *nfout);

extern "C" {

// gibbsa_ with the work arrays FESpace::renum gives it (gibbs.cpp:1131-1142)
int ref_gibbs(long n, long *ptvois, long *vois, long *r, long *pfold, long *pfnew) {
  std::vector<long> m(n + 1), nv(2 * (n + 1)), nx(n + 1), ny(n + 1), nn(n + 1), w1(n + 1), w2(n + 1);
  long impre = 0, nfout = 6;
  return gibbsa_(&n, ptvois, vois, r, m.data(), nv.data(), nx.data(), ny.data(), nn.data(), w1.data(),
                 w2.data(), pfold, pfnew, &impre, &nfout);
}

void *ref_hm_new(int n) { return new HM(n, n, 0, 0); }
void ref_hm_free(void *h) { delete (HM *)h; }

// scatter element contributions in the given order: *npij(i,j) += v (HashMatrix.cpp:1309-1317)
void ref_hm_add(void *h, long ne, const int *I, const int *J, const double *V) {
  HM *A = (HM *)h;
  for (long k = 0; k < ne; ++k) *A->npij(I[k], J[k]) += V[k];
}

void ref_hm_setbc(void *h, const char *onbc, double tgv) {
  HM *A = (HM *)h;
  std::vector<char> w(onbc, onbc + A->n);
  A->SetBC(w.data(), tgv);
}

long ref_hm_nnz(void *h) { return (long)((HM *)h)->nnz; }

void ref_hm_coo(void *h, int *I, int *J, double *V) {
  HM *A = (HM *)h;
  for (size_t k = 0; k < A->nnz; ++k) { I[k] = A->i[k]; J[k] = A->j[k]; V[k] = A->aij[k]; }
}

// sorted CSR of the pattern (HashMatrix::CSR, HashMatrix.cpp:859-867)
void ref_hm_csr(void *h, int *rowptr, int *col, double *val) {
  HM *A = (HM *)h;
  int *IA = 0, *JA = 0; double *AA = 0;
  A->CSR(IA, JA, AA);
  std::memcpy(rowptr, IA, sizeof(int) * (A->n + 1));
  std::memcpy(col, JA, sizeof(int) * A->nnz);
  std::memcpy(val, AA, sizeof(double) * A->nnz);
}

int ref_cg(void *h, const double *b, double *x, double eps, int itmax, int trans, double tgv,
           int *iters) {
  HM *A = (HM *)h;
  RefMat AA(A, trans);
  RefJacobi C(A, tgv);
  std::vector<double> bb(b, b + A->n);
  C.SetInitWithBC(bb.data(), x);
  int it = itmax > 0 ? itmax : A->n;
  double e = eps;
  int r = ConjugueGradient<int, double>(AA, C, bb.data(), x, it, e, 0);
  if (iters) *iters = it;
  return r;
}

int ref_fgmres(void *h, const double *b, double *x, double eps, int itmax, int restart, int trans,
               double tgv, int *iters) {
  HM *A = (HM *)h;
  RefMat AA(A, trans);
  RefJacobi C(A, tgv);
  std::vector<double> bb(b, b + A->n);
  C.SetInitWithBC(bb.data(), x);
  int it = itmax > 0 ? itmax : A->n;
  double e = eps;
  bool r = fgmres<double, int>(AA, C, 1, bb.data(), x, e, it, restart, 0, C.wcl);
  if (iters) *iters = it;
  return r ? 1 : 0;
}

}  // extern "C"
