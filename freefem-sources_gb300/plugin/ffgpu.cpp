// ffgpu.cpp -- FreeFEM plugin: `load "ffgpu"` registers the GB300 solvers.
//
// Build with FreeFEM's own plugin compiler (it adds ff++.hpp's include path and flags):
//     ff-c++ -auto ffgpu.cpp -I<repo>/include <repo>/freefem-sources_gb300/ffgpu/lib/libffgpu.so
// Scripts then select the device solvers by name, exactly like FreeFEM's own:
//     load "ffgpu"
//     matrix A = a(Vh, Vh, solver=GPUCG, eps=1e-10);      // or set(A, solver=GPUCG)
//     u[] = A^-1 * b;   u[] = A'^-1 * b;
//
// Solvers registered (addsolver, src/femlib/SparseLinearSolver.hpp:96-102):
//   GPUCG       Jacobi-PCG on the GPU      -- same algorithm and stopping rule as SolverCG
//                                             (src/femlib/VirtualSolverCG.hpp:113-192)
//   GPUGMRES    right-preconditioned FGMRES -- as SolverGMRES (VirtualSolverCG.hpp:195-257)
//   GPUCGMIXED  FP32 inner PCG + FP64 refinement, same stopping rule on the true residual
// The matrix FreeFEM assembled is uploaded once per numeric state (fac_numeric, in sorted CSR
// via HashMatrix::CSR, HashMatrix.cpp:859-867) and stays on the device with the solver object,
// which the matrix owns (VirtualMatrix.hpp:71-94).  Errors become ExecError / ffassert as in
// FreeFEM's own solvers; there is no CPU fallback.
#include <cmath>
#include <iostream>

#include "ff++.hpp"
#include "ffgpu.h"

namespace {

ffgpu_ctx *g_ctx = nullptr;

ffgpu_ctx *context() {
    if (!g_ctx) {
        int r = ffgpu_ctx_create(0, &g_ctx);
        if (r != FFGPU_OK) {
            g_ctx = nullptr;
            ExecError((std::string("ffgpu: no usable CUDA device: ") + ffgpu_last_error()).c_str());
        }
    }
    return g_ctx;
}

enum Kind { kCG = 0, kGMRES = 1, kMixed = 2 };

template <int KIND>
class SolverGpu : public VirtualSolver<int, double> {
   public:
    // 1 unsym, 2 herm, 4 sym, 8 pos, 16 nopos, 32 seq (as SolverCG / SolverGMRES): full storage
    static const int orTypeSol;
    typedef HashMatrix<int, double> HMat;
    HMat &A;
    ffgpu_matrix *M;
    double eps, tgv;
    long itmax, verb, restart;
    double *veps;
    long *getnbiter;
    long cs, cn;

    SolverGpu(HMat &AA, const Data_Sparse_Solver &ds, Stack)
        : A(AA), M(nullptr), eps(ds.epsilon), tgv(ds.tgv), itmax(ds.itmax), verb(ds.verb),
          restart(ds.NbSpace), veps(ds.veps), getnbiter(ds.getnbiter), cs(0), cn(0) {
        if (ds.precon) ExecError("ffgpu: a script precon= function cannot run on the GPU");
        ffassert(A.n == A.m);
    }
    ~SolverGpu() {
        if (M) ffgpu_matrix_destroy(M);
    }
    void UpdateState() {
        if (A.GetReDoNumerics()) cn++;
        if (A.GetReDoSymbolic()) cs++;
        this->ChangeCodeState(A.n, cs, cn);
    }
    void fac_numeric() {
        int *IA = nullptr, *JA = nullptr;
        double *AA = nullptr;
        A.CSR(IA, JA, AA);
        if (M) {
            ffgpu_matrix_destroy(M);
            M = nullptr;
        }
        int r = ffgpu_matrix_from_csr(context(), A.n, (int64_t)A.nnz, IA, JA, AA, &M);
        if (r != FFGPU_OK) ExecError((std::string("ffgpu upload: ") + ffgpu_last_error()).c_str());
    }
    void dosolver(double *x, double *b, int N, int trans) {
        ffgpu_solver_stats st;
        int r;
        if (KIND == kMixed) {
            ffgpu_ir_params p = {eps, 0.0, 0, 30, tgv, 8, 0};
            r = FFGPU_OK;
            for (int k = 0; k < N && r == FFGPU_OK; ++k)
                r = ffgpu_solve_ir(M, b + (size_t)k * A.n, x + (size_t)k * A.n, &p, &st);
        } else {
            ffgpu_solver_params p = {eps, (int)itmax, (int)restart, tgv, (int)verb, 8};
            r = KIND == kCG ? ffgpu_solve_cg(M, b, x, N, trans, &p, &st)
                            : ffgpu_solve_gmres(M, b, x, N, trans, &p, &st);
        }
        if (r == FFGPU_ENOCONV) {
            std::cerr << "Error: ffgpu Krylov solver did not converge: " << ffgpu_last_error() << std::endl;
            ffassert(0);
        }
        if (r != FFGPU_OK) ExecError((std::string("ffgpu solve: ") + ffgpu_last_error()).c_str());
        if (getnbiter) *getnbiter = st.iterations;
        if (veps) *veps = KIND == kGMRES ? eps : std::sqrt(st.eps2);
        if (verb > 1) std::cout << "  ffgpu: " << st.iterations << " iterations, " << st.elapsed_ms << " ms" << std::endl;
    }
};

template <> const int SolverGpu<kCG>::orTypeSol = 1 | 2 | 4 | 8 | 32;
template <> const int SolverGpu<kGMRES>::orTypeSol = 1 | 2 | 4 | 8 | 16 | 32;
template <> const int SolverGpu<kMixed>::orTypeSol = 1 | 2 | 4 | 8 | 32;

}  // namespace

static void Load_Init() {
    addsolver<SolverGpu<kCG> >("GPUCG", 20);
    addsolver<SolverGpu<kGMRES> >("GPUGMRES", 20);
    addsolver<SolverGpu<kMixed> >("GPUCGMIXED", 20);
    // script constants, as lgfem.cpp:6380-6395 declares CG, GMRES, ...: solver=GPUCG
    static std::string gpucg = "GPUCG", gpugmres = "GPUGMRES", gpumixed = "GPUCGMIXED";
    Global.New("GPUCG", CConstant<std::string *>(&gpucg));
    Global.New("GPUGMRES", CConstant<std::string *>(&gpugmres));
    Global.New("GPUCGMIXED", CConstant<std::string *>(&gpumixed));
    if (verbosity > 1) std::cout << " load: ffgpu (GPUCG, GPUGMRES, GPUCGMIXED)" << std::endl;
}

LOADFUNC(Load_Init)
