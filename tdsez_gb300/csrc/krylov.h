// Flexible GMRES in FP64 on the device with a pluggable preconditioner.
// Internal to the tdz library.
#pragma once

#include <memory>
#include <vector>

#include "blas.h"
#include "oper.h"

namespace tdz {

// z = P^-1 r on FP64 vectors (a preconditioner may work in FP32 inside).
struct Precond {
    virtual ~Precond() = default;
    virtual void apply(const double2 *r, double2 *z, cudaStream_t st) = 0;
    virtual void refresh() {}   // rebuild from the current stage operator
    virtual long long launches() const { return 0; }
    // z = P^-1 r and ||z||^2 into *norm2 (device), in the pass that writes z,
    // where the preconditioner can (has_apply_norm)
    virtual bool has_apply_norm() const { return false; }
    virtual void apply_norm(const double2 *r, double2 *z, double * /*norm2*/, cudaStream_t st) { apply(r, z, st); }
};

struct PcNone : Precond {
    size_t n;
    explicit PcNone(size_t n_) : n(n_) {}
    void apply(const double2 *r, double2 *z, cudaStream_t st) override { blas::copy(r, z, n, TDZ_FP64, st); }
};

struct SolveStats {
    int its = 0;           // iterations of the last solve
    int reason = 0;        // > 0 converged, < 0 diverged (PETSc KSPConvergedReason convention)
    double rnorm = 0.0;    // final residual estimate (absolute)
    double bnorm = 0.0;
};

// FGMRES(m), right preconditioned, classical Gram-Schmidt with one
// re-orthogonalisation (two fused passes per iteration), Givens rotations on
// the host. Replaces KSPFGMRES/KSPGMRES with PC_RIGHT of
// src/propagator.cpp:125-197,315-370 (stop when ||b - A x|| <= rtol ||b||).
struct FGMRES {
    Operator *op = nullptr;
    size_t n = 0;
    int restart = 30;
    Precond *pc = nullptr;
    std::vector<DevBuf> V, Z;
    DevBuf w;
    DevBuf znd;                 // ||z_j||^2 of relaxed columns from the preconditioner's output pass
    blas::Reducer red;
    SolveStats last;
    long long applies = 0;
    long long early_accepts = 0;   // iterations that met the target after one Gram-Schmidt pass
    int aprec = TDZ_FP64;   // operator apply arithmetic: TDZ_FP64 or TDZ_FP64_DF (FP64 vectors either way)
    // Relaxed Arnoldi applies (inexact Krylov): A z_j in FP32 arithmetic
    // while the residual r0 = b - A x of every restart stays in aprec. The
    // FP32 apply's error is bounded elementwise by gamma |A| |z_j| (gamma =
    // k u / (1 - k u), u = 2^-24, k the accumulation depth of the three band
    // stages plus the input and band roundings), so the true residual of the
    // cycle differs from its estimate by at most
    //   sum_j |y_j| gamma || |A| || ||z_j||,
    // with || |A| || bounded from the Kronecker factors (abs_norm_bound). A
    // cycle that reports convergence is accepted when the estimate plus that
    // bound meets the target; otherwise one more restart, whose aprec residual
    // decides. A relaxed cycle that fails to cut the true residual tenfold
    // switches the solve back to exact applies.
    bool relaxed = false;
    DevBuf z32, w32;
    long long relaxed_applies = 0;
    long long relaxed_accepts = 0;   // solves that ended on a certified relaxed cycle

    void setup(Operator *op_, int restart_, Precond *pc_);
    // Solve A x = b (A = the operator's current stage, FP64), x holds the guess.
    // bnorm: ||b|| when the caller has it (< 0: computed here). cn_psi: when
    // the solve converges after one iteration, its last update is fused with
    // the Crank-Nicolson state update psi = 2 x - psi (*cn_done = true; x is
    // then left at its initial guess); otherwise x is the solution as usual.
    SolveStats solve(const double2 *b, double2 *x, double rtol, int maxit, cudaStream_t st, double bnorm = -1.0,
                     double2 *cn_psi = nullptr, bool *cn_done = nullptr);
};

}  // namespace tdz
