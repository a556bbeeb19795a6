// Time steppers on the device: Crank-Nicolson, Pade(2,2), Magnus-4.
// Internal to the tdz library.
#pragma once

#include <memory>

#include "krylov.h"
#include "linesolve.h"
#include "mg.h"

namespace tdz {

struct SolverOptions {
    int restart = 0;      // 0: 30, or 50 above 100000 rows (src/propagator.cpp:132-141)
    int maxit = 1000;
    double rtol = 1e-12;
    int pc = 2;           // 0 none, 1 Kronecker mass, 2 multigrid
    int pc_precision = TDZ_FP32;
    int outer = TDZ_FP64;  // operator applies of FGMRES and the right-hand sides (TDZ_FP64 or TDZ_FP64_DF)
    bool relaxed = false;  // FP32 Arnoldi applies, true residual in `outer` at every restart
    int pc_refresh_its = -1;   // propagators: rebuild the preconditioner above this many iterations (-1: off)
    MGOptions mg;
};

// Kronecker mass preconditioner P = M (exact line solves), FP32 or FP64 inside.
struct PcMass : Precond {
    Operator *op = nullptr;
    KronSolve ks;
    int prec = TDZ_FP32;
    DevBuf buf;
    size_t n = 0;
    void setup(Operator *op_, int prec_);
    void apply(const double2 *r, double2 *z, cudaStream_t st) override;
};

// KSP + PC for the stage operator of one Operator.
struct Solver {
    Operator *op = nullptr;
    SolverOptions opt;
    std::unique_ptr<Precond> pc;
    FGMRES ksp;
    long long solves = 0, its = 0;
    void setup(Operator *op_, const SolverOptions &o, cudaStream_t st);
    // bnorm: ||b|| when the caller has it (< 0: computed in the solve);
    // cn_psi / cn_done: see FGMRES::solve
    SolveStats solve(const double2 *b, double2 *x, cudaStream_t st, double bnorm = -1.0, double2 *cn_psi = nullptr,
                     bool *cn_done = nullptr);
};

// Preconditioner refresh rule of TDSEZPCRefresh (include/tdsez_propagator.hpp:17-31):
// after a (re)build the first solve sets the base; a solve needing more than
// 2*base + 5 iterations (or more than cap, when cap >= 0) asks for a rebuild.
struct PCRefresh {
    int base = -1, rebuilds = 0, cap = -1;
    bool stale(int its) {
        if (cap >= 0 && its > cap) { base = -1; ++rebuilds; return true; }
        if (base < 0) { base = its; return false; }
        if (its <= 2 * base + 5) return false;
        base = -1;
        ++rebuilds;
        return true;
    }
};

struct Propagator {
    Operator *op = nullptr;
    int aprec = TDZ_FP64;         // arithmetic of the right-hand-side applies
    int kind = 0;                 // TDZ_CN, TDZ_PADE22, TDZ_MAGNUS4
    Solver solver[2];             // one per stage shift (CN: one)
    int nsolvers = 1;
    PCRefresh refresh[2];
    size_t n = 0;
    DevBuf rhs, tmp, x0;
    int guess_order = 3;
    DevBuf hist[4][5];
    int hist_count[4] = {0, 0, 0, 0};
    long long solves = 0, its = 0, failures = 0;
    SolveStats last;

    void setup(Operator *op_, int kind_, const SolverOptions &o, int guess_order_, cudaStream_t st);
    void cn_step(double2 *psi, double h, const std::vector<cd> &c, cudaStream_t st);
    void pade_step(double2 *psi, double h, const std::vector<cd> &c, int slot, cudaStream_t st);
    void magnus_step(double2 *psi, double h, const std::vector<cd> &c1, const std::vector<cd> &c2, cudaStream_t st);

  private:
    void extrapolate(int slot, double2 *psi, cudaStream_t st);
    void record(int slot, const double2 *y, const double2 *x, cudaStream_t st);
    void stage_solve(int k, const double2 *b, double2 *x, cudaStream_t st, double bnorm = -1.0,
                     double2 *cn_psi = nullptr, bool *cn_done = nullptr);
};

// Bound states of H c = E M c nearest a target (eigen.cpp)
struct EigenResult {
    std::vector<double> energies, berr;   // ascending energies and their backward errors
    int solves = 0, restarts = 0;
    long long inner_its = 0;
};
// nev eigenpairs nearest `target`; vecs: nev FP64 device vectors (in: a start
// vector in vecs[0], its real part is used; out: M-normalised eigenvectors);
// Lanczos stops when the Ritz residual estimates are below tol |theta|
EigenResult eigen_solve(Operator &op, int nev, double target, double tol, int maxit, const SolverOptions &so,
                        double2 *vecs, cudaStream_t st);

}  // namespace tdz
