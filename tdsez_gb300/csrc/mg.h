// Geometric B-spline multigrid on the device. Internal to the tdz library.
//
// Hierarchy as TDSEZSetupMultigrid (src/multigrid.cpp:205-263): coarse
// knots drop every other simple interior breakpoint, C0 knots stay; the
// prolongation is Boehm knot insertion per axis (multigrid.cpp:52-81),
// applied as a tensor product; coarse operators are the Galerkin products
// P^T A P, formed exactly per axis on the 1D bands (P_d^T B P_d), so every
// level is applied by the same fused kernels and follows stage changes
// without a rebuild. Smoother: Chebyshev iteration in M^-1 A on the
// spectral segment alpha + g [mu_lo, mu_hi] of the stage (M^-1 by exact
// Kronecker line solves); coarsest level: Chebyshev over the whole segment.
#pragma once

#include <memory>
#include <vector>

#include "blas.h"
#include "cnn.h"
#include "fdm.h"
#include "krylov.h"
#include "linesolve.h"
#include "oper.h"

namespace tdz {

// Row-sparse 1D matrix with a fixed row width (prolongation and its transpose).
struct RowSparse {
    int rows = 0, cols = 0, width = 0;
    std::vector<int> col;      // rows * width (-1 = empty)
    std::vector<double> val;
    DevBuf dcol, dval32, dval64;
    void upload();
};

struct MGLevel {
    Space space;                          // sizes of the level
    std::unique_ptr<Operator> op;         // level operator (bands = Galerkin products)
    Operator *opp = nullptr;              // op.get() or the fine operator
    KronSolve minv;
    RowSparse P[3], R[3];                 // to this level from the next coarser: prolongation, restriction
    int n[3] = {1, 1, 1};
    size_t ndof = 0;
    DevBuf x, b, r, d, z, t1, t2;         // working precision vectors
    double mu_lo = 0.0, mu_hi = 0.0;      // spectrum of M^-1 H_E on this level (real part; hi = |mu|max)
    double w_max = 0.0;                   // bound on its imaginary extent (CAP)
};

struct MGOptions {
    int levels = 0;          // 0 = until < 2000 DoFs (MGLevels = 0)
    int smooth = 8;          // Chebyshev degree of pre and post smoothing
    int coarse_its = 12;     // Chebyshev degree of the coarsest solve
    double ratio = 60.0;     // smoothing range [mu_hi / ratio, mu_hi]
    int precision = TDZ_FP32;
    int learned = 0;         // 1: CNN correction of the coarsest solve (FP32 levels)
    int coarse_fdm = 0;      // 1: coarsest level solved by the FDM inverse where it is exact
                             //    (the role of the reference's coarse LU), else the polynomial
};

// Learned coarse correction: after the Chebyshev coarse solve x0 of A_c x = b_c,
// x = x0 + c rms(r) N(r / rms(r)) with r = b_c - A_c x0, c = the training pairs'
// mean ||e|| / ||r||, and N a 3D CNN on the
// coarsest grid (2 channels: real, imaginary) trained on (r / rms(r),
// A_c^-1 r / (c rms(r))) pairs that the solver generates
// (tdz_solver_train_coarse). Unit-RMS inputs and O(1) targets keep the
// ReLU network away from the zero-output collapse. Until trained,
// or with FP64 levels, the plain V-cycle runs.
struct LearnedCoarse {
    CNN net;
    bool on = false, trained = false;
    int width = 32, layers = 4, batch = 8;
    DevBuf in, out, scale;       // planar [2][n] FP32 (batch 1), device ||r||
    DevBuf pin, ptgt;            // training pairs [pairs][2][n]
    int npairs = 0;
    // coarsest-level right-hand sides recorded from the V-cycles of a run
    // (the propagator's own stage solves), the inputs of the training pairs
    DevBuf rec;
    int rec_cap = 0, rec_n = 0;
    bool use_recorded = false;   // train_coarse takes its inputs from rec
    float cscale = 1.f;          // mean ||e|| / ||r|| of the training pairs (output scale)
};

struct Multigrid : Precond {
    Operator *fine = nullptr;
    MGOptions opt;
    std::vector<MGLevel> lv;
    int prec = TDZ_FP32;
    DevBuf in32;                          // FP32 copy of the FP64 input
    long long cycles = 0;
    blas::Reducer red;
    LearnedCoarse lrn;
    std::unique_ptr<PcFDM> cfdm;          // exact coarsest-level inverse (coarse_fdm)
    DevBuf cb64, cx64;                    // its FP64 right-hand side and solution
    long long coarse_exact = 0;           // coarsest solves done by it

    void setup(Operator *fine_, const MGOptions &o, cudaStream_t st);
    void estimate_bounds(cudaStream_t st);
    void vcycle(int l, cudaStream_t st);  // lv[l].b -> lv[l].x
    // learned coarse correction (learned.cu)
    void learned_setup();
    void coarse_correct(MGLevel &m, cudaStream_t st);
    // generate `pairs` pairs at the coarsest level for the current stage and
    // train for `epochs` passes; returns the mean relative loss of the last epoch
    float train_coarse(int pairs, int epochs, float lr, uint64_t seed, cudaStream_t st);
    // record the coarsest right-hand side of the next `capacity` V-cycles
    // (0: stop recording, keep what was recorded)
    void record_coarse(int capacity);
    // train on the recorded right-hand sides (all of them) instead of random ones
    float train_recorded(int epochs, float lr, uint64_t seed, cudaStream_t st);
    // relative error ||e - c|| / ||e|| of the corrected coarse solve c against
    // e = A_c^-1 b on `trials` fresh random right-hand sides, without (first)
    // and with (second) the network
    std::pair<double, double> coarse_gain(int trials, uint64_t seed, cudaStream_t st);
    void apply(const double2 *r, double2 *z, cudaStream_t st) override;
    void refresh() override;
};

// Chebyshev iteration on the level's A x = b (mg_setup.cpp)
void chebyshev(MGLevel &m, int prec, double mu_a, double mu_b, double w, int steps, bool x_zero, cudaStream_t st);

// 1D helpers (mg_setup.cpp)
std::vector<double> coarsen_knots(const std::vector<double> &U, bool *dropped);
int count_spans(const std::vector<double> &U);
// dense-free Boehm prolongation as sparse rows: fine n_f x coarse n_c
RowSparse boehm_prolongation(const std::vector<double> &C, const std::vector<double> &F, int p);
RowSparse transpose(const RowSparse &P);
BandD galerkin(const RowSparse &P, const BandD &B);   // P^T B P (banded, coarse)
// axis contraction out = A (along axis) in, with optional accumulation (mg.cu)
void axis_contract(const RowSparse &A, int axis, const void *in, void *out, int n0, int n1, int n2, bool accumulate,
                   int prec, cudaStream_t st);

}  // namespace tdz
