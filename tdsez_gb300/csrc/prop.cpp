// Crank-Nicolson, Pade(2,2) and Magnus-4 steps on the device.
//
// Crank-Nicolson follows TSTHETA(theta = 1/2) with the IFunction/IJacobian
// of src/monitor.cpp:273-331: the stage equation (M + i h/2 H_E) X = M psi
// with H_E = H(t + h/2), then psi <- 2 X - psi (src/propagator.cpp:94-101).
// Pade(2,2) follows Pade22Step (src/propagator.cpp:564-676): stages
// (M + g_k H_E) y = (M + conj(g_k) H_E) x with g_{1,2} = h(-+sqrt3 + 3i)/12,
// right-hand side 2 M x - A_other x, initial guess x + sum_j w_q,j delta_j
// (binomial weights of order q <= 5). Magnus-4 = EvolveRational's two
// Pade(2,2) half steps with effective fields 2(a2 c1 + a1 c2), 2(a1 c1 + a2 c2)
// (src/propagator.cpp:729-758).
#include "prop.h"

#include "band.h"
#include "fdm.h"

#include <cmath>

namespace tdz {

void PcMass::setup(Operator *op_, int prec_) {
    op = op_;
    prec = prec_;
    n = (size_t)op->sp->ndof();
    std::array<const BandD *, 3> mb{nullptr, nullptr, nullptr};
    for (int d = 0; d < op->sp->dim; ++d) mb[d] = &op->bases[d][kM];
    ks.setup(mb, op->sp->dim);
    buf.alloc(n * (prec == TDZ_FP64 ? sizeof(double2) : sizeof(float2)));
}

void PcMass::apply(const double2 *r, double2 *z, cudaStream_t st) {
    // M^-1 approximates A^-1 up to the (non-zero) stage scalar alpha
    const cd a = 1.0 / op->sigma[0];
    if (prec == TDZ_FP64) {
        blas::copy(r, z, n, TDZ_FP64, st);
        ks.apply(z, TDZ_FP64, st);
        blas::scale(z, a, n, TDZ_FP64, st);
    } else {
        blas::cast(r, TDZ_FP64, buf.ptr, TDZ_FP32, n, st);
        ks.apply(buf.ptr, TDZ_FP32, st);
        blas::cast(buf.ptr, TDZ_FP32, z, TDZ_FP64, n, st);
        blas::scale(z, a, n, TDZ_FP64, st);
    }
}

void Solver::setup(Operator *op_, const SolverOptions &o, cudaStream_t st) {
    op = op_;
    opt = o;
    const long long rows = op->sp->ndof();
    const int restart = o.restart > 0 ? o.restart : (rows > 100000 ? 50 : 30);
    if (o.pc == 0) pc = std::make_unique<PcNone>((size_t)rows);
    else if (o.pc == 1) {
        auto p = std::make_unique<PcMass>();
        p->setup(op, o.pc_precision);
        pc = std::move(p);
    } else if (o.pc == 2) {
        auto p = std::make_unique<Multigrid>();
        MGOptions mo = o.mg;
        mo.precision = o.pc_precision;
        p->setup(op, mo, st);
        pc = std::move(p);
    } else if (o.pc == 3) {
        auto p = std::make_unique<PcFDM>();
        p->setup(op, o.pc_precision);
        pc = std::move(p);
    } else if (o.pc == 4) {
        auto p = std::make_unique<PcBand>();
        p->setup(op);
        pc = std::move(p);
    } else throw Error(TDZ_ERR_ARG, "unknown preconditioner");
    ksp.relaxed = o.relaxed;
    ksp.setup(op, restart, pc.get());
    TDZ_CHECK(o.outer == TDZ_FP64 || o.outer == TDZ_FP64_DF, TDZ_ERR_ARG, "outer precision must be FP64 or FP64_DF");
    ksp.aprec = o.outer;
}

SolveStats Solver::solve(const double2 *b, double2 *x, cudaStream_t st, double bnorm, double2 *cn_psi,
                         bool *cn_done) {
    SolveStats s = ksp.solve(b, x, opt.rtol, opt.maxit, st, bnorm, cn_psi, cn_done);
    if (opt.pc == 3 && static_cast<PcFDM *>(pc.get())->tensor)
        TDZ_CHECK(take_transform_error() == 0, TDZ_ERR_CUDA, "tensor-core transform: a bounded wait ran out");
    ++solves;
    its += s.its;
    return s;
}

void Propagator::setup(Operator *op_, int kind_, const SolverOptions &o, int guess_order_, cudaStream_t st) {
    op = op_;
    kind = kind_;
    TDZ_CHECK(kind >= 0 && kind <= 2, TDZ_ERR_ARG, "unknown propagator kind");
    TDZ_CHECK(guess_order_ >= -1 && guess_order_ <= 5, TDZ_ERR_ARG, "guess order must be -1..5");
    guess_order = guess_order_;
    n = (size_t)op->sp->ndof();
    rhs.alloc(n * sizeof(double2));
    tmp.alloc(n * sizeof(double2));
    x0.alloc(n * sizeof(double2));
    const int slots = kind == 0 ? 1 : (kind == 1 ? 2 : 4);
    for (int s = 0; s < slots; ++s)
        for (int j = 0; j < guess_order; ++j) hist[s][j].alloc(n * sizeof(double2));
    // preconditioners are built from the stage of the first step
    // (src/propagator.cpp:446-460); the multigrid follows later stage changes
    nsolvers = kind == 0 ? 1 : 2;
    aprec = o.outer;
    for (int k = 0; k < nsolvers; ++k) {
        solver[k].setup(op, o, st);
        refresh[k] = PCRefresh{};
        refresh[k].cap = o.pc_refresh_its;
    }
}

void Propagator::extrapolate(int slot, double2 *psi, cudaStream_t st) {
    static const double w[5][5] = {{1, 0, 0, 0, 0}, {2, -1, 0, 0, 0}, {3, -3, 1, 0, 0},
                                   {4, -6, 4, -1, 0}, {5, -10, 10, -5, 1}};
    const int q = std::min(guess_order, hist_count[slot]);
    if (q <= 0) return;
    std::vector<const void *> V(q);
    std::vector<cd> a(q);
    for (int j = 0; j < q; ++j) { V[j] = hist[slot][j].ptr; a[j] = w[q - 1][j]; }
    blas::maxpy(psi, q, V.data(), a.data(), n, TDZ_FP64, st);
}

void Propagator::record(int slot, const double2 *y, const double2 *x, cudaStream_t st) {
    if (guess_order <= 0) return;
    DevBuf oldest = std::move(hist[slot][guess_order - 1]);
    for (int j = guess_order - 1; j > 0; --j) hist[slot][j] = std::move(hist[slot][j - 1]);
    hist[slot][0] = std::move(oldest);
    blas::axpbypcz(hist[slot][0].ptr, 1.0, y, 0.0, x, -1.0, n, TDZ_FP64, st);
    hist_count[slot] = std::min(hist_count[slot] + 1, guess_order);
}

void Propagator::stage_solve(int k, const double2 *b, double2 *x, cudaStream_t st, double bnorm, double2 *cn_psi,
                             bool *cn_done) {
    SolveStats s = solver[k].solve(b, x, st, bnorm, cn_psi, cn_done);
    last = s;
    ++solves;
    its += s.its;
    if (refresh[k].stale(s.its)) solver[k].pc->refresh();
    if (s.reason <= 0) {
        ++failures;
        throw Error(s.reason == -9 ? TDZ_ERR_BREAKDOWN : TDZ_ERR_NOT_CONVERGED,
                    "stage solve did not converge (reason " + std::to_string(s.reason) + ", " +
                        std::to_string(s.its) + " iterations, residual " + std::to_string(s.rnorm / s.bnorm) + ")");
    }
}

void Propagator::cn_step(double2 *psi, double h, const std::vector<cd> &c, cudaStream_t st) {
    op->set_stage(1.0, cd(0.0, 0.5 * h), c);
    double bn = -1.0;
    op->residual(TDZ_MASS, aprec, psi, nullptr, rhs.ptr, st, op->fused_reductions() ? &bn : nullptr);   // M psi
    double2 *X = tmp.as<double2>();
    if (guess_order < 0) {
        solver[0].pc->apply(rhs.as<double2>(), X, st);           // x0 = P^-1 b
    } else {
        blas::copy(psi, X, n, TDZ_FP64, st);
        extrapolate(0, X, st);
    }
    // without extrapolation history X is not needed after the step: the last
    // FGMRES update and psi <- 2 X - psi then share one pass
    bool fused = false;
    stage_solve(0, rhs.as<double2>(), X, st, bn, guess_order <= 0 ? psi : nullptr, &fused);
    if (!fused) {
        record(0, X, psi, st);
        blas::axpby(psi, 2.0, X, -1.0, n, TDZ_FP64, st);       // psi <- 2 X - psi
    }
}

void Propagator::pade_step(double2 *psi, double h, const std::vector<cd> &c, int slot, cudaStream_t st) {
    const double s3 = std::sqrt(3.0);
    const cd g[2] = {h * cd(-s3, 3.0) / 12.0, h * cd(s3, 3.0) / 12.0};
    for (int k = 0; k < 2; ++k) {
        // rhs = (M + conj(g_k) H_E) x = 2 M x - A_{1-k} x
        op->set_stage(1.0, g[1 - k], c);
        op->apply(TDZ_STAGE, aprec, psi, tmp.ptr, st);
        op->apply(TDZ_MASS, aprec, psi, rhs.ptr, st);
        blas::axpby(rhs.ptr, -1.0, tmp.ptr, 2.0, n, TDZ_FP64, st);
        blas::copy(psi, x0.ptr, n, TDZ_FP64, st);               // stage input
        const int s = 2 * slot + k;
        op->set_stage(1.0, g[k], c);
        if (guess_order < 0) solver[k].pc->apply(rhs.as<double2>(), psi, st);   // x0 = P^-1 b
        else extrapolate(s, psi, st);
        stage_solve(k, rhs.as<double2>(), psi, st);
        record(s, psi, x0.as<double2>(), st);
    }
}

void Propagator::magnus_step(double2 *psi, double h, const std::vector<cd> &c1, const std::vector<cd> &c2,
                             cudaStream_t st) {
    const double s3 = std::sqrt(3.0);
    const double a1 = (3.0 - 2.0 * s3) / 12.0, a2 = (3.0 + 2.0 * s3) / 12.0;
    std::vector<cd> ea(c1.size()), eb(c1.size());
    for (size_t i = 0; i < c1.size(); ++i) {
        ea[i] = 2.0 * (a2 * c1[i] + a1 * c2[i]);
        eb[i] = 2.0 * (a1 * c1[i] + a2 * c2[i]);
    }
    pade_step(psi, 0.5 * h, ea, 0, st);
    pade_step(psi, 0.5 * h, eb, 1, st);
}

}  // namespace tdz
