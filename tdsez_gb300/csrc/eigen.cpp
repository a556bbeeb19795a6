// Shift-invert eigensolver for the bound states H c = E M c on the device,
// the role of the SLEPc Krylov-Schur GHEP solve of src/core.cpp:887-1048
// (target, shift offset below it, acceptance by the backward error of
// TDSEZBackwardError, src/core.cpp:474-492, at 1e-8).
//
// Thick-restart Lanczos (the Hermitian form of Krylov-Schur) on
// T = (H - s M)^-1 M, which is self-adjoint in the M inner product with
// eigenvalues theta = 1 / (E - s): the states nearest the target are the
// largest |theta|. The basis V and M V stay on the device in FP64; every
// column is M-orthogonalised against the whole basis twice (classical
// Gram-Schmidt, fused multi-dots); the projected matrix is built on the host
// from the computed coefficients and diagonalised by cyclic Jacobi. A
// restart keeps the k wanted Ritz vectors plus the last Lanczos vector,
// whose couplings to them are the next column's coefficients. The solve of
// (H - s M) y = M v is the library's FGMRES with its preconditioners on the
// stage alpha = -s, g = 1 (the FDM inverse is exact for z-layered operators,
// the multigrid V-cycle general). A real start vector keeps every vector
// real, so the projected matrix is real symmetric.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "prop.h"

namespace tdz {

namespace {

// eigen-decomposition of a real symmetric n x n matrix (row-major A,
// destroyed): eigenvalues w, eigenvectors in the columns of Q (cyclic Jacobi)
void sym_eig(std::vector<double> &A, int n, std::vector<double> &w, std::vector<double> &Q) {
    Q.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double v = A[(size_t)i * n + j] * A[(size_t)i * n + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * std::max(tot, 1e-300)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (std::abs(apq) < 1e-300) continue;
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::abs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {   // A <- J^T A J
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - s * akq;
                    A[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - s * aqk;
                    A[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double qkp = Q[(size_t)k * n + p], qkq = Q[(size_t)k * n + q];
                    Q[(size_t)k * n + p] = c * qkp - s * qkq;
                    Q[(size_t)k * n + q] = s * qkp + c * qkq;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = A[(size_t)i * n + i];
}

}  // namespace

EigenResult eigen_solve(Operator &op, int nev, double target, double tol, int maxit, const SolverOptions &so,
                        double2 *vecs, cudaStream_t st) {
    TDZ_CHECK(nev >= 1 && nev <= 32, TDZ_ERR_ARG, "nev must be 1..32");
    TDZ_CHECK(op.cap_bound == 0.0, TDZ_ERR_UNSUPPORTED,
              "the bound-state solve needs a Hermitian H: build its operator without the absorbing layer");
    const size_t n = (size_t)op.sp->ndof();
    TDZ_CHECK((long long)n > nev, TDZ_ERR_ARG, "more eigenpairs than unknowns");
    // shift slightly below the target (src/core.cpp:919-925)
    const double shift = target - 1e-3 * std::max(1.0, std::abs(target));
    const int m = std::min<long long>((long long)n - 1, std::max(2 * nev + 12, 24));   // basis size
    const int keep = std::min(m - 2, nev + std::max(2, nev / 2));                       // kept at a restart

    // stage A = H - s M and its solver
    op.set_stage(cd(-shift, 0.0), cd(1.0, 0.0), std::vector<cd>(op.coupled.size(), cd(0.0)));
    Solver solver;
    solver.setup(&op, so, st);

    std::vector<DevBuf> V, MV;
    for (int i = 0; i <= m; ++i) {
        V.emplace_back(n * sizeof(double2));
        MV.emplace_back(n * sizeof(double2));
    }
    DevBuf w(n * sizeof(double2)), tmp(n * sizeof(double2));
    std::vector<DevBuf> keepV, keepMV;
    for (int i = 0; i < keep; ++i) {
        keepV.emplace_back(n * sizeof(double2));
        keepMV.emplace_back(n * sizeof(double2));
    }
    blas::Reducer red;
    std::vector<const void *> Vp(m + 1), MVp(m + 1);
    auto refresh_ptrs = [&] {
        for (int i = 0; i <= m; ++i) { Vp[i] = V[i].ptr; MVp[i] = MV[i].ptr; }
    };
    refresh_ptrs();
    const int aprec = TDZ_FP64_DF;

    // M-normalised start vector: the real part of the caller's vecs[0]
    blas::copy(vecs, V[0].ptr, n, TDZ_FP64, st);
    blas::keep_real(V[0].ptr, n, st);
    {
        op.apply(TDZ_MASS, aprec, V[0].ptr, MV[0].ptr, st);
        cd vm;
        const void *one[1] = {V[0].ptr};
        blas::mdot(red, one, 1, MV[0].ptr, n, TDZ_FP64, &vm, st);
        TDZ_CHECK(vm.real() > 0.0 && std::isfinite(vm.real()), TDZ_ERR_ARG, "the start vector is zero or not finite");
        const double s = 1.0 / std::sqrt(vm.real());
        blas::scale(V[0].ptr, s, n, TDZ_FP64, st);
        blas::scale(MV[0].ptr, s, n, TDZ_FP64, st);
    }

    std::vector<double> G((size_t)m * m, 0.0);   // projected matrix V^T M T V
    std::vector<cd> h(m + 1), h2(m + 1);
    int j0 = 0, solves = 0, restarts = 0;
    EigenResult res;
    std::vector<double> theta, S;
    double beta = 0.0;
    std::vector<int> order;
    bool converged = false;
    while (true) {
        for (int j = j0; j < m; ++j) {
            // w = T v_j = (H - s M)^-1 M v_j
            blas::zero(w.ptr, n, TDZ_FP64, st);
            const SolveStats ss = solver.solve(MV[j].as<double2>(), w.as<double2>(), st);
            ++solves;
            TDZ_CHECK(ss.reason > 0, TDZ_ERR_NOT_CONVERGED,
                      "shift-invert solve did not converge (reason " + std::to_string(ss.reason) + ")");
            TDZ_CHECK(solves <= maxit, TDZ_ERR_NOT_CONVERGED,
                      "eigensolve: " + std::to_string(maxit) + " shift-invert solves without convergence");
            // two classical Gram-Schmidt passes in the M inner product
            blas::mdot(red, MVp.data(), j + 1, w.ptr, n, TDZ_FP64, h.data(), st);
            std::vector<cd> a(j + 1);
            for (int i = 0; i <= j; ++i) a[i] = -h[i];
            blas::maxpy(w.ptr, j + 1, Vp.data(), a.data(), n, TDZ_FP64, st);
            blas::mdot(red, MVp.data(), j + 1, w.ptr, n, TDZ_FP64, h2.data(), st);
            for (int i = 0; i <= j; ++i) a[i] = -h2[i];
            blas::maxpy(w.ptr, j + 1, Vp.data(), a.data(), n, TDZ_FP64, st);
            // column j of the projected matrix: G_ij = <v_i, M T v_j> (for the
            // first column after a restart this holds the couplings of the kept
            // Ritz vectors to the continued vector)
            for (int i = 0; i <= j; ++i) G[(size_t)i * m + j] = G[(size_t)j * m + i] = (h[i] + h2[i]).real();
            // beta = ||w||_M, v_{j+1} = w / beta
            op.apply(TDZ_MASS, aprec, w.ptr, MV[j + 1].ptr, st);
            cd wm;
            const void *wp[1] = {w.ptr};
            blas::mdot(red, wp, 1, MV[j + 1].ptr, n, TDZ_FP64, &wm, st);
            beta = std::sqrt(std::max(wm.real(), 0.0));
            TDZ_CHECK(std::isfinite(beta), TDZ_ERR_BREAKDOWN, "eigensolve: non-finite Lanczos vector");
            if (beta == 0.0) beta = 1e-300;   // invariant subspace: the residual estimates are zero
            blas::axpby(V[j + 1].ptr, 1.0 / beta, w.ptr, 0.0, n, TDZ_FP64, st);
            blas::scale(MV[j + 1].ptr, 1.0 / beta, n, TDZ_FP64, st);
            if (j + 1 < m) G[(size_t)(j + 1) * m + j] = G[(size_t)j * m + j + 1] = beta;
        }
        // Ritz pairs of the m x m projected matrix; wanted: largest |theta|
        std::vector<double> A(G);
        sym_eig(A, m, theta, S);
        order.resize(m);
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return std::abs(theta[a]) > std::abs(theta[b]); });
        converged = true;
        for (int i = 0; i < nev; ++i) {
            const int c = order[i];
            const double est = std::abs(beta * S[(size_t)(m - 1) * m + c]);
            if (!(est <= tol * std::abs(theta[c]))) converged = false;
        }
        if (converged) break;
        // thick restart: V <- [V S_keep, v_m], G <- diag(theta_keep)
        ++restarts;
        for (int i = 0; i < keep; ++i) {
            const int c = order[i];
            std::vector<cd> sc(m);
            for (int r = 0; r < m; ++r) sc[r] = S[(size_t)r * m + c];
            blas::zero(keepV[i].ptr, n, TDZ_FP64, st);
            blas::maxpy(keepV[i].ptr, m, Vp.data(), sc.data(), n, TDZ_FP64, st);
            blas::zero(keepMV[i].ptr, n, TDZ_FP64, st);
            blas::maxpy(keepMV[i].ptr, m, MVp.data(), sc.data(), n, TDZ_FP64, st);
        }
        for (int i = 0; i < keep; ++i) {
            std::swap(V[i], keepV[i]);
            std::swap(MV[i], keepMV[i]);
        }
        std::swap(V[keep], V[m]);
        std::swap(MV[keep], MV[m]);
        refresh_ptrs();
        std::fill(G.begin(), G.end(), 0.0);
        for (int i = 0; i < keep; ++i) G[(size_t)i * m + i] = theta[order[i]];
        j0 = keep;
    }

    // Ritz vectors, energies E = s + 1 / theta, M-normalised, backward errors
    // ||H y - E M y|| / ((||H|| + |E| ||M||) ||y||) with native FP64 applies
    const double nH = op.abs_norm_bound(TDZ_HAMILTONIAN), nM = op.abs_norm_bound(TDZ_MASS);
    res.energies.resize(nev);
    res.berr.resize(nev);
    std::vector<int> idx(order.begin(), order.begin() + nev);
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return shift + 1.0 / theta[a] < shift + 1.0 / theta[b]; });
    for (int i = 0; i < nev; ++i) {
        const int c = idx[i];
        std::vector<cd> sc(m);
        for (int r = 0; r < m; ++r) sc[r] = S[(size_t)r * m + c];
        double2 *y = vecs + (size_t)i * n;
        blas::zero(y, n, TDZ_FP64, st);
        blas::maxpy(y, m, Vp.data(), sc.data(), n, TDZ_FP64, st);
        const double E = shift + 1.0 / theta[c];
        op.apply(TDZ_MASS, TDZ_FP64, y, tmp.ptr, st);
        cd ym;
        const void *yp[1] = {y};
        blas::mdot(red, yp, 1, tmp.ptr, n, TDZ_FP64, &ym, st);
        const double sy = 1.0 / std::sqrt(ym.real());
        blas::scale(y, sy, n, TDZ_FP64, st);
        blas::scale(tmp.ptr, sy, n, TDZ_FP64, st);
        op.apply(TDZ_HAMILTONIAN, TDZ_FP64, y, w.ptr, st);
        blas::axpby(w.ptr, -E, tmp.ptr, 1.0, n, TDZ_FP64, st);   // w = H y - E M y
        const double nr = blas::nrm2(red, w.ptr, n, TDZ_FP64, st), ny = blas::nrm2(red, y, n, TDZ_FP64, st);
        res.energies[i] = E;
        res.berr[i] = nr / std::max((nH + std::abs(E) * nM) * ny, 1e-300);
    }
    res.solves = solves;
    res.restarts = restarts;
    res.inner_its = solver.its;
    return res;
}

}  // namespace tdz
