// t-SURFF end term on the device: the flux that still crosses the surface
// after the last sample time T, when the field is over (TDSEZTSurff::EndTerm,
// src/tsurff.cpp:650-976).
//
// After T the Volkov state only gains the phase exp(-i E_k (t - T)),
// E_k = |k + A(T)|^2 / 2m + V0, and psi evolves under the field-free H with
// its absorbing layer, so
//     int_T^inf dt flux_k(t) = flux_k(T)[phi_{E_k}],
//     phi_E = int_0^inf exp(i E s) psi(T + s) ds,   (E M - H) phi_E = i M psi(T),
// the absorber being the outgoing-wave condition. phi_E is solved at energy
// nodes uniform in p = |k + A(T)| and the node fluxes are combined with
// four-point Lagrange weights in p for every momentum.
//
// The reference runs a multi-shift Arnoldi on LU-factorised (or ASM/GMRES)
// poles. Here every node is its own FGMRES solve on the device, warm-started
// from the previous node's solution, with the library's preconditioners:
// the exact banded LU in 1D, the fast-diagonalisation inverse in 2D/3D
// (exact for a separable H: its absorbing layers enter through complex
// symmetric axis pencils). When that inverse is not exact (a non-separable
// potential), it is built for the damped pole E (1 + i eta) (the
// shifted-Laplacian rule the reference uses for its 3D poles) while FGMRES
// solves the undamped system; so is a node at which the exact FP32 inverse
// stagnates (a weakly absorbed box mode next to E: the FP32 inverse of a
// nearly singular stage has no correct digits left).
// The flux of a node is added to the momenta that use it as soon as it is
// solved, so no node solution is kept.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>

#include "band.h"
#include "fdm.h"
#include "prop.h"
#include "tsurff.h"
#include "tsurff_nodes.h"

namespace tdz {


EndTermStats TSurff::end_term(Operator &op, const SolverOptions &so_in, const EndTermOptions &eo, const double2 *psi,
                              std::vector<cd> &out, cudaStream_t st) {
    const auto t_start = std::chrono::steady_clock::now();
    TDZ_CHECK(have_prev, TDZ_ERR_STATE, "the end term needs psi(T) sampled first (the last sample time is T)");
    const Space &s = *op.sp;
    TDZ_CHECK(s.dim == dim, TDZ_ERR_ARG, "operator and t-SURFF spaces differ");
    for (int d = 0; d < dim; ++d) TDZ_CHECK(s.ax[d].n == n[d], TDZ_ERR_ARG, "operator and t-SURFF spaces differ");
    TDZ_CHECK(op.cap_bound > 0.0, TDZ_ERR_ARG,
              "the end term needs the absorbing layer in the operator (it is the outgoing-wave condition)");
    TDZ_CHECK(eo.dp >= 0.0, TDZ_ERR_ARG, "end-term node spacing must be >= 0 (0 = automatic)");
    TDZ_CHECK(eo.dp > 0.0 || eo.cap_width > 0.0, TDZ_ERR_ARG,
              "automatic end-term node spacing needs the width of the absorbing layer");
    const double T = vt;
    // the evolution after T must be field-free
    if (field) {
        double emax = 0.0, eafter = 0.0;
        for (int d = 0; d < dim; ++d)
            for (int j = 0; j <= 200; ++j) {
                emax = std::max(emax, std::abs(field(d, T * j / 200.0, field_ctx)));
                eafter = std::max(eafter, std::abs(field(d, T + j * 0.5 * dt, field_ctx)));
            }
        TDZ_CHECK(eafter <= 1e-8 * std::max(emax, 1e-300), TDZ_ERR_ARG,
                  "t-SURFF end term: the field is not over at the final time (|E| = " + std::to_string(eafter) +
                      " after T, " + std::to_string(emax) + " during the run); end the run after the pulse");
    }

    // kinetic momenta p_q = |k_q + A(T)|, k_x slowest
    std::vector<double> pk(nktot);
    {
        size_t q = 0;
        for (int i = 0; i < nk[0]; ++i)
            for (int j = 0; j < nk[1]; ++j)
                for (int l = 0; l < nk[2]; ++l, ++q) {
                    const double kv[3] = {k[0][i] + A[0], k[1][j] + A[1], k[2][l] + A[2]};
                    pk[q] = std::sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
                }
    }
    const double pmin = *std::min_element(pk.begin(), pk.end()), pmax = *std::max_element(pk.begin(), pk.end());
    double dk_grid = std::numeric_limits<double>::max();
    for (int d = 0; d < dim; ++d)
        if (nk[d] > 1) dk_grid = std::min(dk_grid, (k[d].back() - k[d].front()) / (nk[d] - 1));
    double L = 0.0;   // largest box half-width
    for (int d = 0; d < dim; ++d) L = std::max({L, std::abs(s.ax[d].U.front()), std::abs(s.ax[d].U.back())});
    const double sd = std::sqrt((double)dim);
    const double kcap = eo.cap_width > 0.0 ? 6.555 / eo.cap_width : 0.0;
    const double dp_out = eo.dp > 0.0 ? eo.dp : std::min(dk_grid, 0.25 / (R * sd));
    const double dp_in = eo.dp > 0.0 ? eo.dp : std::min(dp_out, 0.25 / (L * sd));
    const double split = std::min(std::max(2.0 * kcap, pmin), pmax);
    const std::vector<double> node = energy_nodes(pmin, pmax, split, dp_in, dp_out);
    const int nn = (int)node.size();

    // momentum -> four-point Lagrange weights in p on the nodes around p_q,
    // regrouped by node (CSR); one node: weight 1
    std::vector<std::vector<std::pair<int, double>>> per(nn);
    for (size_t q = 0; q < nktot; ++q) {
        double w[4];
        const int j0 = lagrange_weights(node, pk[q], w);
        for (int a = 0; a < std::min(nn, 4); ++a) per[j0 + a].push_back({(int)q, w[a]});
    }
    std::vector<int> start(nn + 1, 0), hq;
    std::vector<double> hw;
    for (int j = 0; j < nn; ++j) {
        for (const auto &e : per[j]) { hq.push_back(e.first); hw.push_back(e.second); }
        start[j + 1] = (int)hq.size();
    }
    upload(eq, hq);
    upload(ew, hw);
    if (amp_end.bytes < nktot * sizeof(double2)) amp_end.alloc(nktot * sizeof(double2));
    TDZ_CUDA(cudaMemsetAsync(amp_end.ptr, 0, nktot * sizeof(double2), st));

    // right-hand side i M psi(T)
    const size_t N = (size_t)s.ndof();
    DevBuf b(N * sizeof(double2)), x(N * sizeof(double2));
    op.apply(TDZ_MASS, TDZ_FP64, psi, b.ptr, st);
    blas::scale(b.ptr, cd(0.0, 1.0), N, TDZ_FP64, st);
    blas::zero(x.ptr, N, TDZ_FP64, st);

    const std::vector<cd> no_field(op.coupled.size(), cd(0.0));
    auto energy = [&](int j) { return node[j] * node[j] / (2.0 * mass) + V0; };
    op.set_stage(cd(energy(0), 0.0), cd(-1.0, 0.0), no_field);
    SolverOptions so = so_in;
    so.rtol = eo.rtol > 0.0 ? eo.rtol : 1e-10;
    so.maxit = eo.maxit > 0 ? eo.maxit : 600;
    Solver sol;
    sol.setup(&op, so, st);
    auto *fdm = so.pc == TDZ_PC_FDM ? static_cast<PcFDM *>(sol.pc.get()) : nullptr;
    auto *band = so.pc == TDZ_PC_BAND ? static_cast<PcBand *>(sol.pc.get()) : nullptr;
    // pole damping: none for an exact inverse, 0.5 otherwise; with an exact
    // FP32 inverse a node whose stage is nearly singular (a weakly absorbed
    // box mode close to E) makes FGMRES stagnate, and that node is finished
    // with the damped pole instead
    const bool eta_auto = eo.eta < 0.0;
    const bool exact_pc = (fdm && fdm->exact_now()) || (band && band->exact);
    const double eta_base = eta_auto ? (exact_pc ? 0.0 : 0.5) : eo.eta;
    const int maxit = so.maxit, first_its = 60;

    EndTermStats stats;
    stats.nodes = nn;
    stats.eta = eta_base;
    for (int j = 0; j + 1 < nn; ++j) stats.dp_max = std::max(stats.dp_max, node[j + 1] - node[j]);
    for (int j = 0; j < nn; ++j) {
        const double E = energy(j);
        auto prepare = [&](double eta) {
            const cd pole(E, eta * std::max(E, 1e-3));
            if (band) {
                // factor the pole, then solve the undamped system with it
                op.set_stage(pole, cd(-1.0, 0.0), no_field);
                band->factor(st);
            }
            op.set_stage(cd(E, 0.0), cd(-1.0, 0.0), no_field);
            if (fdm) {
                fdm->pole = eta > 0.0;
                fdm->pole_sigma = op.sigma;
                fdm->pole_sigma[0] = pole;
            }
        };
        const bool retry = eta_auto && eta_base == 0.0;
        prepare(eta_base);
        sol.opt.maxit = retry ? std::min(first_its, maxit) : maxit;
        SolveStats ss = sol.solve(b.as<double2>(), x.as<double2>(), st);
        int its = ss.its;
        if (ss.reason <= 0 && retry) {
            if (ss.reason == -9) blas::zero(x.ptr, N, TDZ_FP64, st);
            prepare(0.5);
            sol.opt.maxit = std::max(1, maxit - its);
            ss = sol.solve(b.as<double2>(), x.as<double2>(), st);
            its += ss.its;
            ++stats.damped;
        }
        TDZ_CHECK(ss.reason > 0, TDZ_ERR_NOT_CONVERGED,
                  "t-SURFF end term: the solve at E = " + std::to_string(E) + " did not converge (reason " +
                      std::to_string(ss.reason) + ", " + std::to_string(its) + " iterations)");
        stats.its += its;
        stats.max_its = std::max(stats.max_its, its);
        add_weighted_flux(x.as<double2>(), eq.as<int>() + start[j], ew.as<double>() + start[j],
                          start[j + 1] - start[j], st);
    }
    if (fdm) fdm->pole = false;

    std::vector<double2> h(nktot);
    TDZ_CUDA(cudaMemcpyAsync(h.data(), amp_end.ptr, nktot * sizeof(double2), cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    out.resize(nktot);
    for (size_t q = 0; q < nktot; ++q) out[q] = cd(h[q].x, h[q].y);
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    return stats;
}

}  // namespace tdz
