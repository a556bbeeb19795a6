// Multigrid hierarchy, Galerkin bands and the V-cycle (host orchestration).
#include <algorithm>
#include <cmath>
#include <utility>

#include "mg.h"

namespace tdz {

// ---------------------------------------------------------------- 1D pieces
// The coarsening rule of CoarsenKnots (src/multigrid.cpp:25-40): among the
// distinct breakpoints, numbered from the left end, the odd-numbered interior
// ones of multiplicity one are removed; ends and repeated (C0) breakpoints
// stay with their multiplicity.
std::vector<double> coarsen_knots(const std::vector<double> &U, bool *dropped) {
    std::vector<double> C;
    *dropped = false;
    size_t i = 0;
    int number = 0;                // index of the current distinct breakpoint
    while (i < U.size()) {
        size_t j = i;
        while (j < U.size() && U[j] == U[i]) ++j;   // [i, j): one breakpoint
        const bool end = i == 0 || j == U.size();
        const bool simple = j - i == 1;
        if (!end && simple && number % 2 == 1) *dropped = true;
        else C.insert(C.end(), U.begin() + i, U.begin() + j);
        ++number;
        i = j;
    }
    return C;
}

int count_spans(const std::vector<double> &U) {
    int n = 0;
    for (size_t i = 0; i + 1 < U.size(); ++i)
        if (U[i + 1] > U[i]) ++n;
    return n;
}

// Prolongation from the spline space on knots C to the one on F (C a
// subsequence of F, same degree): the coarse basis functions lie in the fine
// space, so their fine coefficients are exactly the L2 projection
//   P = M_F^-1 G,  M_F = (N^F_i, N^F_k),  G = (N^F_i, N^C_j),
// with both inner products integrated exactly by p+1 Gauss points per fine
// span and M_F solved by a banded Cholesky factorisation. This is the matrix
// that Boehm's knot insertion (the reference's Prolongation,
// src/multigrid.cpp:52-81) builds one knot at a time; entries below 1e-10
// (rounding of exact zeros) are dropped.
RowSparse boehm_prolongation(const std::vector<double> &C, const std::vector<double> &F, int p) {
    const int nf = (int)F.size() - p - 1, nc = (int)C.size() - p - 1;
    const int bw = p;                       // half bandwidth of M_F
    std::vector<double> L((size_t)nf * (bw + 1), 0.0);   // lower band: L[i][d] = M(i, i - d)
    std::vector<double> G((size_t)nf * nc, 0.0);
    std::vector<double> gx, gw;
    gauss_legendre(p + 1, gx, gw);
    std::vector<double> vf(2 * (p + 1)), vc(2 * (p + 1));
    for (int k = p; k < nf; ++k) {
        const double a = F[k], b = F[k + 1];
        if (!(b > a)) continue;
        for (int q = 0; q <= p; ++q) {
            const double x = 0.5 * (a + b) + 0.5 * (b - a) * gx[q], wq = 0.5 * (b - a) * gw[q];
            ders_basis(F, p, k, x, 0, vf.data());
            const int sc = find_span(C, p, nc, x);
            ders_basis(C, p, sc, x, 0, vc.data());
            for (int r = 0; r <= p; ++r) {
                const int i = k - p + r;
                for (int r2 = 0; r2 <= r; ++r2) L[(size_t)i * (bw + 1) + (r - r2)] += wq * vf[r] * vf[r2];
                for (int c = 0; c <= p; ++c) G[(size_t)i * nc + (sc - p + c)] += wq * vf[r] * vc[c];
            }
        }
    }
    // banded Cholesky M_F = L L^T in place
    for (int i = 0; i < nf; ++i) {
        for (int d = std::min(bw, i); d >= 1; --d) {
            const int j = i - d;
            double v = L[(size_t)i * (bw + 1) + d];
            for (int e = 1; e <= bw - d && e <= j; ++e) v -= L[(size_t)i * (bw + 1) + d + e] * L[(size_t)j * (bw + 1) + e];
            L[(size_t)i * (bw + 1) + d] = v / L[(size_t)j * (bw + 1)];
        }
        double v = L[(size_t)i * (bw + 1)];
        for (int d = 1; d <= std::min(bw, i); ++d) v -= L[(size_t)i * (bw + 1) + d] * L[(size_t)i * (bw + 1) + d];
        TDZ_CHECK(v > 0.0, TDZ_ERR_INTERNAL, "fine mass matrix not positive definite");
        L[(size_t)i * (bw + 1)] = std::sqrt(v);
    }
    // P = L^-T L^-1 G, column by column
    std::vector<double> P((size_t)nf * nc);
    std::vector<double> y(nf);
    for (int j = 0; j < nc; ++j) {
        for (int i = 0; i < nf; ++i) {
            double v = G[(size_t)i * nc + j];
            for (int d = 1; d <= std::min(bw, i); ++d) v -= L[(size_t)i * (bw + 1) + d] * y[i - d];
            y[i] = v / L[(size_t)i * (bw + 1)];
        }
        for (int i = nf - 1; i >= 0; --i) {
            double v = y[i];
            for (int d = 1; d <= bw && i + d < nf; ++d) v -= L[(size_t)(i + d) * (bw + 1) + d] * y[i + d];
            y[i] = v / L[(size_t)i * (bw + 1)];
        }
        for (int i = 0; i < nf; ++i) P[(size_t)i * nc + j] = y[i];
    }
    RowSparse R;
    R.rows = nf;
    R.cols = nc;
    std::vector<std::vector<std::pair<int, double>>> rows(nf);
    for (int i = 0; i < nf; ++i) {
        for (int j = 0; j < nc; ++j)
            if (std::abs(P[(size_t)i * nc + j]) >= 1e-10) rows[i].push_back({j, P[(size_t)i * nc + j]});
        R.width = std::max(R.width, (int)rows[i].size());
    }
    R.col.assign((size_t)R.rows * R.width, -1);
    R.val.assign((size_t)R.rows * R.width, 0.0);
    for (int i = 0; i < R.rows; ++i)
        for (size_t t = 0; t < rows[i].size(); ++t) {
            R.col[(size_t)i * R.width + t] = rows[i][t].first;
            R.val[(size_t)i * R.width + t] = rows[i][t].second;
        }
    return R;
}

RowSparse transpose(const RowSparse &P) {
    std::vector<std::vector<std::pair<int, double>>> rows(P.cols);
    for (int i = 0; i < P.rows; ++i)
        for (int t = 0; t < P.width; ++t) {
            const int j = P.col[(size_t)i * P.width + t];
            if (j >= 0) rows[j].push_back({i, P.val[(size_t)i * P.width + t]});
        }
    RowSparse R;
    R.rows = P.cols;
    R.cols = P.rows;
    for (auto &r : rows) R.width = std::max(R.width, (int)r.size());
    R.col.assign((size_t)R.rows * R.width, -1);
    R.val.assign((size_t)R.rows * R.width, 0.0);
    for (int j = 0; j < R.rows; ++j)
        for (size_t t = 0; t < rows[j].size(); ++t) {
            R.col[(size_t)j * R.width + t] = rows[j][t].first;
            R.val[(size_t)j * R.width + t] = rows[j][t].second;
        }
    return R;
}

void RowSparse::upload() {
    tdz::upload(dcol, col);
    tdz::upload(dval64, val);
    std::vector<float> v32(val.begin(), val.end());
    tdz::upload(dval32, v32);
}

BandD galerkin(const RowSparse &P, const BandD &B) {
    const int p = B.p;
    BandD Cb(P.cols, p);
    for (int i = 0; i < P.rows; ++i)
        for (int j = std::max(0, i - p); j <= std::min(P.rows - 1, i + p); ++j) {
            const double bij = B.at(i, j);
            if (bij == 0.0) continue;
            for (int s = 0; s < P.width; ++s) {
                const int k = P.col[(size_t)i * P.width + s];
                if (k < 0) break;
                const double pik = P.val[(size_t)i * P.width + s] * bij;
                for (int t = 0; t < P.width; ++t) {
                    const int l = P.col[(size_t)j * P.width + t];
                    if (l < 0) break;
                    TDZ_CHECK(std::abs(k - l) <= p, TDZ_ERR_INTERNAL, "Galerkin product leaves the band");
                    Cb.at(k, l) += pik * P.val[(size_t)j * P.width + t];
                }
            }
        }
    return Cb;
}

// ---------------------------------------------------------------- hierarchy
void Multigrid::setup(Operator *fine_, const MGOptions &o, cudaStream_t st) {
    fine = fine_;
    opt = o;
    prec = o.precision;
    const Space &fs = *fine->sp;
    const int dim = fs.dim;
    TDZ_CHECK(!fine->wall1d, TDZ_ERR_UNSUPPORTED, "multigrid with Dirichlet walls is not supported");
    const int p = fs.ax[0].p;
    // knot hierarchy, finest first
    std::vector<std::array<std::vector<double>, 3>> K(1);
    for (int d = 0; d < dim; ++d) K[0][d] = fs.ax[d].U;
    const int maxLevels = opt.levels > 0 ? opt.levels : 20;
    while ((int)K.size() < maxLevels) {
        auto C = K.back();
        bool any = false;
        long long dofs = 1;
        for (int d = 0; d < dim; ++d) {
            bool dropped = false;
            auto Cd = coarsen_knots(K.back()[d], &dropped);
            if (dropped && count_spans(Cd) >= p + 1) { C[d] = Cd; any = true; }
            dofs *= (long long)C[d].size() - p - 1;
        }
        if (!any) break;
        K.push_back(C);
        if (opt.levels == 0 && dofs < 2000) break;
    }
    const int L = (int)K.size();
    lv.clear();
    lv.resize(L);
    for (int l = 0; l < L; ++l) {
        MGLevel &m = lv[l];
        if (l == 0) {
            m.space = fs;
            m.opp = fine;
        } else {
            m.space.dim = dim;
            m.space.nquad = fs.nquad;
            for (int d = 0; d < dim; ++d) {
                const auto &U = K[l][d];
                // a level carrying the soft-core term needs the full Gauss rule for its quadrature
                const int nq = fine->quad.on ? fs.nquad : std::max(1, std::min(fs.nquad, 2));
                m.space.ax[d].setup(U.data(), (int)U.size(), p, nq);
            }
            // Galerkin operator from the next finer level
            const Operator &fo = *lv[l - 1].opp;
            auto op = std::make_unique<Operator>();
            op->space = m.space;
            op->sp = &op->space;
            op->phys = fo.phys;
            op->P = p;
            op->terms = fo.terms;
            op->coupled = fo.coupled;
            op->sigma = fo.sigma;
            op->stage_set = true;
            for (int d = 0; d < dim; ++d) {
                m.P[d] = boehm_prolongation(K[l][d], K[l - 1][d], p);
                m.R[d] = transpose(m.P[d]);
                m.P[d].upload();
                m.R[d].upload();
                for (const BandD &b : fo.bases[d]) op->bases[d].push_back(galerkin(m.P[d], b));
            }
            op->upload_bases();
            // the non-separable term is rediscretised on the level (its Galerkin
            // product is not a Kronecker sum)
            if (fo.quad.on) op->quad.build(op->space, fo.quad.nsoft, &fo.quad.soft[0][0]);
            m.opp = op.get();
            m.op = std::move(op);
        }
        for (int d = 0; d < 3; ++d) m.n[d] = d < dim ? m.space.ax[d].n : 1;
        m.ndof = (size_t)m.space.ndof();
        std::array<const BandD *, 3> mb{nullptr, nullptr, nullptr};
        for (int d = 0; d < dim; ++d) mb[d] = &m.opp->bases[d][kM];
        m.minv.setup(mb, dim);
        const size_t es = prec == TDZ_FP64 ? sizeof(double2) : sizeof(float2);
        for (DevBuf *b : {&m.x, &m.b, &m.r, &m.d, &m.z, &m.t1, &m.t2}) b->alloc(m.ndof * es);
    }
    red.init();
    estimate_bounds(st);
    if (opt.learned) learned_setup();
    if (opt.coarse_fdm && !lrn.on) {
        MGLevel &c = lv.back();
        const int P = c.space.ax[0].p;
        if (c.space.dim >= 2 && P >= 2 && P <= 5 && c.space.ax[1].p == P && (c.space.dim < 3 || c.space.ax[2].p == P)) {
            c.opp->sigma = fine->sigma;
            cfdm = std::make_unique<PcFDM>();
            cfdm->setup(c.opp, prec);
            cb64.alloc(c.ndof * sizeof(double2));
            cx64.alloc(c.ndof * sizeof(double2));
        }
    }
}

namespace {
// deterministic pseudo-random start vector for the power iterations
void fill_start(DevBuf &v, size_t n, int prec, cudaStream_t st) {
    std::vector<double> h(2 * n);
    uint64_t s = 0x9e3779b97f4a7c15ull;
    for (size_t i = 0; i < 2 * n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        h[i] = (double)(s >> 11) / (double)(1ull << 53) - 0.5;
    }
    if (prec == TDZ_FP64) TDZ_CUDA(cudaMemcpyAsync(v.ptr, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st));
    else {
        std::vector<float> f(h.begin(), h.end());
        TDZ_CUDA(cudaMemcpyAsync(v.ptr, f.data(), f.size() * 4, cudaMemcpyHostToDevice, st));
    }
    TDZ_CUDA(cudaStreamSynchronize(st));
}
}  // namespace

void Multigrid::estimate_bounds(cudaStream_t st) {
    // field coefficients of the current stage: sigma[2+k] = g c_k
    const std::array<cd, 5> sg = fine->sigma;
    std::vector<cd> c;
    for (size_t k = 0; k < fine->coupled.size(); ++k)
        c.push_back(std::abs(sg[1]) > 0 ? sg[2 + k] / sg[1] : cd(0));
    for (auto &m : lv) {
        Operator &op = *m.opp;
        const auto saved = op.sigma;
        op.set_stage(0.0, 1.0, c);          // H_E
        fill_start(m.x, m.ndof, prec, st);
        double lam = 0.0;
        // largest eigenvalue of M^-1 H_E
        for (int it = 0; it < 40; ++it) {
            op.apply(TDZ_STAGE, prec, m.x.ptr, m.t1.ptr, st);
            m.minv.apply(m.t1.ptr, prec, st);
            const double nx = blas::nrm2(red, m.x.ptr, m.ndof, prec, st);
            const double nt = blas::nrm2(red, m.t1.ptr, m.ndof, prec, st);
            lam = nt / std::max(nx, 1e-300);
            blas::axpby(m.x.ptr, cd(1.0 / std::max(nt, 1e-300)), m.t1.ptr, 0.0, m.ndof, prec, st);
        }
        m.mu_hi = 1.05 * lam;
        // lowest: largest eigenvalue of mu_hi - M^-1 H_E
        fill_start(m.x, m.ndof, prec, st);
        double lam2 = 0.0;
        for (int it = 0; it < 40; ++it) {
            op.apply(TDZ_STAGE, prec, m.x.ptr, m.t1.ptr, st);
            m.minv.apply(m.t1.ptr, prec, st);
            blas::axpby(m.t1.ptr, cd(m.mu_hi), m.x.ptr, -1.0, m.ndof, prec, st);
            const double nx = blas::nrm2(red, m.x.ptr, m.ndof, prec, st);
            const double nt = blas::nrm2(red, m.t1.ptr, m.ndof, prec, st);
            lam2 = nt / std::max(nx, 1e-300);
            blas::axpby(m.x.ptr, cd(1.0 / std::max(nt, 1e-300)), m.t1.ptr, 0.0, m.ndof, prec, st);
        }
        m.mu_lo = m.mu_hi - 1.05 * lam2;
        m.w_max = fine->cap_bound;
        op.sigma = saved;
    }
}

void Multigrid::refresh() {}

// Chebyshev iteration on A x = b with M^-1. The eigenvalues of M^-1 A are
// alpha + g mu with mu = mu_r - i mu_i, mu_r in [mu_a, mu_b] (Hermitian part)
// and mu_i in [0, w] (CAP). The iteration uses the ellipse that encloses this
// rectangle (semi-axes sqrt2 times its half-sides; the segment itself when
// w = 0): center theta and focal half-distance delta in the lambda-plane.
// x_zero: x starts at 0.
void chebyshev(MGLevel &m, int prec, double mu_a, double mu_b, double w, int steps, bool x_zero, cudaStream_t st) {
    Operator &op = *m.opp;
    const cd alpha = op.sigma[0], g = op.sigma[1];
    const cd center = cd(0.5 * (mu_a + mu_b), -0.5 * w);
    cd focal;
    if (w <= 0.0) focal = cd(0.5 * (mu_b - mu_a), 0.0);
    else {
        const double a = std::sqrt(2.0) * 0.5 * (mu_b - mu_a), b = std::sqrt(2.0) * 0.5 * w;
        focal = a >= b ? cd(std::sqrt(a * a - b * b), 0.0) : cd(0.0, -std::sqrt(b * b - a * a));
    }
    const cd theta = alpha + g * center;
    const cd delta = g * focal;
    const size_t n = m.ndof;
    // r = b - A x
    if (x_zero) blas::copy(m.b.ptr, m.r.ptr, n, prec, st);
    else {
        op.apply(TDZ_STAGE, prec, m.x.ptr, m.t1.ptr, st);
        blas::axpbypcz(m.r.ptr, 1.0, m.b.ptr, 0.0, m.t1.ptr, -1.0, n, prec, st);
    }
    if (std::abs(delta) <= 1e-12 * std::abs(theta)) {
        // degenerate segment: damped Richardson x += M^-1 r / theta
        blas::copy(m.r.ptr, m.z.ptr, n, prec, st);
        m.minv.apply(m.z.ptr, prec, st);
        if (x_zero) blas::axpby(m.x.ptr, 1.0 / theta, m.z.ptr, 0.0, n, prec, st);
        else blas::axpby(m.x.ptr, 1.0 / theta, m.z.ptr, 1.0, n, prec, st);
        return;
    }
    const cd sigma1 = theta / delta;
    cd rho = 1.0 / sigma1;
    blas::copy(m.r.ptr, m.z.ptr, n, prec, st);
    m.minv.apply(m.z.ptr, prec, st);
    blas::axpby(m.d.ptr, 1.0 / theta, m.z.ptr, 0.0, n, prec, st);
    if (x_zero) blas::copy(m.d.ptr, m.x.ptr, n, prec, st);
    else blas::axpby(m.x.ptr, 1.0, m.d.ptr, 1.0, n, prec, st);
    for (int k = 1; k < steps; ++k) {
        op.apply(TDZ_STAGE, prec, m.d.ptr, m.t1.ptr, st);
        blas::axpby(m.r.ptr, -1.0, m.t1.ptr, 1.0, n, prec, st);
        blas::copy(m.r.ptr, m.z.ptr, n, prec, st);
        m.minv.apply(m.z.ptr, prec, st);
        const cd rn = 1.0 / (2.0 * sigma1 - rho);
        blas::axpby(m.d.ptr, 2.0 * rn / delta, m.z.ptr, rn * rho, n, prec, st);
        blas::axpby(m.x.ptr, 1.0, m.d.ptr, 1.0, n, prec, st);
        rho = rn;
    }
}


void Multigrid::vcycle(int l, cudaStream_t st) {
    MGLevel &m = lv[l];
    const int last = (int)lv.size() - 1;
    if (l == last) {
        if (lrn.on && lrn.rec_n < lrn.rec_cap) {   // a training input from this run
            blas::copy(m.b.ptr, lrn.rec.as<float2>() + (size_t)lrn.rec_n * m.ndof, m.ndof, TDZ_FP32, st);
            ++lrn.rec_n;
        }
        if (cfdm && !lrn.on && cfdm->exact_now()) {
            // the exact fast-diagonalisation inverse of the coarsest operator
            blas::cast(m.b.ptr, prec, cb64.ptr, TDZ_FP64, m.ndof, st);
            cfdm->apply(cb64.as<double2>(), cx64.as<double2>(), st);
            blas::cast(cx64.ptr, TDZ_FP64, m.x.ptr, prec, m.ndof, st);
            ++coarse_exact;
            return;
        }
        chebyshev(m, prec, m.mu_lo, m.mu_hi, m.w_max, opt.coarse_its, true, st);
        if (lrn.on && lrn.trained) coarse_correct(m, st);
        return;
    }
    const double lo = m.mu_hi / opt.ratio;
    chebyshev(m, prec, lo, m.mu_hi, m.w_max, opt.smooth, true, st);
    // r = b - A x
    m.opp->apply(TDZ_STAGE, prec, m.x.ptr, m.t1.ptr, st);
    blas::axpbypcz(m.r.ptr, 1.0, m.b.ptr, 0.0, m.t1.ptr, -1.0, m.ndof, prec, st);
    // restrict: axis 2, then 1, then 0 (shrinking early)
    MGLevel &c = lv[l + 1];
    const int dim = m.space.dim;
    int sh[3] = {m.n[0], m.n[1], m.n[2]};
    const void *src = m.r.ptr;
    void *tmp[2] = {m.t1.ptr, m.t2.ptr};
    int ti = 0;
    for (int d = dim - 1; d >= 0; --d) {
        void *dst = d == 0 ? c.b.ptr : tmp[ti];
        axis_contract(c.R[d], d, src, dst, sh[0], sh[1], sh[2], false, prec, st);
        sh[d] = c.n[d];
        src = dst;
        ti ^= 1;
    }
    vcycle(l + 1, st);
    // prolongate and add: axis 0, 1, 2 (growing late)
    int s2[3] = {c.n[0], c.n[1], c.n[2]};
    src = c.x.ptr;
    ti = 0;
    for (int d = 0; d < dim; ++d) {
        const bool lastp = d == dim - 1;
        void *dst = lastp ? m.x.ptr : tmp[ti];
        axis_contract(c.P[d], d, src, dst, s2[0], s2[1], s2[2], lastp, prec, st);
        s2[d] = m.n[d];
        src = dst;
        ti ^= 1;
    }
    chebyshev(m, prec, lo, m.mu_hi, m.w_max, opt.smooth, false, st);
}

void Multigrid::apply(const double2 *r, double2 *z, cudaStream_t st) {
    // coarse levels follow the current stage scalars of the fine operator
    for (size_t l = 1; l < lv.size(); ++l) lv[l].opp->sigma = fine->sigma;
    MGLevel &f = lv[0];
    blas::cast(r, TDZ_FP64, f.b.ptr, prec, f.ndof, st);
    vcycle(0, st);
    blas::cast(f.x.ptr, prec, z, TDZ_FP64, f.ndof, st);
    ++cycles;
}

}  // namespace tdz
