// Matrix-free operator set: base 1D bands, Kronecker terms and compiled apply
// plans.
//
// Term structure (the operators of TDSEZFormHam, src/assembly/assembly.cpp:703-864,
// the CAP of src/assembly/cap.cpp:40-144 and the dipoles of
// src/tensorops.cpp:40-57, all sums of Kronecker products of 1D bands):
//   M      = M_z (x) M_y (x) M_x
//   K      = 1/2 sum_a  S_a (x) M (x) M            constant mass (times 1/m)
//          = 1/2 sum_a  S_a (x) Mm_l (x) M         mass layered along axis l != a
//          + 1/2        Sm_l (x) M (x) M           (Mm = int B B / m, Sm = int B'B' / m)
//   s V    = s sum_d V_d (x) M (x) M               V = sum_d V_d(x_d)
//   CAP    = -i/m sum_d W_d (x) M (x) M
//   D_a    = X_a (x) M (x) M
// The stage operator A = alpha M + g (H + sum_a c_a D_a) keeps this term list
// with coefficients factor * sigma[scalar], sigma = (alpha, g, g c_0, ...):
// changing the stage changes only scalars, never a band.
#include "oper.h"

#include "blas.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>

namespace tdz {

void Comb::add(int b, int s, cd f) {
    for (int i = 0; i < n; ++i)
        if (base[i] == b && scalar[i] == s) { factor[i] += f; return; }
    TDZ_CHECK(n < kMaxComb, TDZ_ERR_UNSUPPORTED, "too many bands in one combination");
    base[n] = b;
    scalar[n] = s;
    factor[n] = f;
    ++n;
}

int Operator::add_band(int axis, BandD b) {
    bases[axis].push_back(std::move(b));
    return (int)bases[axis].size() - 1;
}

void Operator::build(const Space &s, const tdz_physics &ph) {
    space = s;
    sp = &space;
    phys = ph;
    const int dim = s.dim;
    P = s.ax[0].p;
    for (int d = 1; d < dim; ++d)
        TDZ_CHECK(s.ax[d].p == P || dim == 1, TDZ_ERR_UNSUPPORTED, "all axes must have the same degree");
    TDZ_CHECK(ph.mass_axis < dim, TDZ_ERR_ARG, "mass_axis out of range");
    TDZ_CHECK(!ph.dirichlet || dim == 1, TDZ_ERR_UNSUPPORTED, "Dirichlet walls are supported in 1D only");
    for (int d = 0; d < dim; ++d) {
        const Axis1D &a = s.ax[d];
        add_band(d, a.band(nullptr, 0, 0));   // kM
        add_band(d, a.band(nullptr, 1, 1));   // kS
        add_band(d, a.band_x());              // kX
    }
    const double sgn = -ph.charge;
    auto base_bands = [&]() { return std::array<int, 3>{kM, kM, kM}; };
    terms.clear();
    // mass
    terms.push_back({0, cd(1.0), base_bands()});
    // kinetic
    if (ph.mass_axis < 0) {
        TDZ_CHECK(std::isfinite(ph.inv_mass), TDZ_ERR_ARG, "inv_mass must be finite");
        for (int a = 0; a < dim; ++a) {
            auto b = base_bands();
            b[a] = kS;
            terms.push_back({1, cd(0.5 * ph.inv_mass), b});
        }
    } else {
        TDZ_CHECK(ph.inv_mass_q != nullptr, TDZ_ERR_ARG, "inv_mass_q required for a layered mass");
        const int l = ph.mass_axis;
        const int mm = add_band(l, s.ax[l].band(ph.inv_mass_q, 0, 0));
        const int sm = add_band(l, s.ax[l].band(ph.inv_mass_q, 1, 1));
        for (int a = 0; a < dim; ++a) {
            auto b = base_bands();
            if (a == l) b[a] = sm;
            else { b[a] = kS; b[l] = mm; }
            terms.push_back({1, cd(0.5), b});
        }
    }
    // potential
    for (int d = 0; d < dim; ++d)
        if (ph.pot_q[d]) {
            auto b = base_bands();
            b[d] = add_band(d, s.ax[d].band(ph.pot_q[d], 0, 0));
            terms.push_back({1, cd(sgn), b});
        }
    // CAP; its Rayleigh quotient against M is bounded by the largest profile value
    cap_bound = 0.0;
    for (int d = 0; d < dim; ++d)
        if (ph.cap_q[d]) {
            double mx = 0.0;
            for (size_t k = 0; k < s.ax[d].xq.size(); ++k) mx = std::max(mx, std::abs(ph.cap_q[d][k]));
            cap_bound += mx * std::abs(ph.cap_inv_mass);
        }
    for (int d = 0; d < dim; ++d)
        if (ph.cap_q[d]) {
            auto b = base_bands();
            b[d] = add_band(d, s.ax[d].band(ph.cap_q[d], 0, 0));
            terms.push_back({1, cd(0.0, -ph.cap_inv_mass), b});
        }
    // field terms, coupled axes in order
    coupled.clear();
    for (int a = 0; a < dim; ++a)
        if (ph.coupled[a]) {
            auto b = base_bands();
            b[a] = kX;
            terms.push_back({2 + (int)coupled.size(), cd(1.0), b});
            coupled.push_back(a);
        }
    // 1D homogeneous Dirichlet walls: element rule of TDSEZCompOperatorsDirichlet
    // (src/assembly/assembly.cpp:589-632)
    wall1d = false;
    if (ph.dirichlet) {
        wall1d = true;
        const Axis1D &a = s.ax[0];
        const int np = a.p + 1;
        for (int side = 0; side < 2; ++side) {
            const int e = side == 0 ? 0 : a.nel - 1;
            const int wall = side == 0 ? 0 : a.n - 1;
            double mD = 0.0, ratio = 1.0;
            for (int r = 0; r < np; ++r) {
                const int gidx = a.offset[e] + r;
                if (gidx == 0 || gidx == a.n - 1) continue;
                double haa = 0.0, maa = 0.0;
                for (int q = 0; q < a.nq; ++q) {
                    const size_t k = (size_t)e * a.nq + q;
                    const double w = a.wq[k], nv = a.N[k * np + r], dv = a.dN[k * np + r];
                    const double minv = ph.mass_axis < 0 ? ph.inv_mass : ph.inv_mass_q[k];
                    const double v = ph.pot_q[0] ? ph.pot_q[0][k] : 0.0;
                    haa += w * (0.5 * minv * dv * dv + sgn * v * nv * nv);
                    maa += w * nv * nv;
                }
                if (maa > 0.0) { mD = std::max(mD, maa); ratio = std::max(ratio, std::abs(haa) / maa); }
            }
            if (mD <= 0.0) mD = 1.0;
            const int slot = wall == 0 ? 0 : 1;
            h_wall[slot] += ratio * mD;
            m_wall[slot] += mD;
        }
    }
    // non-separable soft-core centres: per-element quadrature term of H
    quad.build(s, ph.nsoft, ph.soft);
    phys.soft = nullptr;   // the caller's array is not kept
    sigma = {cd(1.0), cd(0.0), cd(0.0), cd(0.0), cd(0.0)};
    upload_bases();
}

std::vector<Term> Operator::terms_for(int which) const {
    std::vector<Term> out;
    switch (which) {
    case TDZ_MASS:
        for (const Term &t : terms) if (t.scalar == 0) out.push_back(t);
        break;
    case TDZ_HAMILTONIAN:
        for (const Term &t : terms) if (t.scalar == 1) out.push_back(t);
        break;
    case TDZ_DIPOLE_X: case TDZ_DIPOLE_Y: case TDZ_DIPOLE_Z: {
        const int a = which - TDZ_DIPOLE_X;
        TDZ_CHECK(a < sp->dim, TDZ_ERR_ARG, "dipole axis beyond the dimension");
        std::array<int, 3> b{kM, kM, kM};
        b[a] = kX;
        out.push_back({0, cd(1.0), b});
        break;
    }
    case TDZ_STAGE:
        out = terms;
        break;
    default:
        throw Error(TDZ_ERR_ARG, "unknown operator id");
    }
    return out;
}

double Operator::abs_norm_bound(int which) const {
    const std::array<cd, 5> sg = sigma_for(which);
    double total = 0.0;
    for (const Term &t : terms_for(which)) {
        double f = std::abs(t.factor * sg[t.scalar]);
        if (f == 0.0) continue;
        for (int d = 0; d < sp->dim; ++d) {
            const BandD &b = bases[d][t.band[d]];
            double mx = 0.0;
            for (int i = 0; i < b.n; ++i) {
                double rs = 0.0;
                for (int o = 0; o < b.bw(); ++o) rs += std::abs(b.v[(size_t)i * b.bw() + o]);
                mx = std::max(mx, rs);
            }
            f *= mx;
        }
        total += f;
    }
    return total;
}

std::array<cd, 5> Operator::sigma_for(int which) const {
    if (which == TDZ_STAGE) return sigma;
    std::array<cd, 5> s{cd(0), cd(0), cd(0), cd(0), cd(0)};
    if (which == TDZ_HAMILTONIAN) s[1] = 1.0; else s[0] = 1.0;
    return s;
}

void Operator::upload_bases() {
    for (int d = 0; d < sp->dim; ++d) {
        std::vector<double> v64;
        std::vector<float> v32, vdf;   // vdf: (hi, lo) pairs, hi + lo = v to about 48 bits
        for (const BandD &b : bases[d])
            for (double v : b.v) {
                v64.push_back(v);
                v32.push_back((float)v);
                vdf.push_back((float)v);
                vdf.push_back((float)(v - (double)(float)v));
            }
        upload(dev64[d], v64);
        upload(dev32[d], v32);
        upload(devdf[d], vdf);
    }
}

void Operator::compile(Plan &pl, const std::vector<Term> &ts) const {
    const int dim = sp->dim;
    const int outer = dim - 1;
    pl.dim = dim;
    pl.xT = pl.yT = pl.zA = pl.zC = Comb{};
    pl.hasA = pl.hasB = pl.hasC = false;
    bool c_set = false;
    cd c_factor = 0;
    int c_scalar = -1, c_base = -1;
    for (const Term &t : ts) {
        if (dim == 1) { pl.zA.add(t.band[0], t.scalar, t.factor); continue; }
        int nonM = 0, axis = -1;
        for (int d = 0; d < dim; ++d)
            if (t.band[d] != kM) { ++nonM; axis = d; }
        if (nonM == 0) { pl.zA.add(kM, t.scalar, t.factor); continue; }
        if (nonM == 1) {
            if (axis == outer) pl.zA.add(t.band[outer], t.scalar, t.factor);
            else if (axis == 0) pl.xT.add(t.band[0], t.scalar, t.factor);
            else pl.yT.add(t.band[1], t.scalar, t.factor);
            continue;
        }
        // layered-mass kinetic term: S on one inner axis, Mm on the outer axis
        TDZ_CHECK(nonM == 2 && t.band[outer] != kM, TDZ_ERR_UNSUPPORTED,
                  "term structure not supported (mass must be layered along the last axis)");
        bool inner_ok = false;
        for (int d = 0; d < outer; ++d)
            if (t.band[d] == kS) inner_ok = true;
        TDZ_CHECK(inner_ok, TDZ_ERR_UNSUPPORTED, "layered term must carry S on an inner axis");
        if (!c_set) { c_set = true; c_factor = t.factor; c_scalar = t.scalar; c_base = t.band[outer]; }
        TDZ_CHECK(c_factor == t.factor && c_scalar == t.scalar && c_base == t.band[outer], TDZ_ERR_UNSUPPORTED,
                  "layered kinetic terms must share one outer band and coefficient");
    }
    if (c_set) { pl.zC.add(c_base, c_scalar, c_factor); pl.hasC = true; }
    pl.hasA = pl.zA.n > 0;
    pl.hasB = pl.xT.n > 0 || pl.yT.n > 0;
}

Plan &Operator::plan(int which) {
    auto it = plans.find(which);
    if (it != plans.end()) return *it->second;
    auto pl = std::make_unique<Plan>();
    pl->which = which;
    compile(*pl, terms_for(which));
    if (wall1d) {
        pl->walls = true;
        if (which == TDZ_MASS || which == TDZ_STAGE) pl->wall_m = 0;
        if (which == TDZ_HAMILTONIAN || which == TDZ_STAGE) pl->wall_h = 1;
    }
    Plan &ref = *pl;
    plans[which] = std::move(pl);
    return ref;
}

void Operator::set_stage(cd alpha, cd g, const std::vector<cd> &c) {
    TDZ_CHECK(c.size() == coupled.size(), TDZ_ERR_ARG,
              "number of field coefficients must equal the number of coupled axes");
    sigma = {alpha, g, cd(0), cd(0), cd(0)};
    for (size_t k = 0; k < c.size(); ++k) sigma[2 + k] = g * c[k];
    stage_set = true;
}

void Operator::apply(int which, int prec, const void *x, void *y, cudaStream_t st) { residual(which, prec, x, nullptr, y, st); }

bool Operator::fused_reductions() const { return sp->dim == 3 && !quad.on; }

namespace {
// one fused-reduction result to the host (synchronises the stream)
cd take_reduction(Operator &op, cudaStream_t st) {
    apply_red_finish(op.red_part.as<double2>(), op.red_res.as<double2>(), st);
    double2 v;
    TDZ_CUDA(cudaMemcpyAsync(&v, op.red_res.ptr, sizeof(double2), cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    return cd(v.x, v.y);
}
void ensure_red(Operator &op) {
    if (op.red_part.ptr) return;
    op.red_part.alloc(sizeof(double2) * kApplyRedCap);
    op.red_res.alloc(sizeof(double2));
}
}  // namespace

void Operator::residual(int which, int prec, const void *x, const void *b, void *y, cudaStream_t st, double *norm) {
    TDZ_CHECK(prec == TDZ_FP32 || prec == TDZ_FP64 || prec == TDZ_FP64_DF || (prec == kPrecF32M64 && f32_on_f64()),
              TDZ_ERR_ARG, "precision must be TDZ_FP32, TDZ_FP64, TDZ_FP64_DF or (3D, no soft-core term) TDZ_FP64_F32");
    TDZ_CHECK(x && y, TDZ_ERR_ARG, "null vector");
    TDZ_CHECK(x != y, TDZ_ERR_ARG, "x and y must not alias");
    if (which == TDZ_STAGE) TDZ_CHECK(stage_set, TDZ_ERR_STATE, "stage coefficients not set");
    Plan &pl = plan(which);
    ApplyExtra ex;
    ex.sub = b;
    const bool fused = norm && fused_reductions();
    if (fused) {
        ensure_red(*this);
        TDZ_CUDA(cudaMemsetAsync(red_part.ptr, 0, sizeof(double2) * kApplyRedCap, st));
        ex.red = red_part.as<double2>();
        ex.red_mode = 1;
    }
    launch_apply(*this, pl, prec, x, y, st, ex);
    if (quad.on && (which == TDZ_HAMILTONIAN || which == TDZ_STAGE)) {
        // y += s (g for the stage) V_q x; minus that for a residual
        const cd coef = -phys.charge * (which == TDZ_STAGE ? sigma[1] : cd(1.0));
        quad.apply(b ? -coef : coef, prec, x, y, st);
    }
    ++launches;
    if (norm) {
        if (fused) {
            const double v = take_reduction(*this, st).real();
            *norm = std::isfinite(v) ? std::sqrt(std::max(0.0, v)) : std::numeric_limits<double>::quiet_NaN();
        } else {
            *norm = blas::nrm2(red, y, (size_t)sp->ndof(), prec == TDZ_FP32 ? TDZ_FP32 : TDZ_FP64, st);
        }
    }
}

void Operator::apply_dot(int which, int prec, const void *x, void *y, const void *v, cd *dot, cudaStream_t st) {
    TDZ_CHECK(prec == TDZ_FP64 || prec == TDZ_FP64_DF || prec == kPrecF32M64, TDZ_ERR_ARG,
              "apply_dot works on FP64 vectors");
    if (!fused_reductions()) {
        apply(which, prec, x, y, st);
        const void *V[1] = {v};
        blas::mdot(red, V, 1, y, (size_t)sp->ndof(), TDZ_FP64, dot, st);
        return;
    }
    TDZ_CHECK(x && y && v, TDZ_ERR_ARG, "null vector");
    TDZ_CHECK(x != y, TDZ_ERR_ARG, "x and y must not alias");
    if (which == TDZ_STAGE) TDZ_CHECK(stage_set, TDZ_ERR_STATE, "stage coefficients not set");
    Plan &pl = plan(which);
    ensure_red(*this);
    TDZ_CUDA(cudaMemsetAsync(red_part.ptr, 0, sizeof(double2) * kApplyRedCap, st));
    ApplyExtra ex;
    ex.red = red_part.as<double2>();
    ex.dotv = v;
    ex.red_mode = 2;
    launch_apply(*this, pl, prec, x, y, st, ex);
    ++launches;
    *dot = take_reduction(*this, st);
}

void Operator::observables(const double2 *psi, std::vector<cd> &out, cudaStream_t st) {
    const int dim = sp->dim;
    const size_t n = (size_t)sp->ndof();
    const int k = 2 + dim;
    if ((int)obs_buf.size() < k) {
        obs_buf.clear();
        for (int i = 0; i < k; ++i) obs_buf.emplace_back(n * sizeof(double2));
    }
    const int which[5] = {TDZ_MASS, TDZ_HAMILTONIAN, TDZ_DIPOLE_X, TDZ_DIPOLE_Y, TDZ_DIPOLE_Z};
    std::vector<const void *> V(k);
    for (int i = 0; i < k; ++i) {
        apply(which[i], TDZ_FP64_DF, psi, obs_buf[i].ptr, st);
        V[i] = obs_buf[i].ptr;
    }
    std::vector<cd> d(k);
    blas::mdot(red, V.data(), k, psi, n, TDZ_FP64, d.data(), st);   // conj(A psi) . psi
    out.resize(k);
    for (int i = 0; i < k; ++i) out[i] = std::conj(d[i]);
}

}  // namespace tdz
