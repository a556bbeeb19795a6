// t-SURFF surface flux on the device (FP64): trace of psi and (1/m) d_n psi
// at the surface Gauss points, the factorised flux of FluxGrid
// (src/tsurff.cpp:478-534) as two small contractions per face, and the
// trapezoid accumulation of AddFlux (src/tsurff.cpp:439-469). The Volkov
// integrals (RK4, src/tsurff.cpp:395-428) are advanced on the host.
#include "tsurff.h"

#include <array>
#include <cmath>

#include "cplx.cuh"

namespace tdz {

namespace {

__device__ __forceinline__ double2 cexpi(double a) {
    double s, c;
    sincos(a, &s, &c);
    return make_double2(c, s);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

struct AxisView {
    int n, p, Q;
    const int *off;
    const double *val, *der;    // [Q][p+1]
};

struct FaceParams {
    AxisView b, c;
    int a, side;                 // normal axis, side (0: -R, 1: +R)
    int stride[3];               // coefficient strides per axis
    int wall_off;                // first basis index of the normal axis at the wall
    int pa;                      // degree of the normal axis
    const double *wval, *wder;   // p+1 values / derivatives at the wall
    const double *xb, *xc, *wb, *wc;   // node coordinates and weights
    double Ab, Ac, inv_mass, sigma;
};

// g[0] = -e (1/m) d_n psi, g[1] = -i sigma e psi / m with e = w exp(-i A_t.x_t)
__global__ void k_trace(FaceParams f, const double2 *__restrict__ psi, double2 *__restrict__ g) {
    const int Qb = f.b.Q, Qc = f.c.Q;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= Qb * Qc) return;
    const int ib = idx / Qc, ic = idx % Qc;
    const int ob = f.b.off[ib], oc = f.c.off[ic];
    double2 v = make_double2(0, 0), dn = make_double2(0, 0);
    for (int ja = 0; ja <= f.pa; ++ja) {
        const double va = f.wval[ja], da = f.wder[ja];
        const size_t ia = (size_t)(f.wall_off + ja) * f.stride[f.a];
        for (int jb = 0; jb <= f.b.p; ++jb) {
            const double vb = f.b.val[ib * (f.b.p + 1) + jb];
            const size_t ibb = ia + (size_t)(ob + jb) * f.stride[(f.a == 0) ? 1 : 0];
            for (int jc = 0; jc <= f.c.p; ++jc) {
                const double vc = f.c.val[ic * (f.c.p + 1) + jc];
                const size_t e = ibb + (size_t)(oc + jc) * f.stride[(f.a == 2) ? 1 : 2];
                const double2 ps = psi[e];
                const double wv = va * vb * vc, wd = da * vb * vc;
                v.x += wv * ps.x; v.y += wv * ps.y;
                dn.x += wd * ps.x; dn.y += wd * ps.y;
            }
        }
    }
    dn.x *= f.sigma * f.inv_mass;
    dn.y *= f.sigma * f.inv_mass;
    const double xb = f.xb[ib], xc = f.xc[ic];
    double2 e = cexpi(-(f.Ab * xb + f.Ac * xc));
    const double w = f.wb[ib] * f.wc[ic];
    e.x *= w; e.y *= w;
    const double2 g1 = cmul(e, dn);
    // -i sigma e psi / m
    const double2 ev = cmul(e, v);
    const double s = f.sigma * f.inv_mass;
    g[idx] = make_double2(-g1.x, -g1.y);
    g[(size_t)Qb * Qc + idx] = make_double2(s * ev.y, -s * ev.x);
}

// H[s][ib][kc] = sum_ic g[s][ib][ic] Ec[kc][ic]
__global__ void k_face_c(const double2 *__restrict__ g, const double2 *__restrict__ Ec, int Qb, int Qc, int nc,
                         double2 *__restrict__ H) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2 * Qb * nc) return;
    const int s = idx / (Qb * nc), r = idx % (Qb * nc), ib = r / nc, kc = r % nc;
    const double2 *gr = g + (size_t)s * Qb * Qc + (size_t)ib * Qc;
    const double2 *er = Ec + (size_t)kc * Qc;
    double2 acc = make_double2(0, 0);
    for (int q = 0; q < Qc; ++q) {
        const double2 a = gr[q], b = er[q];
        acc.x += a.x * b.x - a.y * b.y;
        acc.y += a.x * b.y + a.y * b.x;
    }
    H[idx] = acc;
}

// T[s][kb][kc] = sum_ib Eb[kb][ib] H[s][ib][kc]
__global__ void k_face_b(const double2 *__restrict__ H, const double2 *__restrict__ Eb, int Qb, int nb, int nc,
                         double2 *__restrict__ T) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2 * nb * nc) return;
    const int s = idx / (nb * nc), r = idx % (nb * nc), kb = r / nc, kc = r % nc;
    double2 acc = make_double2(0, 0);
    for (int q = 0; q < Qb; ++q) {
        const double2 a = Eb[(size_t)kb * Qb + q], b = H[(size_t)s * Qb * nc + (size_t)q * nc + kc];
        acc.x += a.x * b.x - a.y * b.y;
        acc.y += a.x * b.y + a.y * b.x;
    }
    T[idx] = acc;
}

struct KGrid {
    int nk[3];
    const double *k[3];
};

// cur(k) += exp(-i (k_a + A_a) sigma R) (T_1 + (k_a + A_a) T_2)
__global__ void k_face_acc(KGrid kg, int a, int b, int c, double Aa, double sigmaR, const double2 *__restrict__ T,
                           double2 *__restrict__ cur, int first) {
    const size_t tot = (size_t)kg.nk[0] * kg.nk[1] * kg.nk[2];
    const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= tot) return;
    int kk[3];
    kk[2] = (int)(idx % kg.nk[2]);
    kk[1] = (int)((idx / kg.nk[2]) % kg.nk[1]);
    kk[0] = (int)(idx / ((size_t)kg.nk[2] * kg.nk[1]));
    const int nb = kg.nk[b], nc = kg.nk[c];
    const double ka = kg.k[a][kk[a]] + Aa;
    const double2 ph = cexpi(-ka * sigmaR);
    const double2 t1 = T[(size_t)kk[b] * nc + kk[c]];
    const double2 t2 = T[(size_t)nb * nc + (size_t)kk[b] * nc + kk[c]];
    const double2 sum = make_double2(t1.x + ka * t2.x, t1.y + ka * t2.y);
    const double2 v = cmul(ph, sum);
    double2 o = first ? make_double2(0, 0) : cur[idx];
    o.x += v.x;
    o.y += v.y;
    cur[idx] = o;
}

// cur *= pre * prod_d exp(i (t k_d^2 / 2m + k_d B_d / m)); amp += h (prev + cur); prev = cur
__global__ void k_finish(KGrid kg, double2 pre, double t, double inv2m, double invm, double B0, double B1,
                         double B2, double h, int have_prev, double2 *cur, double2 *prev, double2 *amp) {
    const size_t tot = (size_t)kg.nk[0] * kg.nk[1] * kg.nk[2];
    const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= tot) return;
    int kk[3];
    kk[2] = (int)(idx % kg.nk[2]);
    kk[1] = (int)((idx / kg.nk[2]) % kg.nk[1]);
    kk[0] = (int)(idx / ((size_t)kg.nk[2] * kg.nk[1]));
    const double Bs[3] = {B0, B1, B2};
    double phase = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double k = kg.k[d][kk[d]];
        phase += t * k * k * inv2m + k * Bs[d] * invm;
    }
    const double2 c = cmul(cmul(pre, cexpi(phase)), cur[idx]);
    if (have_prev) {
        const double2 p = prev[idx];
        double2 a = amp[idx];
        a.x += h * (p.x + c.x);
        a.y += h * (p.y + c.y);
        amp[idx] = a;
    }
    prev[idx] = c;
}

inline int blocks_for(size_t n, int t = 256) { return (int)((n + t - 1) / t); }

}  // namespace

void TSurff::setup(const Space &s, const tdz_tsurff_opts &o, tdz_field_fn f, void *ctx) {
    dim = s.dim;
    R = o.radius;
    mass = o.mass > 0 ? o.mass : 1.0;
    V0 = o.v0;
    sign = -o.charge;
    dt = o.dt;
    TDZ_CHECK(dt > 0, TDZ_ERR_ARG, "t-SURFF needs the time step");
    TDZ_CHECK(R > 0, TDZ_ERR_ARG, "t-SURFF radius must be positive");
    field = f;
    field_ctx = ctx;
    nq = o.nquad > 0 ? o.nquad : s.nquad;
    std::vector<double> gx, gw;
    gauss_legendre(nq, gx, gw);
    nktot = 1;
    for (int d = 0; d < 3; ++d) {
        AxisTables &T = ax[d];
        nodes[d].clear();
        weights[d].clear();
        k[d].clear();
        if (d >= dim) {
            nodes[d] = {0.0};
            weights[d] = {1.0};
            k[d] = {0.0};
            nk[d] = 1;
            T.n = 1; T.p = 0; T.Q = 1;
            upload(T.off, std::vector<int>{0});
            upload(T.val, std::vector<double>{1.0});
            upload(T.der, std::vector<double>{0.0});
            T.wall_off[0] = T.wall_off[1] = 0;
            T.wall_val[0] = T.wall_val[1] = {1.0};
            T.wall_der[0] = T.wall_der[1] = {0.0};
        } else {
            const Axis1D &A = s.ax[d];
            TDZ_CHECK(A.U.front() < -R && A.U.back() > R, TDZ_ERR_ARG, "t-SURFF surface is not inside the box");
            for (size_t j = 0; j + 1 < A.U.size(); ++j) {
                const double lo = std::max(A.U[j], -R), hi = std::min(A.U[j + 1], R);
                if (hi <= lo) continue;
                for (int q = 0; q < nq; ++q) {
                    nodes[d].push_back(0.5 * (lo + hi) + 0.5 * (hi - lo) * gx[q]);
                    weights[d].push_back(0.5 * (hi - lo) * gw[q]);
                }
            }
            T.n = A.n;
            T.p = A.p;
            T.Q = (int)nodes[d].size();
            std::vector<int> off(T.Q);
            std::vector<double> val((size_t)T.Q * (A.p + 1)), der((size_t)T.Q * (A.p + 1)), tmp(2 * (A.p + 1));
            for (int q = 0; q < T.Q; ++q) {
                const int sp = find_span(A.U, A.p, A.n, nodes[d][q]);
                ders_basis(A.U, A.p, sp, nodes[d][q], 1, tmp.data());
                off[q] = sp - A.p;
                for (int r = 0; r <= A.p; ++r) { val[(size_t)q * (A.p + 1) + r] = tmp[r]; der[(size_t)q * (A.p + 1) + r] = tmp[A.p + 1 + r]; }
            }
            upload(T.off, off);
            upload(T.val, val);
            upload(T.der, der);
            hoff[d] = off;
            hval[d].assign(val.begin(), val.end());
            for (int side = 0; side < 2; ++side) {
                const double x = side ? R : -R;
                const int sp = find_span(A.U, A.p, A.n, x);
                ders_basis(A.U, A.p, sp, x, 1, tmp.data());
                T.wall_off[side] = sp - A.p;
                T.wall_val[side].assign(tmp.begin(), tmp.begin() + A.p + 1);
                T.wall_der[side].assign(tmp.begin() + A.p + 1, tmp.begin() + 2 * (A.p + 1));
            }
            nk[d] = std::max(1, o.nk[d]);
            for (int i = 0; i < nk[d]; ++i)
                k[d].push_back(nk[d] == 1 ? o.kmin[d] : o.kmin[d] + i * (o.kmax[d] - o.kmin[d]) / (nk[d] - 1));
        }
        n[d] = T.n;
        // exp(-i k x_q) table
        std::vector<double2> ek((size_t)nk[d] * T.Q);
        for (int i = 0; i < nk[d]; ++i)
            for (int q = 0; q < T.Q; ++q) {
                const double a = -k[d][i] * nodes[d][q];
                ek[(size_t)i * T.Q + q] = make_double2(std::cos(a), std::sin(a));
            }
        upload(T.ek, ek);
        nktot *= nk[d];
    }
    size_t gmax = 0, hmax = 0, tmax = 0;
    for (int a = 0; a < dim; ++a) {
        const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
        gmax = std::max(gmax, (size_t)2 * ax[b].Q * ax[c].Q);
        hmax = std::max(hmax, (size_t)2 * ax[b].Q * nk[c]);
        tmax = std::max(tmax, (size_t)2 * nk[b] * nk[c]);
    }
    g.alloc(gmax * sizeof(double2));
    H.alloc(hmax * sizeof(double2));
    T.alloc(tmax * sizeof(double2) * 2 * dim);
    for (DevBuf *b : {&cur, &prev, &amp}) b->alloc(nktot * sizeof(double2));
    TDZ_CUDA(cudaMemset(amp.ptr, 0, nktot * sizeof(double2)));
    // wall values and node coordinates / weights per axis
    std::vector<double> wv, wd;
    for (int d = 0; d < 3; ++d)
        for (int side = 0; side < 2; ++side) {
            wv.insert(wv.end(), ax[d].wall_val[side].begin(), ax[d].wall_val[side].end());
            wd.insert(wd.end(), ax[d].wall_der[side].begin(), ax[d].wall_der[side].end());
            wv.resize(wv.size() + (16 - ax[d].wall_val[side].size()), 0.0);
            wd.resize(wd.size() + (16 - ax[d].wall_der[side].size()), 0.0);
        }
    upload(wallv, wv);
    upload(walld, wd);
    std::vector<double> xw;
    for (int d = 0; d < 3; ++d) xw.insert(xw.end(), nodes[d].begin(), nodes[d].end());
    for (int d = 0; d < 3; ++d) xw.insert(xw.end(), weights[d].begin(), weights[d].end());
    std::vector<double> kall;
    for (int d = 0; d < 3; ++d) kall.insert(kall.end(), k[d].begin(), k[d].end());
    upload(phase, xw);        // node coordinates then weights
    kdev_host = kall;
    upload(kdev, kall);
}

namespace {
using Volkov7 = std::array<double, 7>;   // A_x, A_y, A_z, B_x, B_y, B_z, C
// one classical fourth-order Runge-Kutta step (Kutta's tableau) of y' = f(t, y)
template <class F> Volkov7 rk4_step(const F &f, double t, const Volkov7 &y, double h) {
    auto along = [&](const Volkov7 &s, double c) {
        Volkov7 r;
        for (int i = 0; i < 7; ++i) r[i] = y[i] + c * s[i];
        return r;
    };
    const Volkov7 s1 = f(t, y);
    const Volkov7 s2 = f(t + 0.5 * h, along(s1, 0.5 * h));
    const Volkov7 s3 = f(t + 0.5 * h, along(s2, 0.5 * h));
    const Volkov7 s4 = f(t + h, along(s3, h));
    Volkov7 out;
    for (int i = 0; i < 7; ++i) out[i] = y[i] + h * (s1[i] + 2.0 * (s2[i] + s3[i]) + s4[i]) / 6.0;
    return out;
}
}  // namespace

// Volkov phases of the surface states from the last sample time to t:
// A' = -s E(t), B' = A, C' = |A|^2 / 2m + V0, by Runge-Kutta substeps of at
// most dt/2 (the substep rule of AdvanceVolkov, src/tsurff.cpp:395-428, which
// the flux's parity with the reference depends on)
void TSurff::advance_volkov(double t) {
    const double span = t - vt;
    if (span <= 0) return;
    const int substeps = std::max(1, (int)std::ceil(span / (0.5 * dt) - 1e-9));
    const double ds = span / substeps;
    auto deriv = [&](double tt, const Volkov7 &y) {
        Volkov7 d{};
        double a2 = 0.0;
        for (int a = 0; a < 3; ++a) {
            d[a] = (a < dim && field) ? -sign * field(a, tt, field_ctx) : 0.0;
            d[3 + a] = y[a];
            a2 += y[a] * y[a];
        }
        d[6] = a2 / (2.0 * mass) + V0;
        return d;
    };
    Volkov7 y{A[0], A[1], A[2], B[0], B[1], B[2], C};
    for (int k = 0; k < substeps; ++k) y = rk4_step(deriv, vt + k * ds, y, ds);
    for (int a = 0; a < 3; ++a) { A[a] = y[a]; B[a] = y[3 + a]; }
    C = y[6];
    vt = t;
}

KGridHost TSurff::kgrid() const {
    KGridHost kg;
    size_t ka = 0;
    for (int d = 0; d < 3; ++d) {
        kg.nk[d] = nk[d];
        kg.k[d] = kdev.as<double>() + ka;
        ka += k[d].size();
    }
    return kg;
}

// cur(k) = the surface integral of the flux of psi against the Volkov states
// at the current Volkov time, before the common factor (FluxGrid)
void TSurff::surface_flux(const double2 *psi, cudaStream_t st) {
    const double *xw = phase.as<double>();
    size_t xoff[3], woff[3], acc = 0;
    for (int d = 0; d < 3; ++d) { xoff[d] = acc; acc += nodes[d].size(); }
    for (int d = 0; d < 3; ++d) { woff[d] = acc; acc += weights[d].size(); }
    const KGridHost kh = kgrid();
    KGrid kg;
    for (int d = 0; d < 3; ++d) { kg.nk[d] = kh.nk[d]; kg.k[d] = kh.k[d]; }
    int first = 1;
    for (int a = 0; a < dim; ++a)
        for (int side = 0; side < 2; ++side) {
            const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
            FaceParams f;
            f.b = {ax[b].n, ax[b].p, ax[b].Q, ax[b].off.as<int>(), ax[b].val.as<double>(), ax[b].der.as<double>()};
            f.c = {ax[c].n, ax[c].p, ax[c].Q, ax[c].off.as<int>(), ax[c].val.as<double>(), ax[c].der.as<double>()};
            f.a = a;
            f.side = side;
            f.stride[0] = 1;
            f.stride[1] = n[0];
            f.stride[2] = n[0] * n[1];
            f.wall_off = ax[a].wall_off[side];
            f.pa = ax[a].p;
            f.wval = wallv.as<double>() + (a * 2 + side) * 16;
            f.wder = walld.as<double>() + (a * 2 + side) * 16;
            f.xb = xw + xoff[b];
            f.xc = xw + xoff[c];
            f.wb = xw + woff[b];
            f.wc = xw + woff[c];
            f.Ab = A[b];
            f.Ac = A[c];
            f.inv_mass = 1.0 / mass;
            f.sigma = side ? 1.0 : -1.0;
            const int Qb = ax[b].Q, Qc = ax[c].Q;
            k_trace<<<blocks_for((size_t)Qb * Qc), 256, 0, st>>>(f, psi, g.as<double2>());
            k_face_c<<<blocks_for((size_t)2 * Qb * nk[c]), 256, 0, st>>>(g.as<double2>(), ax[c].ek.as<double2>(), Qb,
                                                                        Qc, nk[c], H.as<double2>());
            double2 *Tf = T.as<double2>();
            k_face_b<<<blocks_for((size_t)2 * nk[b] * nk[c]), 256, 0, st>>>(H.as<double2>(), ax[b].ek.as<double2>(),
                                                                            Qb, nk[b], nk[c], Tf);
            k_face_acc<<<blocks_for(nktot), 256, 0, st>>>(kg, a, b, c, A[a], f.sigma * R, Tf, cur.as<double2>(), first);
            first = 0;
            TDZ_CUDA(cudaGetLastError());
            count_launch(4);
        }
}

void TSurff::sample(double t, const double2 *psi, cudaStream_t st) {
    if (have_prev && t == prevT) return;
    TDZ_CHECK(!have_prev || t > prevT, TDZ_ERR_ARG, "t-SURFF sample times must increase");
    advance_volkov(t);
    surface_flux(psi, st);
    const KGridHost kh = kgrid();
    KGrid kg;
    for (int d = 0; d < 3; ++d) { kg.nk[d] = kh.nk[d]; kg.k[d] = kh.k[d]; }
    const double two_pi = 2.0 * std::acos(-1.0);
    const double pref = 0.5 * std::pow(two_pi, -0.5 * dim);
    // pre = (i/2) (2 pi)^{-d/2} exp(i C)
    const double2 pre = make_double2(-pref * std::sin(C), pref * std::cos(C));
    k_finish<<<blocks_for(nktot), 256, 0, st>>>(kg, pre, vt, 0.5 / mass, 1.0 / mass, B[0], B[1], B[2],
                                                 0.5 * (t - prevT), have_prev ? 1 : 0, cur.as<double2>(),
                                                 prev.as<double2>(), amp.as<double2>());
    TDZ_CUDA(cudaGetLastError());
    count_launch();
    prevT = t;
    have_prev = true;
    ++samples;
}

namespace {
// amp[q_e] += w_e pre exp(i (t |k|^2 / 2m + k.B / m)) cur[q_e]; the entries of
// one node name distinct momenta
__global__ void k_end_acc(KGrid kg, double2 pre, double t, double inv2m, double invm, double B0, double B1, double B2,
                          const int *__restrict__ q, const double *__restrict__ w, int m,
                          const double2 *__restrict__ cur, double2 *__restrict__ amp) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const size_t idx = (size_t)q[e];
    int kk[3];
    kk[2] = (int)(idx % kg.nk[2]);
    kk[1] = (int)((idx / kg.nk[2]) % kg.nk[1]);
    kk[0] = (int)(idx / ((size_t)kg.nk[2] * kg.nk[1]));
    const double Bs[3] = {B0, B1, B2};
    double phase = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double k = kg.k[d][kk[d]];
        phase += t * k * k * inv2m + k * Bs[d] * invm;
    }
    const double2 c = cmul(cmul(pre, cexpi(phase)), cur[idx]);
    double2 a = amp[idx];
    a.x += w[e] * c.x;
    a.y += w[e] * c.y;
    amp[idx] = a;
}
}  // namespace

void TSurff::add_weighted_flux(const double2 *phi, const int *q, const double *w, int m, cudaStream_t st) {
    if (m <= 0) return;
    surface_flux(phi, st);
    const KGridHost kh = kgrid();
    KGrid kg;
    for (int d = 0; d < 3; ++d) { kg.nk[d] = kh.nk[d]; kg.k[d] = kh.k[d]; }
    const double pref = 0.5 * std::pow(2.0 * std::acos(-1.0), -0.5 * dim);
    const double2 pre = make_double2(-pref * std::sin(C), pref * std::cos(C));
    k_end_acc<<<blocks_for((size_t)m), 256, 0, st>>>(kg, pre, vt, 0.5 / mass, 1.0 / mass, B[0], B[1], B[2], q, w, m,
                                                      cur.as<double2>(), amp_end.as<double2>());
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

namespace {
// out[a][k][b] = sum_i F[k][i] in[a][i][b] (complex, double-float arithmetic)
__global__ void k_axis_dense(const double2 *__restrict__ F, const double2 *__restrict__ in, double2 *__restrict__ out,
                             long long A, int nk, int ni, long long B) {
    const long long total = A * nk * B;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long b = t % B, r = t / B;
        const int k = (int)(r % nk);
        const long long a = r / nk;
        cdff acc;
        acc.x = dff(0.f);
        acc.y = dff(0.f);
        const double2 *fk = F + (size_t)k * ni;
        const double2 *ia = in + (size_t)a * ni * B + b;
        for (int i = 0; i < ni; ++i) {
            const cdff f = load_c<cdff, double2>(fk[i]);
            const cdff v = load_c<cdff, double2>(ia[(size_t)i * B]);
            cfma(acc, f, v);
        }
        out[t] = store_c<double2, cdff>(cnorm(acc));
    }
}
}  // namespace

void TSurff::interior(const double2 *psi, std::vector<cd> &out, cudaStream_t st) {
    // F_d[k][i] = sum_q w_q exp(-i (k + A_d) x_q) B_i(x_q) over the in-box nodes
    for (int d = 0; d < 3; ++d) {
        std::vector<double2> f((size_t)nk[d] * n[d], make_double2(0.0, 0.0));
        if (d >= dim) {
            f[0] = make_double2(1.0, 0.0);
        } else {
            const int pp = ax[d].p + 1;
            for (size_t q = 0; q < nodes[d].size(); ++q)
                for (int kk = 0; kk < nk[d]; ++kk) {
                    const double ph = -(k[d][kk] + A[d]) * nodes[d][q];
                    const cd e = weights[d][q] * cd(std::cos(ph), std::sin(ph));
                    for (int b = 0; b < pp; ++b) {
                        const int i = hoff[d][q] + b;
                        const cd v = e * hval[d][q * pp + b];
                        double2 &z = f[(size_t)kk * n[d] + i];
                        z.x += v.real();
                        z.y += v.imag();
                    }
                }
        }
        upload(F[d], f);
    }
    // contract x, then y, then z: [z][y][x] -> [z][y][kx] -> [z][ky][kx] -> [kz][ky][kx]
    const size_t w0 = (size_t)n[2] * n[1] * nk[0], w1 = (size_t)n[2] * nk[1] * nk[0];
    if (work[0].bytes < w0 * sizeof(double2)) work[0].alloc(w0 * sizeof(double2));
    if (work[1].bytes < std::max(w1, nktot) * sizeof(double2)) work[1].alloc(std::max(w1, nktot) * sizeof(double2));
    auto pass = [&](const double2 *src, double2 *dst, long long a, int d, long long b) {
        const long long total = a * nk[d] * b;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 16LL * sm_count());
        k_axis_dense<<<blocks, 256, 0, st>>>(F[d].as<double2>(), src, dst, a, nk[d], n[d], b);
        TDZ_CUDA(cudaGetLastError());
        count_launch();
    };
    pass(psi, work[0].as<double2>(), (long long)n[2] * n[1], 0, 1);
    pass(work[0].as<double2>(), work[1].as<double2>(), n[2], 1, nk[0]);
    pass(work[1].as<double2>(), work[0].as<double2>(), 1, 2, (long long)nk[1] * nk[0]);
    std::vector<double2> h(nktot);
    TDZ_CUDA(cudaMemcpyAsync(h.data(), work[0].ptr, nktot * sizeof(double2), cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    // times the Volkov phase (2 pi)^(-d/2) exp(i (C + T k^2 / 2m + k.B / m)), k_x slowest
    const double norm = std::pow(2.0 * M_PI, -0.5 * dim);
    out.assign(nktot, cd(0.0));
    for (int i = 0; i < nk[0]; ++i)
        for (int j = 0; j < nk[1]; ++j)
            for (int l = 0; l < nk[2]; ++l) {
                const double kv[3] = {k[0][i], k[1][j], k[2][l]};
                double ph = C;
                for (int d = 0; d < dim; ++d) ph += vt * kv[d] * kv[d] / (2.0 * mass) + kv[d] * B[d] / mass;
                const double2 g = h[((size_t)l * nk[1] + j) * nk[0] + i];
                out[((size_t)i * nk[1] + j) * nk[2] + l] = norm * cd(std::cos(ph), std::sin(ph)) * cd(g.x, g.y);
            }
}

}  // namespace tdz
