// Tensor B-spline space on the host (FP64): Gauss-Legendre rule, Cox-de Boor
// basis with derivatives, 1D band matrices.
//
// Follows PetIGA's IGABasis tables as TDSE-Z uses them: element = non-empty
// knot span, Gauss points mapped to the span, weight * detJac
// (src/tensorops.cpp:40-57); the basis recursion is Piegl-Tiller A2.2/A2.3
// (the reference's src/tsurff.cpp:47-66 uses the same published algorithm).
#include "space.h"

#include <algorithm>
#include <cmath>

namespace tdz {

// Gauss-Legendre rule on [-1, 1] by Golub-Welsch: the nodes are the
// eigenvalues of the symmetric tridiagonal Jacobi matrix of the Legendre
// recurrence (zero diagonal, off-diagonal k / sqrt(4 k^2 - 1)), found here by
// cyclic Jacobi rotations; each node is then polished by Newton steps on
// P_n and its weight taken as 2 / ((1 - x^2) P_n'(x)^2) (Abramowitz-Stegun
// 25.4.29), which is accurate to rounding for every n.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    std::vector<double> J((size_t)n * n, 0.0);
    for (int k = 1; k < n; ++k) J[(size_t)(k - 1) * n + k] = J[(size_t)k * n + k - 1] = k / std::sqrt(4.0 * k * k - 1.0);
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) off += J[(size_t)i * n + j] * J[(size_t)i * n + j];
        if (off < 1e-32) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = J[(size_t)p * n + q];
                if (std::abs(apq) < 1e-300) continue;
                const double th = (J[(size_t)q * n + q] - J[(size_t)p * n + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::abs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; ++k) {
                    const double kp = J[(size_t)k * n + p], kq = J[(size_t)k * n + q];
                    J[(size_t)k * n + p] = c * kp - sn * kq;
                    J[(size_t)k * n + q] = sn * kp + c * kq;
                }
                for (int k = 0; k < n; ++k) {
                    const double pk = J[(size_t)p * n + k], qk = J[(size_t)q * n + k];
                    J[(size_t)p * n + k] = c * pk - sn * qk;
                    J[(size_t)q * n + k] = sn * pk + c * qk;
                }
            }
    }
    x.resize(n);
    w.resize(n);
    // P_n(t) and P_n'(t) by the three-term recurrence
    auto legendre = [n](double t, double *d) {
        double p0 = 1.0, p1 = t;
        if (n == 0) { *d = 0.0; return 1.0; }
        for (int k = 2; k <= n; ++k) {
            const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        *d = n * (t * p1 - p0) / (t * t - 1.0);
        return p1;
    };
    for (int i = 0; i < n; ++i) {
        double t = J[(size_t)i * n + i], d = 1.0;
        for (int it = 0; it < 3; ++it) {
            const double v = legendre(t, &d);
            t -= v / d;
        }
        legendre(t, &d);
        x[i] = t;
        w[i] = 2.0 / ((1.0 - t * t) * d * d);
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return x[a] < x[b]; });
    std::vector<double> xs(n), ws(n);
    for (int i = 0; i < n; ++i) { xs[i] = x[idx[i]]; ws[i] = w[idx[i]]; }
    x.swap(xs);
    w.swap(ws);
}

int find_span(const std::vector<double> &U, int p, int n, double x) {
    if (x >= U[n]) return n - 1;
    int lo = p, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x < U[mid]) hi = mid; else lo = mid;
    }
    return lo;
}

void ders_basis(const std::vector<double> &U, int p, int s, double x, int nd, double *out) {
    std::vector<double> ndu((p + 1) * (p + 1), 0.0), left(p + 1, 0.0), right(p + 1, 0.0), a(2 * (p + 1), 0.0);
    auto NDU = [&](int i, int j) -> double & { return ndu[i * (p + 1) + j]; };
    NDU(0, 0) = 1.0;
    for (int j = 1; j <= p; ++j) {
        left[j] = x - U[s + 1 - j];
        right[j] = U[s + j] - x;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            NDU(j, r) = right[r + 1] + left[j - r];
            const double temp = NDU(r, j - 1) / NDU(j, r);
            NDU(r, j) = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        NDU(j, j) = saved;
    }
    for (int r = 0; r <= p; ++r) out[r] = NDU(r, p);
    for (int r = 0; r <= p; ++r) {
        int s1 = 0, s2 = 1;
        auto A = [&](int row, int col) -> double & { return a[row * (p + 1) + col]; };
        A(0, 0) = 1.0;
        for (int k = 1; k <= nd; ++k) {
            double d = 0.0;
            const int rk = r - k, pk = p - k;
            if (r >= k) {
                A(s2, 0) = A(s1, 0) / NDU(pk + 1, rk);
                d = A(s2, 0) * NDU(rk, pk);
            }
            const int j1 = rk >= -1 ? 1 : -rk;
            const int j2 = (r - 1 <= pk) ? k - 1 : p - r;
            for (int j = j1; j <= j2; ++j) {
                A(s2, j) = (A(s1, j) - A(s1, j - 1)) / NDU(pk + 1, rk + j);
                d += A(s2, j) * NDU(rk + j, pk);
            }
            if (r <= pk) {
                A(s2, k) = -A(s1, k - 1) / NDU(pk + 1, r);
                d += A(s2, k) * NDU(r, pk);
            }
            out[k * (p + 1) + r] = d;
            std::swap(s1, s2);
        }
    }
    double fac = p;
    for (int k = 1; k <= nd; ++k) {
        for (int r = 0; r <= p; ++r) out[k * (p + 1) + r] *= fac;
        fac *= (p - k);
    }
}

void Axis1D::setup(const double *knots, int nknots, int degree, int nquad) {
    TDZ_CHECK(degree >= 1 && degree <= 15, TDZ_ERR_ARG, "degree must be in [1, 15]");
    TDZ_CHECK(nquad >= 1 && nquad <= 32, TDZ_ERR_ARG, "nquad must be in [1, 32]");
    TDZ_CHECK(nknots >= 2 * (degree + 1), TDZ_ERR_ARG, "too few knots for the degree");
    p = degree;
    nq = nquad;
    U.assign(knots, knots + nknots);
    for (int i = 0; i + 1 < nknots; ++i) TDZ_CHECK(U[i + 1] >= U[i], TDZ_ERR_ARG, "knots must be non-decreasing");
    n = nknots - p - 1;
    span.clear();
    offset.clear();
    for (int k = p; k < n; ++k)
        if (U[k + 1] > U[k]) { span.push_back(k); offset.push_back(k - p); }
    nel = (int)span.size();
    TDZ_CHECK(nel >= 1, TDZ_ERR_ARG, "axis has no non-empty knot span");
    std::vector<double> gx, gw;
    gauss_legendre(nq, gx, gw);
    xq.assign((size_t)nel * nq, 0.0);
    wq.assign((size_t)nel * nq, 0.0);
    N.assign((size_t)nel * nq * (p + 1), 0.0);
    dN.assign((size_t)nel * nq * (p + 1), 0.0);
    std::vector<double> tmp(2 * (p + 1));
    for (int e = 0; e < nel; ++e) {
        const double a = U[span[e]], b = U[span[e] + 1];
        for (int q = 0; q < nq; ++q) {
            const double x = 0.5 * (a + b) + 0.5 * (b - a) * gx[q];
            const size_t k = (size_t)e * nq + q;
            xq[k] = x;
            wq[k] = gw[q] * 0.5 * (b - a);
            ders_basis(U, p, span[e], x, 1, tmp.data());
            for (int r = 0; r <= p; ++r) {
                N[k * (p + 1) + r] = tmp[r];
                dN[k * (p + 1) + r] = tmp[(p + 1) + r];
            }
        }
    }
}

BandD Axis1D::band(const double *f, int da, int db) const {
    BandD A(n, p);
    const std::vector<double> &Ta = da ? dN : N, &Tb = db ? dN : N;
    for (int e = 0; e < nel; ++e)
        for (int q = 0; q < nq; ++q) {
            const size_t k = (size_t)e * nq + q;
            const double w = wq[k] * (f ? f[k] : 1.0);
            if (w == 0.0) continue;
            const double *ra = &Ta[k * (p + 1)], *rb = &Tb[k * (p + 1)];
            for (int a = 0; a <= p; ++a)
                for (int b = 0; b <= p; ++b) A.at(offset[e] + a, offset[e] + b) += w * ra[a] * rb[b];
        }
    return A;
}

BandD Axis1D::band_x() const {
    std::vector<double> f(xq);
    return band(f.data(), 0, 0);
}

}  // namespace tdz
