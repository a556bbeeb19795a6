// Tensor B-spline space on the host (FP64): Gauss-Legendre rule, Cox-de Boor
// basis with derivatives, 1D band matrices.
//
// Follows PetIGA's IGABasis tables as TDSE-Z uses them: element = non-empty
// knot span, Gauss points mapped to the span, weight * detJac
// (src/tensorops.cpp:40-57); the Gauss rule is the Newton iteration of
// src/tsurff.cpp:24-44 and the basis recursion Piegl-Tiller A2.2/A2.3 as in
// src/tsurff.cpp:47-66.
#include "space.h"

#include <algorithm>
#include <cmath>

namespace tdz {

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const double pi = std::acos(-1.0);
    for (int j = 0; j < n; ++j) {
        double z = std::cos(pi * (j + 0.75) / (n + 0.5)), der = 1;
        for (int it = 0; it < 100; ++it) {
            double p = 1, p0 = 0;
            for (int k = 1; k <= n; ++k) {
                const double old = p;
                p = ((2 * k - 1) * z * p - (k - 1) * p0) / k;
                p0 = old;
            }
            der = n * (z * p - p0) / (z * z - 1);
            const double dz = p / der;
            z -= dz;
            if (std::abs(dz) < 1e-15) break;
        }
        double p = 1, p0 = 0;
        for (int k = 1; k <= n; ++k) {
            const double old = p;
            p = ((2 * k - 1) * z * p - (k - 1) * p0) / k;
            p0 = old;
        }
        der = n * (z * p - p0) / (z * z - 1);
        x[j] = z;
        w[j] = 2 / ((1 - z * z) * der * der);
    }
    // ascending order
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
