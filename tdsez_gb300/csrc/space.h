// Host-side tensor B-spline space: knots, element Gauss rule, basis tables and
// 1D band matrices (FP64). Internal to the tdz library.
#pragma once

#include <array>
#include <vector>

#include "common.h"

namespace tdz {

// Banded 1D matrix, n rows x (2p+1): entry (i, j) at i*(2p+1) + (j - i + p)
// (the layout of src/tensorops.cpp:40-57); entries outside the matrix are 0.
template <class S> struct Band {
    int n = 0, p = 0;
    std::vector<S> v;
    Band() = default;
    Band(int n_, int p_) : n(n_), p(p_), v((size_t)n_ * (2 * p_ + 1), S(0)) {}
    int bw() const { return 2 * p + 1; }
    S &at(int i, int j) { return v[(size_t)i * bw() + (j - i + p)]; }
    S at(int i, int j) const { return v[(size_t)i * bw() + (j - i + p)]; }
};
using BandD = Band<double>;
using BandZ = Band<cd>;

struct Axis1D {
    int p = 0, n = 0, nel = 0, nq = 0;
    std::vector<double> U;          // knots
    std::vector<int> span, offset;  // per element: knot span, first basis index
    std::vector<double> xq, wq;     // nel*nq points and weights*detJac
    std::vector<double> N, dN;      // nel*nq*(p+1) values and first derivatives

    void setup(const double *knots, int nknots, int degree, int nquad);
    // A_ij = sum_q w_q f(x_q) B_i^(da) B_j^(db); f = nullptr means 1.
    BandD band(const double *f, int da, int db) const;
    // Band of x * f(x) (dipole weight).
    BandD band_x() const;
};

struct Space {
    int dim = 0, nquad = 0;
    std::array<Axis1D, 3> ax;
    long long ndof() const {
        long long n = 1;
        for (int d = 0; d < dim; ++d) n *= ax[d].n;
        return n;
    }
};

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);
// Values and derivatives 0..nd of the p+1 non-zero B-splines of span s at x.
void ders_basis(const std::vector<double> &U, int p, int s, double x, int nd, double *out /*(nd+1)*(p+1)*/);
int find_span(const std::vector<double> &U, int p, int n, double x);

}  // namespace tdz
