// Kronecker inverse of the B-spline overlap, M^-1 = M_z^-1 (x) M_y^-1 (x) M_x^-1,
// by banded Cholesky line solves along each axis. Internal.
#pragma once

#include "space.h"

namespace tdz {

// Banded Cholesky factor of an SPD band: n rows x (p+1), entry j of row i is
// L(i, i-p+j); slot p holds 1/L(i, i).
struct BandChol {
    int n = 0, p = 0;
    std::vector<double> L;
    DevBuf L32, L64;
    void factor(const BandD &A);   // throws if A is not SPD
    void upload();
};

// x <- (A_axis^-1 along one axis) x for an array of shape (n2, n1, n0), x fastest.
void line_solve(const BandChol &F, int axis, void *x, int n0, int n1, int n2, int prec, cudaStream_t st);

// Kronecker solve with one factor per axis (dim axes).
struct KronSolve {
    int dim = 0, n[3] = {1, 1, 1};
    BandChol f[3];
    void setup(const std::array<const BandD *, 3> &bands, int dim_);
    void apply(void *x, int prec, cudaStream_t st) const;   // in place
};

}  // namespace tdz
