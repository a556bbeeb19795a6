// Exact banded LU preconditioner for 1D stage operators. Internal.
#pragma once

#include "krylov.h"

namespace tdz {

// P = A: LU factorisation with partial pivoting (FP64 complex, on the device)
// of the assembled 1D stage operator A = alpha M + g (H + c D), walls
// included. Row i of the factor array holds columns i - p .. i + 2p (the
// lower band, the diagonal and the upper band widened by the row
// interchanges); the multipliers of L overwrite the eliminated lower band.
// The factorisation follows the stage it was built from: refresh() marks it
// stale, and the next apply refactors on its own stream. Plays the role of
// the sparse LU that the reference applies to small 1D/2D problems (MUMPS,
// src/tsurff.cpp:803-814; src/multigrid.cpp:315-324).
struct PcBand : Precond {
    Operator *op = nullptr;
    int n = 0, p = 0;
    bool exact = true;        // false: the operator has a term the 1D band leaves out
    bool stale = true;
    DevBuf lu, piv, err;
    std::vector<double2> hband;    // host assembly of the stage band, [n][3p+1]
    long long factorizations = 0;
    void setup(Operator *op_);
    void factor(cudaStream_t st);
    void refresh() override { stale = true; }
    void apply(const double2 *r, double2 *z, cudaStream_t st) override;
};

}  // namespace tdz
