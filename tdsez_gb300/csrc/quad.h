// Non-separable potential term by per-element quadrature. Internal.
//
//   (V_q)_ab = s sum_q w_q V(x_q) B_a(x_q) B_b(x_q),
//   V(r) = sum_k -Z_k / sqrt(|r - c_k|^2 + a_k)          (soft-core centres)
// the s V block of TDSEZFormHam (src/assembly/assembly.cpp:703-864) and of the
// sum-factorised element kernel SumFactElement (src/assembly/sumfact.cpp:471-523)
// for a potential that is not a sum of one-axis functions (the 2D and 3D
// soft-core Coulomb cases). Applied matrix-free: per element the (p+1)^d
// local coefficients are interpolated to the Q^d Gauss points one axis at a
// time, multiplied by w V (V evaluated in the kernel from the closed form, no
// table), projected back one axis at a time and added to y.
#pragma once

#include "space.h"

namespace tdz {

constexpr int kMaxSoft = 8;

struct QuadTerm {
    bool on = false;
    int nsoft = 0;
    double soft[kMaxSoft][5] = {};    // Z, cx, cy, cz, a
    int dim = 0, p = 0, nq = 0;
    int nel[3] = {1, 1, 1}, n[3] = {1, 1, 1};
    bool consecutive = false;         // every element's window starts one coefficient after the last one's
    // per axis: first basis index per element, basis values [e][q][a], weights [e][q], points [e][q]
    DevBuf off[3], N32[3], N64[3], w64[3], x64[3], w32[3], x32[3];
    void build(const Space &s, int nsoft_, const double *soft_);
    // y += coef * V_q x (complex coef; prec TDZ_FP32 or FP64 vectors)
    void apply(cd coef, int prec, const void *x, void *y, cudaStream_t st) const;
};

}  // namespace tdz
