// Fast-diagonalisation preconditioner for operators whose inner axes carry
// only mass and stiffness (the z-layered structure). Internal.
#pragma once

#include <vector>

#include "krylov.h"
#include "tgemm.h"

namespace tdz {

// Generalised symmetric eigenproblem S V = M V diag(lam), V^T M V = I
// (dense, host, FP64; Cholesky reduction + cyclic Jacobi).
void gen_eig(const BandD &S, const BandD &M, std::vector<double> &V, std::vector<double> &lam);
// The same for a complex symmetric band S ([n][2p+1]) against the real SPD M:
// S V = M V diag(lam), V^T M V = I (bilinear, not Hermitian). Returns false
// when no such basis is found to working accuracy (eig_cs.cpp).
bool gen_eig_complex(const std::vector<cd> &S, int p, const BandD &M, std::vector<cd> &V, std::vector<cd> &lam);

// A = (M_x (x) M_y) (x) Bz + (S_x (x) M_y + M_x (x) S_y) (x) Cz with Bz, Cz
// combinations of the outer-axis base bands. Then
//   A^-1 = (V_x (x) V_y (x) I) [ (Bz + (lam_i + lam_j) Cz)^-1 ]_{ij} (V_x^T (x) V_y^T (x) I),
// applied as dense transforms along x and y and one banded complex LU solve
// per (i, j) line along z, in FP32 (tensor-core transforms in 3D) or FP64.
struct PcFDM : Precond {
    Operator *op = nullptr;
    int dim = 0, P = 0;
    int n[3] = {1, 1, 1};
    size_t N = 0;
    DevBuf V[2], VT[2];        // FP32 n_d x n_d (row-major) eigenvectors and their transpose
                               // (complex FP32 when cplx)
    DevBuf lam[2];             // FP32 eigenvalues per inner axis
    DevBuf lami[2];            // their imaginary parts (cplx)
    // inner-axis pencils: 0 = stiffness only; 1 = S_d = all inner one-axis
    // terms on the common stage scalar pencil_scalar (exact for operators with
    // potentials and absorbing layers on the inner axes, no field there)
    int pencil = 0, pencil_scalar = 1;
    bool cplx = false;         // some axis pencil is complex symmetric (absorbing layer)
    std::vector<int> dropped;  // stage scalars of inner terms left out of the pencil (pencil 1)
    // the inverse is exact (to FP32) for the operator's current stage: nothing
    // dropped, or the dropped terms' stage scalars are zero now
    bool exact_now() const;
    DevBuf zb;                 // FP32 band rows of the line matrices, Bc then Cc, [2][n_outer][2P+1]
    DevBuf b1, b2, ufac;       // FP32 work vectors and the saved elimination states of the line solves
    bool exact = true;         // false: inner one-axis terms were dropped (stiffness-only pencil, or a
                               // field along an inner axis)
    // 3D with n_x, n_y <= 256: transforms on the tensor cores (tcgen05, TF32 hi/lo split) over
    // row-planar FP32 buffers pa ([z][y][c][x], pitch ldx) and pb ([z][x][c][y], pitch ldy)
    bool tensor = false;
    TransformMat Tf[2], Ti[2];
    DevBuf pa, pb;
    int ldx = 0, ldy = 0;
    long long applies = 0;
    // with `pole`, the line solves use these stage scalars instead of the
    // operator's (a preconditioner for a shifted copy of the stage, e.g. the
    // complex-shifted poles of the t-SURFF end term)
    bool pole = false;
    std::array<cd, 5> pole_sigma{};
    bool f64 = false;          // FP64 preconditioner: SIMT FP64 transforms and FP64 line solves
                               // (partial pivoting; factors in ufac, interchanges in piv64)
    DevBuf piv64;
    DevBuf npart;              // per-block partial sums of ||z||^2 (apply_norm)
    double *norm_out = nullptr;   // set during apply_norm
    void setup(Operator *op_, int prec = TDZ_FP32);
    void apply(const double2 *r, double2 *z, cudaStream_t st) override;
    // the tensor-core path forms ||z||^2 in its output layout pass
    bool has_apply_norm() const override { return tensor; }
    void apply_norm(const double2 *r, double2 *z, double *norm2, cudaStream_t st) override;
};

}  // namespace tdz
