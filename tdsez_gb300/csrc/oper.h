// Matrix-free operator: Kronecker terms, compiled apply plans and device
// copies of the bands. Internal to the tdz library.
#pragma once

#include <array>
#include <map>
#include <memory>
#include <vector>

#include "blas.h"
#include "quad.h"
#include "space.h"

namespace tdz {

constexpr int kMaxComb = 8;   // base bands in one combination
// internal name of TDZ_FP64_F32: FP32 arithmetic on FP64 vectors (3D
// operators without the quadrature term), the certified FP32 Arnoldi apply
constexpr int kPrecF32M64 = TDZ_FP64_F32;

// coef * (band[2] (x) band[1] (x) band[0]); band ids index the per-axis base
// band lists of the operator. The coefficient is factor * sigma[scalar] with
// sigma = (alpha, g, g c_0, g c_1, g c_2) of the current stage.
struct Term {
    int scalar;
    cd factor;
    std::array<int, 3> band;
};

// Linear combination sum_i factor_i sigma[scalar_i] B_{base_i} of base bands
// of one axis; evaluated into kernel parameters at every launch.
struct Comb {
    int n = 0;
    std::array<int, kMaxComb> base{}, scalar{};
    std::array<cd, kMaxComb> factor{};
    void add(int b, int s, cd f);
};

// Three-stream form of every operator of the hot path (outer axis = last):
//   stream A:  T_out (x) M (x) M                       one-axis terms of the outer axis and alpha M
//   stream B:  M_out (x) [M_y (x) T_x + T_y (x) M_x]    one-axis terms of the inner axes
//   stream C:  Mm_out (x) [M_y (x) S_x + S_y (x) M_x]   kinetic terms of a mass layered
//                                                       along the outer axis
// T_x, T_y, T_out and the stream-C outer coefficient are combinations of
// real base bands with complex stage scalars. In 1D everything is stream A.
struct Plan {
    int which = 0, dim = 0;
    bool hasA = false, hasB = false, hasC = false;
    Comb xT, yT, zA, zC;
    bool walls = false;                         // 1D Dirichlet walls pinned in this plan
    int wall_m = -1, wall_h = -1;               // 1D walls: sigma index of M / H diagonal
};

struct Operator {
    const Space *sp = nullptr;
    Space space;                                // private copy
    tdz_physics phys{};
    int P = 0;                                  // common degree (2D/3D kernels)
    std::array<std::vector<BandD>, 3> bases;    // base bands per axis
    std::array<DevBuf, 3> dev32, dev64, devdf;  // base bands on the device per axis (FP32, FP64, double-float)
    std::vector<Term> terms;                    // all terms of the stage operator
    std::vector<int> coupled;                   // coupled axes in order
    double cap_bound = 0.0;                     // bound on the CAP part of M^-1 H (Rayleigh quotient)
    QuadTerm quad;                              // non-separable soft-core potential (per-element quadrature)
    // 1D Dirichlet walls: wall diagonal of H and M
    bool wall1d = false;
    double h_wall[2] = {0, 0}, m_wall[2] = {0, 0};
    std::array<cd, 5> sigma{};                  // current stage scalars
    bool stage_set = false;
    std::map<int, std::unique_ptr<Plan>> plans; // by TDZ_* operator id
    long long launches = 0;

    void build(const Space &s, const tdz_physics &ph);
    int add_band(int axis, BandD b);
    void upload_bases();
    std::vector<Term> terms_for(int which) const;
    std::array<cd, 5> sigma_for(int which) const;
    Plan &plan(int which);                      // build on first use
    void compile(Plan &pl, const std::vector<Term> &ts) const;
    void set_stage(cd alpha, cd g, const std::vector<cd> &c);
    void apply(int which, int prec, const void *x, void *y, cudaStream_t st);
    // y = b - op x in one pass (b and y FP64 for TDZ_FP64 / TDZ_FP64_DF);
    // b may be null (y = op x). With norm: *norm = ||y|| (fused into the
    // store for 3D operators without the quadrature term; synchronises)
    void residual(int which, int prec, const void *x, const void *b, void *y, cudaStream_t st,
                  double *norm = nullptr);
    // y = op x and *dot = <v, y> = sum conj(v) y (FP64 vectors; synchronises)
    void apply_dot(int which, int prec, const void *x, void *y, const void *v, cd *dot, cudaStream_t st);
    DevBuf red_part, red_res;      // fused-reduction partials and result
    blas::Reducer red;             // unfused reductions (allocated on first use, then reused)
    bool fused_reductions() const;
    // upper bound on || |A| ||_2 for operator `which` at the current stage:
    // sum over Kronecker terms of |coefficient| times the product of the
    // terms' 1D max absolute row sums (|A| is symmetric, so its 2-norm is at
    // most its infinity norm); the quadrature term is not included
    double abs_norm_bound(int which) const;
    // FP32 arithmetic on FP64 vectors available (3D, no quadrature term)
    bool f32_on_f64() const { return sp->dim == 3 && !quad.on; }
    // <psi|M|psi>, <psi|H|psi>, <psi|D_a|psi> (FP64 psi); see tdz_observables
    std::vector<DevBuf> obs_buf;
    void observables(const double2 *psi, std::vector<cd> &out, cudaStream_t st);
};

// base band ids present on every axis
enum BaseId { kM = 0, kS = 1, kX = 2 };

// launch-shape autotuning of the 3D apply (apply.cu; on by default)
void set_autotune(int on);
// fixed launch shape of every fused 3D apply (tile_x, run; 0 = autotune), apply.cu
void set_forced_shape(int txw, int run);

// kernel launchers (apply.cu)
// Extras of one apply, fused into its store: y = sub - op x when sub is
// non-null (a residual); for 3D, per-CTA partial sums of |y|^2 (red_mode 1)
// or of conj(dotv) y (red_mode 2) into red[0 .. kApplyRedCap).
constexpr int kApplyRedCap = 4096;   // partial-sum slots (CTAs of one 3D launch)
// red[0 .. kApplyRedCap) summed into *out (device), fixed order
void apply_red_finish(const double2 *part, double2 *out, cudaStream_t st);
struct ApplyExtra {
    const void *sub = nullptr;
    double2 *red = nullptr;
    const void *dotv = nullptr;
    int red_mode = 0;
};
void launch_apply(const Operator &op, const Plan &pl, int prec, const void *x, void *y, cudaStream_t st,
                  const ApplyExtra &ex = ApplyExtra{});
// error word of the 3D apply kernels (a bounded wait that ran out), read and
// cleared (synchronises the device)
int take_apply_error();

}  // namespace tdz
