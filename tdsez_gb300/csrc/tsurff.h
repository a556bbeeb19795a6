// t-SURFF surface flux on the device (FP64). Internal to the tdz library.
#pragma once

#include <array>
#include <vector>

#include "space.h"

namespace tdz {

struct TSurff {
    int dim = 0;
    double R = 0, mass = 1, V0 = 0, sign = 1, dt = 0;
    tdz_field_fn field = nullptr;
    void *field_ctx = nullptr;
    int nq = 0;
    std::array<std::vector<double>, 3> nodes, weights;   // tangential Gauss nodes in [-R, R] per axis
    std::array<int, 3> nk{1, 1, 1};
    std::array<std::vector<double>, 3> k;                // momentum grid axes
    size_t nktot = 1;
    // device tables
    struct AxisTables {
        int n = 0, p = 0, Q = 0;
        DevBuf off, val, der;          // per node: first basis index, p+1 values, p+1 derivatives
        int wall_off[2] = {0, 0};      // at x = -R, +R
        std::vector<double> wall_val[2], wall_der[2];
        DevBuf ek;                     // exp(-i k x_q): [nk][Q] complex
    };
    std::array<AxisTables, 3> ax;
    DevBuf wallv, walld;                // per axis, side: p+1 values and derivatives at -R/+R
    DevBuf g, H, T;                     // face work arrays
    DevBuf cur, prev, amp;              // momentum arrays (complex)
    DevBuf phase;                       // node coordinates then weights (3 axes)
    DevBuf kdev;                        // momentum axes
    std::vector<double> kdev_host;
    // Volkov integrals
    double A[3] = {0, 0, 0}, B[3] = {0, 0, 0}, C = 0, vt = 0, prevT = 0;
    bool have_prev = false;
    long long samples = 0;
    int n[3] = {1, 1, 1};

    // host copies of the in-box node tables (first basis index, p+1 values per node)
    std::array<std::vector<int>, 3> hoff;
    std::array<std::vector<double>, 3> hval;
    DevBuf F[3], work[2];               // interior projection: per-axis tables and work arrays

    void setup(const Space &s, const tdz_tsurff_opts &o, tdz_field_fn f, void *ctx);
    // <chi_k(t_last) | theta psi> over the box |x_d| < R (TDSEZTSurff::Interior /
    // Project, src/tsurff.cpp:565-639): out (host) nk complex values, k_x slowest
    void interior(const double2 *psi, std::vector<cd> &out, cudaStream_t st);
    void advance_volkov(double t);
    void sample(double t, const double2 *psi, cudaStream_t st);
};

}  // namespace tdz
