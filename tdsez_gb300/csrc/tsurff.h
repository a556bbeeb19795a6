// t-SURFF surface flux on the device (FP64). Internal to the tdz library.
#pragma once

#include <array>
#include <vector>

#include "space.h"

namespace tdz {

struct Operator;
struct SolverOptions;

// momentum grid axes on the device
struct KGridHost {
    int nk[3];
    const double *k[3];
};

// t-SURFF end term: options and what the run took
struct EndTermOptions {
    double dp = 0.0;          // node spacing in |k + A(T)|; 0 = automatic (SurffEndTermDk = 0)
    double cap_width = 0.0;   // width of the absorbing layer (sets the refined range below 2 k_cap)
    double eta = -1.0;        // pole damping of the preconditioner: E (1 + i eta); < 0 = automatic
    double rtol = 1e-10;      // relative residual of every node's solve
    int maxit = 600;          // FGMRES iterations per node
};
struct EndTermStats {
    int nodes = 0;            // energy nodes
    long long its = 0;        // FGMRES iterations over all nodes
    int max_its = 0;          // largest per node
    double dp_max = 0.0;      // largest node spacing
    double eta = 0.0;         // pole damping used
    int damped = 0;           // nodes finished with the damped pole after a stagnating undamped start
    double seconds = 0.0;
};

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
    DevBuf amp_end;                     // end-term amplitudes
    DevBuf eq, ew;                      // end term: (momentum, weight) entries grouped by node

    void setup(const Space &s, const tdz_tsurff_opts &o, tdz_field_fn f, void *ctx);
    // <chi_k(t_last) | theta psi> over the box |x_d| < R (TDSEZTSurff::Interior /
    // Project, src/tsurff.cpp:565-639): out (host) nk complex values, k_x slowest
    void interior(const double2 *psi, std::vector<cd> &out, cudaStream_t st);
    void advance_volkov(double t);
    KGridHost kgrid() const;
    // cur = the flux of psi at the current Volkov time without the common factor
    void surface_flux(const double2 *psi, cudaStream_t st);
    void sample(double t, const double2 *psi, cudaStream_t st);
    // amp_end[q_e] += w_e flux(phi)(q_e) over m entries (q_e, w_e), the flux at
    // the last sample with its Volkov factor and no time weight
    void add_weighted_flux(const double2 *phi, const int *q, const double *w, int m, cudaStream_t st);
    // The flux after the last sample time T (the field must be over):
    // sum over energy nodes E_j of Lagrange weights times the flux of
    // phi_j = (E_j M - H)^-1 i M psi(T), H = op's field-free Hamiltonian with
    // its absorbing layer (TDSEZTSurff::EndTerm, src/tsurff.cpp:650-976).
    // out (host): nktot complex amplitudes, k_x slowest.
    EndTermStats end_term(Operator &op, const SolverOptions &so, const EndTermOptions &eo, const double2 *psi,
                          std::vector<cd> &out, cudaStream_t st);
};

}  // namespace tdz
