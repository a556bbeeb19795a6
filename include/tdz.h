/*
 * tdz.h - C ABI of the GB300 propagation library for TDSE-Z's hot path.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes, no
 * exceptions across the boundary. Vectors are device arrays of interleaved
 * complex numbers (re, im) in the natural B-spline ordering, x fastest
 * (index i + n_x (j + n_y k)); TDZ_FP32 means complex float (8 bytes per
 * coefficient), TDZ_FP64 complex double (16 bytes). Device buffers passed in
 * are owned by the caller; handles own their internal work buffers, which are
 * allocated when the handle is created. Streams are cudaStream_t passed as
 * void* (NULL = the legacy default stream).
 *
 * Each entry point names the reference interface it replaces
 * (paths are relative to the TDSE-Z source tree).
 */
#ifndef TDZ_H
#define TDZ_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int tdz_status;
#define TDZ_OK 0
#define TDZ_ERR_ARG 1            /* invalid argument */
#define TDZ_ERR_CUDA 2           /* CUDA runtime error */
#define TDZ_ERR_NOT_CONVERGED 3  /* Krylov solve hit its iteration limit */
#define TDZ_ERR_STATE 4          /* object not set up for this call */
#define TDZ_ERR_UNSUPPORTED 5    /* configuration not supported */
#define TDZ_ERR_BREAKDOWN 6      /* Krylov breakdown / non-finite residual */
#define TDZ_ERR_INTERNAL 7

#define TDZ_FP32 0
#define TDZ_FP64 1
/* FP64 vectors (complex double in memory) whose operator apply computes in
 * double-float arithmetic on the FP32 pipes: about 48 significant bits, a
 * relative error near 1e-14, several times the speed of native FP64 on
 * GB300. Accepted by tdz_operator_apply and as tdz_solver_opts.outer_precision. */
#define TDZ_FP64_DF 2
/* FP64 vectors whose operator apply computes in FP32 arithmetic (inputs
 * truncated to 24 bits, results widened exactly): the FP32 apply's accuracy
 * at FP64 storage, for corrections whose own size bounds the error (relaxed
 * Krylov steps). 3D operators without the soft-core quadrature term;
 * accepted by tdz_operator_apply. */
#define TDZ_FP64_F32 3

/* operators selectable in tdz_operator_apply */
#define TDZ_MASS 0        /* M  = int B_i B_j                                  */
#define TDZ_HAMILTONIAN 1 /* H  = K[1/m] + s V (+ CAP if present)             */
#define TDZ_DIPOLE_X 2    /* D_x = int x B_i B_j                               */
#define TDZ_DIPOLE_Y 3
#define TDZ_DIPOLE_Z 4
#define TDZ_STAGE 5       /* A = alpha M + g (H + sum_a c_a D_a), see set_stage */

typedef struct tdz_space tdz_space;
typedef struct tdz_op tdz_op;

/* Message of the last failed call on this thread ("" if none). */
const char *tdz_last_error(void);

/* Library version string. */
const char *tdz_version(void);

/* Number of device kernels this library has launched in this process. */
long long tdz_launch_count(void);

/* ---------------------------------------------------------------- space
 * Tensor B-spline space: per axis (x first) a clamped knot vector of
 * nknots[d] values and degree[d]; nquad Gauss-Legendre points per element
 * and axis. Replaces the IGA set-up of src/core.cpp:1787-2046
 * (IGASetQuadrature, IGAAxisSetKnots / IGAAxisInitUniform, IGASetUp).
 */
tdz_status tdz_space_create(int dim, const int *degree, const int *nknots, const double *const *knots,
                            int nquad, tdz_space **out);
/* n basis functions, nel non-empty knot spans and the degree of an axis. */
tdz_status tdz_space_axis(const tdz_space *s, int axis, int *n, int *nel, int *degree);
/* Total number of coefficients (prod_d n_d). */
tdz_status tdz_space_ndof(const tdz_space *s, long long *ndof);
/* Quadrature points and weights (times the element Jacobian) of one axis,
 * nel*nquad values each, element-major (PetIGA IGABasis point/weight*detJac). */
tdz_status tdz_space_quadrature(const tdz_space *s, int axis, double *x, double *w);
/* L2 load vector of one axis: out_i = sum_q w_q B_i(x_q) f(x_q) for complex
 * values f at the quadrature points of the axis (interleaved re/im, nel*nquad
 * of them); out has n complex entries (host arrays). With tdz_operator_mass_solve
 * this is the M-projection of a separable initial state (the wave-packet
 * projection of src/core.cpp:1187-1228, there by CG on the assembled M). */
tdz_status tdz_space_project(const tdz_space *s, int axis, const double *f_q, double *out);
void tdz_space_destroy(tdz_space *s);

/* -------------------------------------------------------------- physics
 * Separable carrier description. The potential and the mass are given as
 * values at the 1D quadrature points, so that every operator is a sum of
 * Kronecker products of 1D banded matrices:
 *   V(r) = sum_d V_d(x_d)                 (pot_q[d], NULL = no term)
 *   1/m  = inv_mass (mass_axis < 0) or 1/m(x_a) on axis a = mass_axis
 *   CAP  = -i cap_inv_mass sum_d W_d(x_d) (cap_q[d], NULL = no layer)
 * The carrier sign s = -charge multiplies V and the field terms
 * (include/tdsez_parser.hpp:86-105,190-194).
 */
typedef struct tdz_physics {
    double charge;              /* q (Charge); s = -q                          */
    double inv_mass;            /* 1/m for a constant mass                      */
    int mass_axis;              /* -1 = constant mass                           */
    const double *inv_mass_q;   /* 1/m at the quadrature points of mass_axis    */
    const double *pot_q[3];     /* V_d at the quadrature points of axis d       */
    const double *cap_q[3];     /* W_d at the quadrature points of axis d       */
    double cap_inv_mass;        /* 1/m scale of the CAP (TDSEZCapMassScale)     */
    int coupled[3];             /* 1 = field couples on this axis (dipole term) */
    int dirichlet;              /* 1 = homogeneous Dirichlet walls (1D only)    */
    int nsoft;                  /* soft-core centres (2D/3D, at most 8)         */
    const double *soft;         /* nsoft x 5: Z, cx, cy, cz, a; adds the non-
                                   separable V(r) = -Z / sqrt(|r - c|^2 + a),
                                   e.g. V = -1/sqrt(x^2+y^2+1), applied by
                                   per-element quadrature (TDSEZFormHam,
                                   src/assembly/assembly.cpp:703-864)        */
} tdz_physics;

/* ------------------------------------------------------------- operator
 * Matrix-free operator set of one space and physics: M, H (K + sV + CAP) and
 * the dipoles D_a as sums of Kronecker products of 1D bands, applied by fused
 * sm_103a kernels. Replaces the assembled AIJ matrices of
 * TDSEZCore::Assemble (src/core.cpp:22-105), TDSEZAssembler
 * (src/assembler_class.cpp:102-272) and the factorised apply of
 * TDSEZTensorOps::Setup (src/tensorops.cpp:16-81).
 */
tdz_status tdz_operator_create(const tdz_space *s, const tdz_physics *phys, tdz_op **out);
/* Stage coefficients of A = alpha M + g (H + sum_a c_a D_a), c over the
 * coupled axes in x, y, z order (nc of them, interleaved re/im). Replaces
 * the value passes BuildStageMatrix / UpdateStageBase / TDSEZFusedStage
 * (src/propagator.cpp:374-551) and the CN IJacobian J = i a M - H - sum c D
 * (src/monitor.cpp:294-331, as alpha = -i a, g = 1 up to the sign). Takes
 * effect for TDZ_STAGE applies issued after the call on any stream. */
tdz_status tdz_operator_set_stage(tdz_op *op, double alpha_re, double alpha_im, double g_re, double g_im,
                                  int nc, const double *c);
/* y = op x. Replaces MatMult on M, H, D_a and the stage matrices
 * (src/propagator.cpp:622-623, src/monitor.cpp:114-116) and
 * TDSEZTensorOps::Apply (src/tensorops.cpp:155-188). x and y must not alias.
 * precision: TDZ_FP32, TDZ_FP64, or TDZ_FP64_DF / TDZ_FP64_F32 (FP64 vectors);
 * FP64 vectors must be 16-byte aligned. */
tdz_status tdz_operator_apply(tdz_op *op, int which, int precision, const void *x, void *y, void *stream);
/* x <- M^-1 x in place (exact Kronecker inverse of the overlap, banded
 * Cholesky line solves), FP32 or FP64 device vector. */
tdz_status tdz_operator_mass_solve(tdz_op *op, int precision, void *x, void *stream);
/* Launch-shape autotuning of the fused 3D apply: with on = 1 (the default)
 * the first apply of each kernel variant and grid size times the candidate
 * tile widths and z chunks on the caller's stream (CUDA events, about 30 ms
 * once) and keeps the fastest; with on = 0 a fixed heuristic picks them. */
void tdz_set_autotune(int on);
/* A fixed launch shape for every fused 3D apply: tile width tile_x (16..32,
 * a multiple of 4) and run length `run` (z planes of the (tile, z) order per
 * CTA, at least 4p); tile_x <= 0 or run <= 0 returns to autotuning. Also set
 * by TDZ_APPLY3D_SHAPE="tile_x,run" in the environment at load time. For
 * reproducing a measured shape and for parity tests at given launch shapes;
 * no counterpart in the reference. */
void tdz_set_apply3d_shape(int tile_x, int run);
/* Observables of a state (FP64 device vector psi) in one call: the monitor
 * products of TDSEZManager::MonitorProducts (src/manager.cpp:584-672) reduced
 * to expectation values. out (host, 2 + 2 + 2 dim doubles):
 *   out[0]            <psi|M|psi>   (the norm; real)
 *   out[1]            0
 *   out[2], out[3]    <psi|H|psi>   (energy; complex with a CAP)
 *   out[4 + 2a], +1   <psi|D_a|psi> (dipole along axis a; a < dim)
 * The applies run in double-float arithmetic (TDZ_FP64_DF) and the
 * reductions are the deterministic FP64 multi-dot; work buffers are allocated
 * on the first call. Synchronises the stream (the values are returned). */
tdz_status tdz_observables(tdz_op *op, const void *psi, double *out, void *stream);
/* Number of fused-apply kernel launches issued so far by this operator. */
long long tdz_operator_launches(const tdz_op *op);
void tdz_operator_destroy(tdz_op *op);

/* --------------------------------------------------------------- solver
 * FGMRES (FP64, right preconditioned) on the stage operator of an operator
 * set, with a preconditioner built on the device. Replaces KSPSetOperators /
 * KSPSolve with the KSP configuration of src/propagator.cpp:125-197,315-370
 * and the multigrid of TDSEZSetupMultigrid (src/multigrid.cpp:205-327).
 * The solve stops when ||b - A x|| <= rtol ||b|| (true residual norm of
 * right-preconditioned FGMRES).
 */
typedef struct tdz_solver tdz_solver;
#define TDZ_PC_NONE 0
#define TDZ_PC_MASS 1 /* exact Kronecker inverse of the overlap M           */
#define TDZ_PC_MG 2   /* geometric B-spline multigrid V-cycle               */
#define TDZ_PC_FDM 3  /* fast diagonalisation: exact inverse (FP32, or FP64
                         with pc_precision = TDZ_FP64) of separable
                         operators: inner axes with only mass and stiffness
                         (the z-layered structure), or, with a constant mass,
                         inner-axis potentials and absorbing layers (complex
                         symmetric axis pencils); terms of other stage
                         scalars on the inner axes (a field along them) and
                         non-separable potentials are left out             */
#define TDZ_PC_BAND 4 /* 1D: exact banded LU with partial pivoting (FP64) of
                         the stage operator, refactored when the refresh rule
                         asks (tdz_pc_refresh_stale) or the end term moves to
                         its next energy                                      */
typedef struct tdz_solver_opts {
    int restart;        /* Krylov restart; 0 = 30, or 50 above 100000 rows   */
    int maxit;          /* iteration cap; 0 = 1000                           */
    double rtol;        /* relative residual; 0 = 1e-12                      */
    int pc;             /* TDZ_PC_*                                          */
    int pc_precision;   /* TDZ_FP32 (mixed precision) or TDZ_FP64            */
    int mg_levels;      /* 0 = coarsen until < 2000 DoFs (MGLevels = 0)      */
    int mg_smooth;      /* Chebyshev degree of pre/post smoothing; 0 = 8     */
    int mg_coarse_its;  /* Chebyshev degree on the coarsest level; 0 = 12    */
    int outer_precision;/* operator applies of the FP64 Krylov method and the
                           step right-hand sides: TDZ_FP64 (also 0) or
                           TDZ_FP64_DF                                        */
    int mg_learned;     /* 1 = learned CNN correction of the coarsest solve
                           (TDZ_PC_MG with FP32 levels; active once trained by
                           tdz_solver_train_coarse)                          */
    int relaxed;        /* 1 = relaxed (inexact) Krylov: the Arnoldi applies
                           A z_j in FP32, the residual b - A x of every
                           restart in outer_precision. A cycle that reports
                           convergence is accepted when the estimate plus
                           the bound sum_j |y_j| gamma |||A||| ||z_j|| on its gap
                           to the true residual meets rtol (rnorm returns
                           that sum), else one more restart residual
                           decides                                           */
    int pc_refresh_its; /* propagators: > 0 also rebuild the preconditioner
                           whenever a stage solve takes more than this many
                           iterations (-tdsez_pc_refresh_its); 0 = only the
                           2 base + 5 rule of tdz_pc_refresh_stale           */
    int mg_coarse;      /* coarsest-level solve of TDZ_PC_MG: 0 = Chebyshev
                           polynomial of degree mg_coarse_its; 1 = the FDM
                           inverse of the coarsest operator when it is exact
                           there (separable stage; the role of the reference's
                           coarse LU, src/multigrid.cpp:314-325), else the
                           polynomial                                         */
} tdz_solver_opts;
/* Set up the solver for the current stage of op (call set_stage first). */
tdz_status tdz_solver_create(tdz_op *op, const tdz_solver_opts *opts, void *stream, tdz_solver **out);
/* Solve A x = b (FP64 device vectors; x holds the initial guess).
 * its / reason / rnorm may be NULL. reason > 0: converged; < 0: diverged
 * (PETSc KSPConvergedReason numbering: -3 iteration cap, -9 NaN/Inf). */
tdz_status tdz_solver_solve(tdz_solver *s, const void *b, void *x, void *stream, int *its, int *reason,
                            double *rnorm);
/* z = P^-1 r: one application of the solver's preconditioner (one V-cycle
 * for TDZ_PC_MG) on FP64 device vectors; the PCShell PCApply of a PETSc
 * adapter (the PCMG V-cycle of src/multigrid.cpp:275-325). */
tdz_status tdz_solver_precondition(tdz_solver *s, const void *r, void *z, void *stream);
void tdz_solver_destroy(tdz_solver *s);

/* Train the learned coarse correction of a TDZ_PC_MG solver created with
 * mg_learned = 1, for the operator's current stage: `pairs` (residual, error)
 * pairs generated at the coarsest level by the solver itself (random coarse
 * right-hand sides, the production Chebyshev coarse solve, a 10x longer
 * solve for the error), then `epochs` passes of Adam (learning rate lr,
 * batches of 8) with the hand-written CNN kernels. *loss (may be NULL): mean
 * relative squared error of the last epoch. No counterpart in the reference
 * (whose coarse solve is a MUMPS LU, src/multigrid.cpp:315-324). */
tdz_status tdz_solver_train_coarse(tdz_solver *s, int pairs, int epochs, float lr, unsigned long long seed,
                                   float *loss, void *stream);
/* Relative error of the coarsest-level solve against a 10x longer solve on
 * `trials` random right-hand sides, without (*plain) and with (*learned) the
 * trained network: what the network gains at its own task. */
tdz_status tdz_solver_coarse_gain(tdz_solver *s, int trials, unsigned long long seed, double *plain,
                                  double *learned, void *stream);

/* out = sum_i conj(x_i) y_i over n complex coefficients (FP32 or FP64 device
 * vectors), accumulated in FP64 by a deterministic two-pass reduction (the
 * VecDot of the Krylov and monitor paths, e.g. <psi|D|psi> after
 * tdz_operator_apply). out: one complex double (16 bytes) in device memory.
 * The per-block partial sums live in library-owned device scratch, one per
 * (device, stream), allocated on the first call on that stream: calls on
 * different streams may overlap, calls on one stream are ordered by it. */
tdz_status tdz_vec_dot(const void *x, const void *y, long long n, int precision, void *out, void *stream);

/* out[i] = sum_j conj(V_i[j]) w[j] for i < k (any k): the fused multi-dot of
 * the classical Gram-Schmidt passes (VecMDot). V: host array of k device
 * vector pointers; out: k complex doubles in device memory. Same reduction
 * and the same per-(device, stream) scratch as tdz_vec_dot (chunks of 16
 * vectors per pass). */
tdz_status tdz_vec_mdot(const void *const *V, int k, const void *w, long long n, int precision, void *out,
                        void *stream);

/* Allocation-free tdz_vec_mdot, for callers that cannot allocate device memory
 * (a host application that owns every device allocation, e.g. a PETSc build
 * with a fixed device pool, or a time step that must not hit cudaMalloc's
 * implicit synchronisation). No counterpart in the reference.
 * The per-block partial sums live in a static device array of the library
 * (8 x 304 complex doubles = 38 KB, held by every GPU that loads the library
 * until the process exits); at most 8 dot products per call, larger k is
 * rejected with TDZ_ERR_ARG. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress); make it before any stream capture.
 * With lazy module loading (CUDA_MODULE_LOADING=LAZY, the default) that
 * first look-up may also load the library's device code onto the device,
 * which the driver does without a cudaMalloc but with memory of its own.
 * The address is then cached for the life of the device's primary context:
 * after cudaDeviceReset the cache is stale, so do not call this entry point
 * after a reset. All calls share the array: calls that overlap on the GPU
 * (different streams, or different host threads on one device) race. Calls
 * no cudaMalloc / cudaFree and no allocating library routine. */
tdz_status tdz_vec_mdot_noalloc(const void *const *V, int k, const void *w, long long n, int precision, void *out,
                                void *stream);

/* Batched complex-by-real transform on the tensor cores (tcgen05, TF32 with
 * a hi/lo split of both operands: FP32 accuracy), the eigenvector transform of the
 * fast-diagonalisation preconditioner; the counterpart of the per-axis
 * contraction of TDSEZTensorOps::Term (src/tensorops.cpp:97-153) for a dense
 * matrix:
 *   out[((p N + n) 2 + c) ldo + r] = sum_k in[((p R + r) 2 + c) ldi + k] B[k N + n]
 * for planes p < planes, rows r < R, parts c (0 real, 1 imaginary), n < N <= 256.
 * B: K x N row-major FP64 host matrix; in/out: FP32 device arrays, 16-byte
 * aligned, ldi a multiple of 4 and >= K, ldo >= R. Uploads B on every call
 * (set-up and tests; the preconditioner keeps its matrices resident). */
tdz_status tdz_plane_transform(const double *B, int K, int N, const float *in, int planes, int R, int ldi, float *out,
                               int ldo, void *stream);

/* ----------------------------------------------------------- propagator
 * Time steps of TDSEZPropagator::Evolve (CN, src/propagator.cpp:78-251) and
 * EvolveRational / Pade22Step (src/propagator.cpp:564-769) on a device state
 * psi (FP64). Field coefficients are the values c_a = s E_a(t) of the
 * coupled axes (TDSEZManager::TermCoefficients, src/manager.cpp:1020-1027):
 *   TDZ_CN, TDZ_PADE22: c1 at t + h/2 (c2 unused)
 *   TDZ_MAGNUS4:        c1 at t + (1/2 - sqrt3/6) h, c2 at t + (1/2 + sqrt3/6) h
 * A failed stage solve returns TDZ_ERR_NOT_CONVERGED / TDZ_ERR_BREAKDOWN
 * (the PetscCheck(reason > 0) of src/propagator.cpp:671-672).
 */
typedef struct tdz_prop tdz_prop;
/* Physical field E_a(t) of axis a (0 on uncoupled axes), a host callback. */
typedef double (*tdz_field_fn)(int axis, double t, void *ctx);
#define TDZ_CN 0
#define TDZ_PADE22 1
#define TDZ_MAGNUS4 2
/* guess_order: 0..5, the initial guess of each stage solve extrapolated from
 * the previous steps (-pade_guess_order, src/propagator.cpp:634-637); -1,
 * the preconditioner's answer x0 = P^-1 b (with the exact FDM inverse this
 * leaves a residual near FP32 rounding, and one FGMRES iteration ends the
 * solve). */
tdz_status tdz_prop_create(tdz_op *op, int kind, const tdz_solver_opts *opts, int guess_order, void *stream,
                           tdz_prop **out);
tdz_status tdz_prop_step(tdz_prop *p, void *psi, double h, const double *c1, const double *c2, void *stream);
/* Batched steps: count independent propagations (each its own tdz_prop, psi,
 * field coefficients c1[i] / c2[i] and stream streams[i]; grids, degrees and
 * physics may differ) advanced by one step h each, concurrently. Host threads
 * (threads; 0 = 16) take the runs from a shared counter and step them on
 * their own streams, so the GPU overlaps the small kernels and host
 * synchronisations of many runs, for intensity and phase scans. Returns the
 * first failure (tdz_last_error names the run); the other runs still step.
 * No counterpart in the reference (one propagation per process there). */
tdz_status tdz_prop_step_batch(int count, tdz_prop *const *props, void *const *psis, double h,
                               const double *const *c1, const double *const *c2, void *const *streams, int threads);

/* Totals: stage solves, Krylov iterations, FP64 operator applies of the
 * solver, multigrid cycles; last solve's iterations and relative residual. */
tdz_status tdz_prop_stats(const tdz_prop *p, long long *solves, long long *its, long long *applies,
                          long long *cycles, int *last_its, double *last_rres);
/* Learned coarse correction trained on the propagation itself (propagators
 * created with TDZ_PC_MG, FP32 levels and mg_learned = 1): record_coarse
 * makes each stage solver's V-cycles store the coarsest-level right-hand side
 * of their next `capacity` cycles (0 stops recording); the steps taken
 * meanwhile are ordinary steps. train_coarse then builds the training pairs
 * from the recorded right-hand sides (production coarse solve, its residual,
 * a 10x longer solve for the error, as tdz_solver_train_coarse) and trains
 * each solver's network; *loss: the largest mean relative loss of the last
 * epoch, *pairs: the pairs used. No counterpart in the reference. */
tdz_status tdz_prop_record_coarse(tdz_prop *p, int capacity);
tdz_status tdz_prop_train_coarse(tdz_prop *p, int epochs, float lr, unsigned long long seed, float *loss,
                                 int *pairs, void *stream);
/* Preconditioner rebuilds the refresh rule asked for (tdz_pc_refresh_stale
 * over the stage solves of this propagator). */
tdz_status tdz_prop_refreshes(const tdz_prop *p, long long *rebuilds);
void tdz_prop_destroy(tdz_prop *p);

/* -------------------------------------------------------------- bound states
 * nev eigenpairs of H c = E M c nearest `target`, in FP64 on the device: the
 * SLEPc Krylov-Schur shift-invert GHEP solve of src/core.cpp:887-1048
 * (shift 1e-3 max(1, |target|) below the target, Krylov-Schur in its
 * Hermitian form: thick-restart Lanczos on (H - s M)^-1 M in the M inner
 * product; inner solves by this library's FGMRES with `inner`'s
 * preconditioner on the stage alpha = -s, g = 1, or, with inner = NULL, the
 * FDM inverse in 3D and the multigrid otherwise, rtol 1e-11). vecs: nev FP64
 * device vectors of ndof coefficients each, back to back; on entry vecs[0]
 * holds a start vector (its real part is used: any real vector not
 * M-orthogonal to the wanted states), on return the M-normalised
 * eigenvectors in ascending energy. energies (host, nev), berr (host, may be
 * NULL): the backward errors ||H v - E M v|| / ((||H|| + |E| ||M||) ||v||)
 * of TDSEZBackwardError (src/core.cpp:474-492) with native FP64 applies and
 * upper bounds of the norms; the reference accepts 1e-8. The Lanczos run
 * stops when every wanted Ritz residual estimate is below tol |theta|, or
 * fails (TDZ_ERR_NOT_CONVERGED) after maxit inner solves. The operator must
 * carry no absorbing layer (H Hermitian); its stage coefficients are
 * overwritten. */
tdz_status tdz_eigen_solve(tdz_op *op, int nev, double target, double tol, int maxit, const tdz_solver_opts *inner,
                           void *vecs, double *energies, double *berr, int *solves, void *stream);

/* Preconditioner refresh rule of TDSEZPCRefresh::Stale
 * (include/tdsez_propagator.hpp:17-31): the preconditioner built from one
 * stage is reused; the first solve after a build sets base, and a solve
 * needing more than 2 base + 5 iterations, or more than cap when cap >= 0
 * (-tdsez_pc_refresh_its), asks for a rebuild. Start from
 * {base = -1, rebuilds = 0, cap}. Host only. */
typedef struct tdz_pc_refresh {
    int base;
    int rebuilds;
    int cap;
} tdz_pc_refresh;
/* Record a solve of `its` iterations; returns 1 when the preconditioner
 * should be rebuilt before the next solve, else 0. */
int tdz_pc_refresh_stale(tdz_pc_refresh *r, int its);

/* Strong-field check of TDSEZSetupMultigrid (src/multigrid.cpp:213-237):
 * *ratio = tau max_t sum_a |E_a(t)| L_a over 4 T / dt + 1 samples of [0, T],
 * with L_a = max(|lo_a|, |hi_a|) of the space's box and tau the stage scale
 * of the propagator kind (CN dt/2, Pade(2,2) dt/sqrt12, Magnus-4
 * dt/(2 sqrt12)); field(a, t, ctx) returns the physical field. Above 1.5 the
 * field term dominates the stage operator and multigrid may not converge
 * (the reference warns; the host layer here does the same). Host only. */
tdz_status tdz_strong_field_ratio(const tdz_space *s, int kind, double dt, double final_time, tdz_field_fn field,
                                  void *ctx, double *ratio);

/* --------------------------------------------------------------- t-SURFF
 * Photoelectron amplitudes from the surface flux through the box |x_d| = R
 * (TDSEZTSurff, include/tdsez_tsurff.hpp, src/tsurff.cpp:112-559): surface
 * Gauss points of every knot span inside [-R, R], trace of psi and
 * (1/m) d_n psi, Volkov integrals A' = -s E, B' = A, C' = |A|^2/2m + V0 by
 * RK4 substeps of at most dt/2, flux on the momentum grid factorised by axis
 * (FluxGrid), trapezoid accumulation over samples (AddFlux). Momenta are
 * ordered k_x slowest, k_z fastest. The field callback returns the physical
 * field E_a(t) (0 on uncoupled axes).
 */
typedef struct tdz_tsurff tdz_tsurff;
typedef struct tdz_tsurff_opts {
    double radius;      /* SurffRadius R                                     */
    int nquad;          /* Gauss points per span on the surface; 0 = space's */
    int nk[3];          /* momentum grid points per axis (used axes)          */
    double kmin[3], kmax[3];
    double mass;        /* exterior mass                                     */
    double v0;          /* exterior carrier potential s V (Ha)               */
    double charge;      /* q; s = -q                                         */
    double dt;          /* TimeStep                                          */
} tdz_tsurff_opts;
tdz_status tdz_tsurff_create(const tdz_space *s, const tdz_tsurff_opts *o, tdz_field_fn field, void *ctx,
                             tdz_tsurff **out);
/* Add the flux of psi (FP64 device vector) at time t (increasing). */
tdz_status tdz_tsurff_sample(tdz_tsurff *ts, double t, const void *psi, void *stream);
/* Accumulated amplitudes b(k), prod(nk) complex values (host array). */
tdz_status tdz_tsurff_amplitudes(tdz_tsurff *ts, double *out, void *stream);
/* Projection of psi (FP64 device vector, normally psi(T)) inside the box
 * |x_d| < R onto the Volkov states at the last sample time: the interior term
 * of TDSEZTSurff::Interior / Project (src/tsurff.cpp:565-639),
 *   phi(k) sum_ijl c_ijl F_x[k_x][i] F_y[k_y][j] F_z[k_z][l],
 *   F_d[k][i] = sum_q w_q exp(-i (k + A_d) x_q) B_i(x_q) over the in-box nodes,
 *   phi(k) = (2 pi)^(-d/2) exp(i (C + T |k|^2 / 2m + k.B / m)),
 * with the axis contractions on the device (double-float arithmetic). Adding
 * it to tdz_tsurff_amplitudes gives the spectrum of a run that ends before
 * all of the wave packet has left the box. out (host): prod(nk) complex
 * values, k_x slowest. Synchronises the stream. */
tdz_status tdz_tsurff_interior(tdz_tsurff *ts, const void *psi, double *out, void *stream);
/* End term: the flux still to cross the surface after the last sample time
 * T, for a run that ends after the pulse (TDSEZTSurff::EndTerm,
 * src/tsurff.cpp:650-976; SurffEndTerm = 1). With the field off after T,
 *   b_end(k) = flux_k(T)[phi_E],  (E M - H) phi_E = i M psi(T),  E = |k + A(T)|^2/2m + V0,
 * H the field-free Hamiltonian of op including its absorbing layer (required:
 * it is the outgoing-wave condition). phi_E is solved on energy nodes uniform
 * in p = |k + A(T)| (spacing dp; automatic: min(grid spacing, 0.25/(R sqrt d)),
 * refined to 0.25/(L sqrt d) below 2 k_cap, k_cap = 6.555 / cap_width, L the
 * largest box half-width) and the node fluxes are combined with four-point
 * Lagrange weights in p. Every node is one FGMRES solve (FP64, relative
 * residual rtol) on the device, warm-started from the previous node, with
 * the preconditioner of `inner` (NULL: the exact banded LU in 1D, the FP64
 * FDM inverse in 2D/3D, built for the damped pole E (1 + i eta) when it is not
 * exact; an exact FP32 inverse that stagnates at a nearly singular node is
 * replaced by the damped pole for that node). psi: psi(T) (FP64 device
 * vector), sampled at T before the call. out (host): prod(nk) complex
 * values, k_x slowest, to be added to tdz_tsurff_amplitudes. stats (host,
 * may be NULL, 7 doubles): nodes, total FGMRES iterations, largest per node,
 * largest node spacing, eta used, seconds, nodes that needed the damped pole. Fails (TDZ_ERR_ARG) when the field is not over at T. The
 * operator's stage coefficients are overwritten. */
typedef struct tdz_tsurff_end_opts {
    double dp;          /* node spacing in p (SurffEndTermDk); 0 = automatic  */
    double cap_width;   /* absorbing-layer width; needed when dp = 0          */
    double eta;         /* preconditioner pole damping; < 0 = automatic      */
    double rtol;        /* per-node relative residual; 0 = 1e-10              */
    int maxit;          /* per-node FGMRES iterations; 0 = 600                */
} tdz_tsurff_end_opts;
tdz_status tdz_tsurff_end_term(tdz_tsurff *ts, tdz_op *op, const tdz_solver_opts *inner,
                               const tdz_tsurff_end_opts *o, const void *psi, double *out, double *stats,
                               void *stream);
/* Volkov integrals at the last sample: A[3], B[3], C, t (8 doubles). */
tdz_status tdz_tsurff_volkov(const tdz_tsurff *ts, double *abct);
/* What the spectra file records about the sampler (the attributes of
 * src/tsurff.cpp:1044-1053), 8 doubles: last sample time, radius, exterior
 * mass, exterior potential, number of surface points (Gauss nodes on the
 * 2 dim faces |x_a| = R, src/tsurff.cpp:152-179), number of samples, number
 * of momenta, dimension. */
tdz_status tdz_tsurff_info(const tdz_tsurff *ts, double *info);
void tdz_tsurff_destroy(tdz_tsurff *ts);

/* ------------------------------------------------------ learned correction
 * Small 3D convolutional network (3x3x3 convolutions, zero padding, ReLU
 * between layers, BF16 weights, FP32 accumulation) with hand-written
 * forward, backward and Adam kernels. It is trained on residual/error pairs
 * that the solver generates and serves as a learned coarse correction inside
 * the multigrid cycle (no counterpart in the reference, which has ASM/ILU
 * and PCMG only). Tensors are FP32 device arrays [batch][channel][D][H][W].
 */
typedef struct tdz_cnn tdz_cnn;
tdz_status tdz_cnn_create(int cin, int width, int cout, int layers, int D, int H, int W, int batch,
                          unsigned long long seed, tdz_cnn **out);
tdz_status tdz_cnn_forward(tdz_cnn *n, const float *in, float *out, int batch, void *stream);
/* One Adam step on the relative MSE sum_b ||y_b - t_b||^2 / ||t_b||^2 / B. */
tdz_status tdz_cnn_train_step(tdz_cnn *n, const float *in, const float *target, int batch, float lr, void *stream);
/* Loss accumulated since the last call (resets it). */
tdz_status tdz_cnn_loss(tdz_cnn *n, float *loss, void *stream);
/* Number of parameters; get / set the FP32 master parameters (per layer:
 * weights [co][ci][3][3][3], then bias [co]); gradients of the last step. */
tdz_status tdz_cnn_num_params(const tdz_cnn *n, long long *count);
tdz_status tdz_cnn_get_params(const tdz_cnn *n, float *host);
tdz_status tdz_cnn_set_params(tdz_cnn *n, const float *host);
tdz_status tdz_cnn_get_grads(const tdz_cnn *n, float *host);
void tdz_cnn_destroy(tdz_cnn *n);

/* --------------------------------------------------------- output files
 * HDF5 files of the reference's output schema, written by the library
 * itself (host only, no HDF5 library): the classic layout that every HDF5
 * reader opens (version-0 superblock, one root group, contiguous float64
 * datasets, float64 attributes on the root group).
 *
 * tdz_h5_write: a flat file, as the t-SURFF spectra writer makes it
 * (WriteReal / WriteAttribute, src/tsurff.cpp:74-92,1018-1057). Dataset i
 * is names[i] of rank ranks[i] (1..8), its extents the next ranks[i]
 * entries of dims (slowest first, each >= 1), its values data[i]
 * (row-major). Attribute j is attr_names[j], a rank-1 array of attr_lens[j]
 * values attr_data[j]. The file is written beside `path` and renamed over
 * it; parent directories are created. */
tdz_status tdz_h5_write(const char *path, int ndatasets, const char *const *names, const int *ranks,
                        const long long *dims, const double *const *data, int nattrs, const char *const *attr_names,
                        const long long *attr_lens, const double *const *attr_data);

/* The observables file of a propagation (td/<name>_observables.h5):
 * TDSEZManager::WriteHDF5 (src/manager.cpp:51-201). Five float64 datasets,
 * one row per recorded step: dipoles (1 + 3 dim columns: t, E_a, D_a, A_a),
 * populations (1 + n_bound: t, P_n), energies (7: t, Kin, Pot, Int, Tot,
 * InvMass, Norm), currents (11, or 15 in 3D) and autocorrelation (3: t,
 * Re C, Im C). Rows are buffered on the host; the file is rewritten with
 * every row so far when flush_rows rows are pending (<= 0: 5000, the
 * reference's buffer), on tdz_obsfile_flush and on tdz_obsfile_close, the
 * first write replacing any file at `path`. The reference appends to
 * chunked, extendable datasets instead; readers see the same arrays. A
 * handle is used by one thread at a time (the reference writes from rank 0
 * only); different handles are independent. */
typedef struct tdz_obsfile tdz_obsfile;
#define TDZ_OBS_DIPOLES 0
#define TDZ_OBS_POPULATIONS 1
#define TDZ_OBS_ENERGIES 2
#define TDZ_OBS_CURRENTS 3
#define TDZ_OBS_AUTOCORRELATION 4
tdz_status tdz_obsfile_open(const char *path, int dim, int n_bound, long long flush_rows, tdz_obsfile **out);
/* Columns of dataset `set` (TDZ_OBS_*), time column included; -1 for an
 * unknown set. */
int tdz_obsfile_columns(const tdz_obsfile *f, int set);
/* Appends one row at time t to every dataset: rows[set] holds the
 * columns(set) - 1 values after the time column, or is NULL (zeros); rows
 * may be NULL. */
tdz_status tdz_obsfile_record(tdz_obsfile *f, double t, const double *const *rows);
/* Rows recorded, and rows already in the file. */
tdz_status tdz_obsfile_rows(const tdz_obsfile *f, long long *recorded, long long *written);
tdz_status tdz_obsfile_flush(tdz_obsfile *f);
/* Flushes and frees the handle (freed also when the flush fails). */
tdz_status tdz_obsfile_close(tdz_obsfile *f);

#ifdef __cplusplus
}
#endif

#endif /* TDZ_H */
