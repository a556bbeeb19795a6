// extern "C" boundary of the tdz library: every entry point catches the C++
// error of its body and returns a status code; the message is kept per thread
// for tdz_last_error(). Mirrors the PetscErrorCode / PetscCall convention of
// the reference (every call returns a code, no exception crosses the ABI).
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "oper.h"
#include "prop.h"
#include "tgemm.h"
#include "tsurff.h"
#include "cnn.h"
#include "h5file.h"

struct tdz_space {
    tdz::Space s;
};
struct tdz_op {
    tdz::Operator o;
    std::unique_ptr<tdz::KronSolve> minv;
};
struct tdz_solver {
    tdz::Solver s;
};
struct tdz_prop {
    tdz::Propagator p;
};
struct tdz_tsurff {
    tdz::TSurff t;
};
struct tdz_cnn {
    tdz::CNN n;
};
struct tdz_obsfile {
    tdz::ObsFile f;
};

namespace tdz {
static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
static std::atomic<long long> g_launches{0};
void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
int sm_count() {
    static std::mutex mu;
    static std::map<int, int> cache;
    int dev = 0;
    TDZ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int n = 0;
    TDZ_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    n = std::max(1, n);
    cache[dev] = n;
    return n;
}
}  // namespace tdz

template <class F> static tdz_status guarded(F &&f) {
    try {
        f();
        tdz::g_last_error.clear();
        return TDZ_OK;
    } catch (const tdz::Error &e) {
        tdz::set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        tdz::set_last_error("host allocation failed");
        return TDZ_ERR_INTERNAL;
    } catch (const std::exception &e) {
        tdz::set_last_error(e.what());
        return TDZ_ERR_INTERNAL;
    }
}

extern "C" {

const char *tdz_last_error(void) { return tdz::g_last_error.c_str(); }

const char *tdz_version(void) { return "tdz 0.1 (sm_103a)"; }

long long tdz_launch_count(void) { return tdz::launch_count(); }

tdz_status tdz_space_create(int dim, const int *degree, const int *nknots, const double *const *knots, int nquad,
                            tdz_space **out) {
    return guarded([&] {
        TDZ_CHECK(out, TDZ_ERR_ARG, "out is null");
        *out = nullptr;
        TDZ_CHECK(dim >= 1 && dim <= 3, TDZ_ERR_ARG, "dim must be 1, 2 or 3");
        TDZ_CHECK(degree && nknots && knots, TDZ_ERR_ARG, "null axis description");
        auto h = std::make_unique<tdz_space>();
        h->s.dim = dim;
        h->s.nquad = nquad;
        for (int d = 0; d < dim; ++d) {
            TDZ_CHECK(knots[d], TDZ_ERR_ARG, "null knot vector");
            h->s.ax[d].setup(knots[d], nknots[d], degree[d], nquad);
        }
        *out = h.release();
    });
}

tdz_status tdz_space_axis(const tdz_space *s, int axis, int *n, int *nel, int *degree) {
    return guarded([&] {
        TDZ_CHECK(s, TDZ_ERR_ARG, "space is null");
        TDZ_CHECK(axis >= 0 && axis < s->s.dim, TDZ_ERR_ARG, "axis out of range");
        const tdz::Axis1D &a = s->s.ax[axis];
        if (n) *n = a.n;
        if (nel) *nel = a.nel;
        if (degree) *degree = a.p;
    });
}

tdz_status tdz_space_ndof(const tdz_space *s, long long *ndof) {
    return guarded([&] {
        TDZ_CHECK(s && ndof, TDZ_ERR_ARG, "null argument");
        *ndof = s->s.ndof();
    });
}

tdz_status tdz_space_quadrature(const tdz_space *s, int axis, double *x, double *w) {
    return guarded([&] {
        TDZ_CHECK(s, TDZ_ERR_ARG, "space is null");
        TDZ_CHECK(axis >= 0 && axis < s->s.dim, TDZ_ERR_ARG, "axis out of range");
        const tdz::Axis1D &a = s->s.ax[axis];
        if (x) std::memcpy(x, a.xq.data(), a.xq.size() * sizeof(double));
        if (w) std::memcpy(w, a.wq.data(), a.wq.size() * sizeof(double));
    });
}

tdz_status tdz_space_project(const tdz_space *s, int axis, const double *f_q, double *out) {
    return guarded([&] {
        TDZ_CHECK(s && f_q && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(axis >= 0 && axis < s->s.dim, TDZ_ERR_ARG, "axis out of range");
        const tdz::Axis1D &a = s->s.ax[axis];
        std::vector<tdz::cd> acc(a.n, 0.0);
        const int np = a.p + 1;
        for (int e = 0; e < a.nel; ++e)
            for (int q = 0; q < a.nq; ++q) {
                const size_t k = (size_t)e * a.nq + q;
                const tdz::cd f(f_q[2 * k], f_q[2 * k + 1]);
                for (int r = 0; r < np; ++r) acc[a.offset[e] + r] += a.wq[k] * a.N[k * np + r] * f;
            }
        for (int i = 0; i < a.n; ++i) { out[2 * i] = acc[i].real(); out[2 * i + 1] = acc[i].imag(); }
    });
}

void tdz_space_destroy(tdz_space *s) { delete s; }

tdz_status tdz_operator_create(const tdz_space *s, const tdz_physics *phys, tdz_op **out) {
    return guarded([&] {
        TDZ_CHECK(s && phys && out, TDZ_ERR_ARG, "null argument");
        *out = nullptr;
        auto h = std::make_unique<tdz_op>();
        h->o.build(s->s, *phys);
        *out = h.release();
    });
}

tdz_status tdz_operator_set_stage(tdz_op *op, double alpha_re, double alpha_im, double g_re, double g_im, int nc,
                                  const double *c) {
    return guarded([&] {
        TDZ_CHECK(op, TDZ_ERR_ARG, "operator is null");
        TDZ_CHECK(nc >= 0 && nc <= 3 && (nc == 0 || c), TDZ_ERR_ARG, "bad field coefficients");
        std::vector<tdz::cd> cc(nc);
        for (int k = 0; k < nc; ++k) cc[k] = tdz::cd(c[2 * k], c[2 * k + 1]);
        op->o.set_stage(tdz::cd(alpha_re, alpha_im), tdz::cd(g_re, g_im), cc);
    });
}

tdz_status tdz_operator_apply(tdz_op *op, int which, int precision, const void *x, void *y, void *stream) {
    return guarded([&] {
        TDZ_CHECK(op, TDZ_ERR_ARG, "operator is null");
        op->o.apply(which, precision, x, y, static_cast<cudaStream_t>(stream));
    });
}

tdz_status tdz_operator_mass_solve(tdz_op *op, int precision, void *x, void *stream) {
    return guarded([&] {
        TDZ_CHECK(op && x, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(precision == TDZ_FP32 || precision == TDZ_FP64, TDZ_ERR_ARG, "bad precision");
        if (!op->minv) {
            auto ks = std::make_unique<tdz::KronSolve>();
            std::array<const tdz::BandD *, 3> mb{nullptr, nullptr, nullptr};
            for (int d = 0; d < op->o.sp->dim; ++d) mb[d] = &op->o.bases[d][tdz::kM];
            ks->setup(mb, op->o.sp->dim);
            op->minv = std::move(ks);
        }
        op->minv->apply(x, precision, static_cast<cudaStream_t>(stream));
        TDZ_CUDA(cudaGetLastError());
    });
}

long long tdz_operator_launches(const tdz_op *op) { return op ? op->o.launches : 0; }

void tdz_operator_destroy(tdz_op *op) { delete op; }

namespace {
// Reduction scratch of tdz_vec_dot / tdz_vec_mdot, one per (device, stream),
// allocated and initialised on first use under the lock: calls on different
// streams never share partial sums, calls on one stream are ordered by it.
std::mutex g_dot_mu;
std::map<std::pair<int, cudaStream_t>, std::unique_ptr<tdz::blas::Reducer>> g_dot_scratch;

tdz::blas::Reducer *dot_scratch(cudaStream_t st) {
    int dev = 0;
    TDZ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_dot_mu);
    auto &slot = g_dot_scratch[{dev, st}];
    if (!slot) {
        auto r = std::make_unique<tdz::blas::Reducer>();
        r->init();
        slot = std::move(r);
    }
    return slot.get();
}
}  // namespace

tdz_status tdz_vec_dot(const void *x, const void *y, long long n, int precision, void *out, void *stream) {
    return guarded([&] {
        TDZ_CHECK(x && y && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(n >= 0, TDZ_ERR_ARG, "negative length");
        TDZ_CHECK(precision == TDZ_FP32 || precision == TDZ_FP64, TDZ_ERR_ARG, "bad precision");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        tdz::blas::Reducer *r = dot_scratch(st);
        tdz::blas::dot_device(*r, x, y, (size_t)n, precision, static_cast<double2 *>(out), st);
    });
}

tdz_status tdz_vec_mdot(const void *const *V, int k, const void *w, long long n, int precision, void *out,
                        void *stream) {
    return guarded([&] {
        TDZ_CHECK(V && w && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(k >= 1 && n >= 0, TDZ_ERR_ARG, "bad sizes");
        TDZ_CHECK(precision == TDZ_FP32 || precision == TDZ_FP64, TDZ_ERR_ARG, "bad precision");
        for (int i = 0; i < k; ++i) TDZ_CHECK(V[i], TDZ_ERR_ARG, "null vector in V");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        tdz::blas::Reducer *r = dot_scratch(st);
        double2 *o = static_cast<double2 *>(out);
        for (int c0 = 0; c0 < k; c0 += tdz::blas::kMaxDot) {
            const int kk = std::min(tdz::blas::kMaxDot, k - c0);
            tdz::blas::mdot_partials(V + c0, kk, w, (size_t)n, precision, r->partial.as<double2>(), r->blocks, o + c0, st);
        }
    });
}

tdz_status tdz_vec_mdot_noalloc(const void *const *V, int k, const void *w, long long n, int precision, void *out,
                                void *stream) {
    return guarded([&] {
        TDZ_CHECK(V && w && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(n >= 0, TDZ_ERR_ARG, "negative length");
        TDZ_CHECK(precision == TDZ_FP32 || precision == TDZ_FP64, TDZ_ERR_ARG, "bad precision");
        for (int i = 0; i < k; ++i) TDZ_CHECK(V[i], TDZ_ERR_ARG, "null vector in V");
        tdz::mdot_noalloc(V, k, w, (size_t)n, precision, static_cast<double2 *>(out), static_cast<cudaStream_t>(stream));
    });
}

static tdz::SolverOptions solver_options(const tdz_solver_opts *o) {
    tdz::SolverOptions so;
    if (!o) return so;
    so.restart = o->restart;
    so.maxit = o->maxit > 0 ? o->maxit : 1000;
    so.rtol = o->rtol > 0 ? o->rtol : 1e-12;
    so.pc = o->pc;
    so.pc_precision = o->pc_precision;
    TDZ_CHECK(so.pc_precision == TDZ_FP32 || so.pc_precision == TDZ_FP64, TDZ_ERR_ARG, "bad pc_precision");
    so.mg.levels = o->mg_levels;
    so.mg.smooth = o->mg_smooth > 0 ? o->mg_smooth : 8;
    so.mg.coarse_its = o->mg_coarse_its > 0 ? o->mg_coarse_its : 12;
    so.outer = o->outer_precision == 0 ? TDZ_FP64 : o->outer_precision;
    so.mg.learned = o->mg_learned;
    so.relaxed = o->relaxed != 0;
    so.pc_refresh_its = o->pc_refresh_its > 0 ? o->pc_refresh_its : -1;
    TDZ_CHECK(o->mg_coarse == 0 || o->mg_coarse == 1, TDZ_ERR_ARG, "mg_coarse must be 0 or 1");
    so.mg.coarse_fdm = o->mg_coarse;
    TDZ_CHECK(so.outer == TDZ_FP64 || so.outer == TDZ_FP64_DF, TDZ_ERR_ARG,
              "outer_precision must be TDZ_FP64 or TDZ_FP64_DF");
    return so;
}

tdz_status tdz_plane_transform(const double *B, int K, int N, const float *in, int planes, int R, int ldi, float *out,
                               int ldo, void *stream) {
    return guarded([&] {
        TDZ_CHECK(B && in && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(K >= 1 && N >= 1 && planes >= 1 && R >= 1, TDZ_ERR_ARG, "sizes must be positive");
        TDZ_CHECK(ldi % 4 == 0 && ldi >= K && ldo >= R, TDZ_ERR_ARG, "bad pitches");
        tdz::TransformMat T;
        T.build(std::vector<double>(B, B + (size_t)K * N), K, N);
        tdz::transform(T, in, planes, R, ldi, out, ldo, static_cast<cudaStream_t>(stream));
        TDZ_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
        TDZ_CHECK(tdz::take_transform_error() == 0, TDZ_ERR_CUDA, "tensor-core transform: a bounded wait ran out");
    });
}

void tdz_set_autotune(int on) { tdz::set_autotune(on); }

void tdz_set_apply3d_shape(int tile_x, int run) { tdz::set_forced_shape(tile_x, run); }

tdz_status tdz_observables(tdz_op *op, const void *psi, double *out, void *stream) {
    return guarded([&] {
        TDZ_CHECK(op && psi && out, TDZ_ERR_ARG, "null argument");
        std::vector<tdz::cd> v;
        op->o.observables(static_cast<const double2 *>(psi), v, static_cast<cudaStream_t>(stream));
        out[0] = v[0].real();
        out[1] = 0.0;
        for (size_t i = 1; i < v.size(); ++i) {
            out[2 * i] = v[i].real();
            out[2 * i + 1] = v[i].imag();
        }
    });
}

tdz_status tdz_solver_create(tdz_op *op, const tdz_solver_opts *opts, void *stream, tdz_solver **out) {
    return guarded([&] {
        TDZ_CHECK(op && out, TDZ_ERR_ARG, "null argument");
        *out = nullptr;
        TDZ_CHECK(op->o.stage_set, TDZ_ERR_STATE, "stage coefficients not set");
        auto h = std::make_unique<tdz_solver>();
        h->s.setup(&op->o, solver_options(opts), static_cast<cudaStream_t>(stream));
        *out = h.release();
    });
}

tdz_status tdz_solver_solve(tdz_solver *s, const void *b, void *x, void *stream, int *its, int *reason,
                            double *rnorm) {
    return guarded([&] {
        TDZ_CHECK(s && b && x, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(b != x, TDZ_ERR_ARG, "b and x must not alias");
        tdz::SolveStats st = s->s.solve(static_cast<const double2 *>(b), static_cast<double2 *>(x),
                                        static_cast<cudaStream_t>(stream));
        if (its) *its = st.its;
        if (reason) *reason = st.reason;
        if (rnorm) *rnorm = st.rnorm;
    });
}

static tdz::Multigrid *learned_mg(tdz_solver *s) {
    TDZ_CHECK(s, TDZ_ERR_ARG, "null solver");
    TDZ_CHECK(s->s.opt.pc == TDZ_PC_MG, TDZ_ERR_STATE, "the learned coarse correction needs TDZ_PC_MG");
    auto *mg = static_cast<tdz::Multigrid *>(s->s.pc.get());
    TDZ_CHECK(mg->lrn.on, TDZ_ERR_STATE, "solver created without mg_learned (or with FP64 levels)");
    return mg;
}

tdz_status tdz_solver_train_coarse(tdz_solver *s, int pairs, int epochs, float lr, unsigned long long seed,
                                   float *loss, void *stream) {
    return guarded([&] {
        tdz::Multigrid *mg = learned_mg(s);
        TDZ_CHECK(lr > 0.f && std::isfinite(lr), TDZ_ERR_ARG, "learning rate must be positive");
        const float l = mg->train_coarse(pairs, epochs, lr, seed, static_cast<cudaStream_t>(stream));
        if (loss) *loss = l;
    });
}

tdz_status tdz_solver_coarse_gain(tdz_solver *s, int trials, unsigned long long seed, double *plain,
                                  double *learned, void *stream) {
    return guarded([&] {
        tdz::Multigrid *mg = learned_mg(s);
        TDZ_CHECK(trials >= 1, TDZ_ERR_ARG, "trials must be positive");
        const auto g = mg->coarse_gain(trials, seed, static_cast<cudaStream_t>(stream));
        if (plain) *plain = g.first;
        if (learned) *learned = g.second;
    });
}

tdz_status tdz_solver_precondition(tdz_solver *s, const void *r, void *z, void *stream) {
    return guarded([&] {
        TDZ_CHECK(s && r && z, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(r != z, TDZ_ERR_ARG, "r and z must not alias");
        s->s.pc->apply(static_cast<const double2 *>(r), static_cast<double2 *>(z), static_cast<cudaStream_t>(stream));
    });
}

void tdz_solver_destroy(tdz_solver *s) { delete s; }

tdz_status tdz_prop_create(tdz_op *op, int kind, const tdz_solver_opts *opts, int guess_order, void *stream,
                           tdz_prop **out) {
    return guarded([&] {
        TDZ_CHECK(op && out, TDZ_ERR_ARG, "null argument");
        *out = nullptr;
        auto h = std::make_unique<tdz_prop>();
        if (!op->o.stage_set) op->o.set_stage(1.0, 0.0, std::vector<tdz::cd>(op->o.coupled.size()));
        h->p.setup(&op->o, kind, solver_options(opts), guess_order, static_cast<cudaStream_t>(stream));
        *out = h.release();
    });
}

tdz_status tdz_prop_step(tdz_prop *p, void *psi, double h, const double *c1, const double *c2, void *stream) {
    return guarded([&] {
        TDZ_CHECK(p && psi, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(h > 0.0 && std::isfinite(h), TDZ_ERR_ARG, "time step must be positive");
        const size_t nc = p->p.op->coupled.size();
        std::vector<tdz::cd> a(nc), b(nc);
        for (size_t k = 0; k < nc; ++k) {
            TDZ_CHECK(c1 != nullptr, TDZ_ERR_ARG, "field coefficients required");
            a[k] = c1[k];
            if (p->p.kind == TDZ_MAGNUS4) {
                TDZ_CHECK(c2 != nullptr, TDZ_ERR_ARG, "Magnus-4 needs two sets of field coefficients");
                b[k] = c2[k];
            }
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        double2 *v = static_cast<double2 *>(psi);
        if (p->p.kind == TDZ_CN) p->p.cn_step(v, h, a, st);
        else if (p->p.kind == TDZ_PADE22) p->p.pade_step(v, h, a, 0, st);
        else p->p.magnus_step(v, h, a, b, st);
    });
}

tdz_status tdz_prop_step_batch(int count, tdz_prop *const *props, void *const *psis, double h,
                               const double *const *c1, const double *const *c2, void *const *streams, int threads) {
    if (count < 0 || (count > 0 && (!props || !psis || !streams))) {
        tdz::set_last_error("bad batch arguments");
        return TDZ_ERR_ARG;
    }
    const int nt = std::max(1, std::min(threads > 0 ? threads : 16, std::max(count, 1)));
    std::atomic<int> next{0};
    std::mutex mu;
    tdz_status first = TDZ_OK;
    std::string first_msg;
    auto worker = [&]() {
        while (true) {
            const int i = next.fetch_add(1);
            if (i >= count) break;
            const tdz_status s = tdz_prop_step(props[i], psis[i], h, c1 ? c1[i] : nullptr, c2 ? c2[i] : nullptr,
                                               streams[i]);
            if (s != TDZ_OK) {
                std::lock_guard<std::mutex> lk(mu);
                if (first == TDZ_OK) {
                    first = s;
                    first_msg = "batch run " + std::to_string(i) + ": " + tdz_last_error();
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < nt; ++k) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    if (first != TDZ_OK) tdz::set_last_error(first_msg);
    return first;
}

tdz_status tdz_prop_stats(const tdz_prop *p, long long *solves, long long *its, long long *applies, long long *cycles,
                          int *last_its, double *last_rres) {
    return guarded([&] {
        TDZ_CHECK(p, TDZ_ERR_ARG, "null argument");
        long long ap = 0, cy = 0;
        for (int k = 0; k < p->p.nsolvers; ++k) {
            ap += p->p.solver[k].ksp.applies;
            if (auto *mg = dynamic_cast<const tdz::Multigrid *>(p->p.solver[k].pc.get())) cy += mg->cycles;
        }
        if (solves) *solves = p->p.solves;
        if (its) *its = p->p.its;
        if (applies) *applies = ap;
        if (cycles) *cycles = cy;
        if (last_its) *last_its = p->p.last.its;
        if (last_rres) *last_rres = p->p.last.bnorm > 0 ? p->p.last.rnorm / p->p.last.bnorm : 0.0;
    });
}

tdz_status tdz_eigen_solve(tdz_op *op, int nev, double target, double tol, int maxit, const tdz_solver_opts *inner,
                           void *vecs, double *energies, double *berr, int *solves, void *stream) {
    return guarded([&] {
        TDZ_CHECK(op && vecs && energies, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(tol > 0.0 && maxit > 0, TDZ_ERR_ARG, "tol and maxit must be positive");
        TDZ_CHECK(reinterpret_cast<uintptr_t>(vecs) % 16 == 0, TDZ_ERR_ARG, "vecs must be 16-byte aligned");
        tdz::SolverOptions so;
        if (inner) {
            so = solver_options(inner);
        } else {   // exact FDM inverse for 3D, multigrid otherwise; FP32 inside FP64 FGMRES
            so.pc = op->o.sp->dim == 3 ? TDZ_PC_FDM : TDZ_PC_MG;
            so.rtol = 1e-11;
            so.outer = TDZ_FP64_DF;
        }
        const tdz::EigenResult r = tdz::eigen_solve(op->o, nev, target, tol, maxit, so, static_cast<double2 *>(vecs),
                                                    static_cast<cudaStream_t>(stream));
        for (int i = 0; i < nev; ++i) {
            energies[i] = r.energies[i];
            if (berr) berr[i] = r.berr[i];
        }
        if (solves) *solves = r.solves;
    });
}

static std::vector<tdz::Multigrid *> prop_learned_mgs(tdz_prop *p) {
    TDZ_CHECK(p, TDZ_ERR_ARG, "null propagator");
    std::vector<tdz::Multigrid *> out;
    for (int k = 0; k < p->p.nsolvers; ++k) {
        TDZ_CHECK(p->p.solver[k].opt.pc == TDZ_PC_MG, TDZ_ERR_STATE, "the learned coarse correction needs TDZ_PC_MG");
        auto *mg = static_cast<tdz::Multigrid *>(p->p.solver[k].pc.get());
        TDZ_CHECK(mg->lrn.on, TDZ_ERR_STATE, "propagator created without mg_learned (or with FP64 levels)");
        out.push_back(mg);
    }
    return out;
}

tdz_status tdz_prop_record_coarse(tdz_prop *p, int capacity) {
    return guarded([&] {
        for (tdz::Multigrid *mg : prop_learned_mgs(p)) mg->record_coarse(capacity);
    });
}

tdz_status tdz_prop_train_coarse(tdz_prop *p, int epochs, float lr, unsigned long long seed, float *loss,
                                 int *pairs, void *stream) {
    return guarded([&] {
        TDZ_CHECK(lr > 0.f && std::isfinite(lr) && epochs >= 1, TDZ_ERR_ARG, "bad epochs or learning rate");
        float l = 0.f;
        int np = 0;
        for (tdz::Multigrid *mg : prop_learned_mgs(p)) {
            np += mg->lrn.rec_n;
            l = std::max(l, mg->train_recorded(epochs, lr, seed, static_cast<cudaStream_t>(stream)));
        }
        if (loss) *loss = l;
        if (pairs) *pairs = np;
    });
}

tdz_status tdz_prop_refreshes(const tdz_prop *p, long long *rebuilds) {
    return guarded([&] {
        TDZ_CHECK(p && rebuilds, TDZ_ERR_ARG, "null argument");
        *rebuilds = (long long)p->p.refresh[0].rebuilds + p->p.refresh[1].rebuilds;
    });
}

void tdz_prop_destroy(tdz_prop *p) { delete p; }

int tdz_pc_refresh_stale(tdz_pc_refresh *r, int its) {
    if (!r) return 0;
    tdz::PCRefresh f;
    f.base = r->base;
    f.rebuilds = r->rebuilds;
    f.cap = r->cap;
    const bool stale = f.stale(its);
    r->base = f.base;
    r->rebuilds = f.rebuilds;
    return stale ? 1 : 0;
}

tdz_status tdz_strong_field_ratio(const tdz_space *s, int kind, double dt, double final_time, tdz_field_fn field,
                                  void *ctx, double *ratio) {
    return guarded([&] {
        TDZ_CHECK(s && field && ratio, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(dt > 0.0 && final_time >= 0.0, TDZ_ERR_ARG, "dt must be positive, final_time non-negative");
        TDZ_CHECK(kind >= 0 && kind <= 2, TDZ_ERR_ARG, "unknown propagator kind");
        const double s12 = std::sqrt(12.0);
        const double tau = kind == TDZ_CN ? 0.5 * dt : (kind == TDZ_PADE22 ? dt / s12 : dt / (2.0 * s12));
        double L[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < s->s.dim; ++a) {
            const auto &U = s->s.ax[a].U;
            L[a] = std::max(std::abs(U.front()), std::abs(U.back()));
        }
        const long long n = (long long)std::ceil(4.0 * final_time / dt);
        double worst = 0.0;
        for (long long i = 0; i <= n; ++i) {
            const double t = final_time * (double)i / (double)std::max<long long>(n, 1);
            double v = 0.0;
            for (int a = 0; a < s->s.dim; ++a) v += std::abs(field(a, t, ctx)) * L[a];
            worst = std::max(worst, v);
        }
        *ratio = tau * worst;
    });
}

tdz_status tdz_tsurff_create(const tdz_space *s, const tdz_tsurff_opts *o, tdz_field_fn field, void *ctx,
                             tdz_tsurff **out) {
    return guarded([&] {
        TDZ_CHECK(s && o && out, TDZ_ERR_ARG, "null argument");
        *out = nullptr;
        auto h = std::make_unique<tdz_tsurff>();
        h->t.setup(s->s, *o, field, ctx);
        *out = h.release();
    });
}

tdz_status tdz_tsurff_sample(tdz_tsurff *ts, double t, const void *psi, void *stream) {
    return guarded([&] {
        TDZ_CHECK(ts && psi, TDZ_ERR_ARG, "null argument");
        ts->t.sample(t, static_cast<const double2 *>(psi), static_cast<cudaStream_t>(stream));
    });
}

tdz_status tdz_tsurff_amplitudes(tdz_tsurff *ts, double *out, void *stream) {
    return guarded([&] {
        TDZ_CHECK(ts && out, TDZ_ERR_ARG, "null argument");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        TDZ_CUDA(cudaMemcpyAsync(out, ts->t.amp.ptr, ts->t.nktot * sizeof(double2), cudaMemcpyDeviceToHost, st));
        TDZ_CUDA(cudaStreamSynchronize(st));
    });
}

tdz_status tdz_tsurff_interior(tdz_tsurff *ts, const void *psi, double *out, void *stream) {
    return guarded([&] {
        TDZ_CHECK(ts && psi && out, TDZ_ERR_ARG, "null argument");
        std::vector<tdz::cd> v;
        ts->t.interior(static_cast<const double2 *>(psi), v, static_cast<cudaStream_t>(stream));
        for (size_t i = 0; i < v.size(); ++i) { out[2 * i] = v[i].real(); out[2 * i + 1] = v[i].imag(); }
    });
}

tdz_status tdz_tsurff_end_term(tdz_tsurff *ts, tdz_op *op, const tdz_solver_opts *inner,
                               const tdz_tsurff_end_opts *o, const void *psi, double *out, double *stats,
                               void *stream) {
    return guarded([&] {
        TDZ_CHECK(ts && op && psi && out, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(reinterpret_cast<uintptr_t>(psi) % 16 == 0, TDZ_ERR_ARG, "psi must be 16-byte aligned");
        tdz::SolverOptions so;
        if (inner) {
            so = solver_options(inner);
        } else {   // exact banded LU in 1D, fast diagonalisation in 2D/3D (degrees 2..5)
            const int dim = op->o.sp->dim, p = op->o.sp->ax[0].p;
            so.pc = dim == 1 ? TDZ_PC_BAND : (p >= 2 && p <= 5 ? TDZ_PC_FDM : TDZ_PC_MASS);
            // FP64: the complex eigenbases of absorbing layers can be far from
            // orthogonal, and nodes next to weakly absorbed box modes are
            // nearly singular; an FP32 inverse loses every digit there
            so.pc_precision = TDZ_FP64;
            so.outer = TDZ_FP64;
            so.restart = 60;
        }
        tdz::EndTermOptions eo;
        if (o) {
            eo.dp = o->dp;
            eo.cap_width = o->cap_width;
            eo.eta = o->eta;
            if (o->rtol > 0.0) eo.rtol = o->rtol;
            if (o->maxit > 0) eo.maxit = o->maxit;
        }
        std::vector<tdz::cd> v;
        const tdz::EndTermStats r = ts->t.end_term(op->o, so, eo, static_cast<const double2 *>(psi), v,
                                                   static_cast<cudaStream_t>(stream));
        for (size_t i = 0; i < v.size(); ++i) { out[2 * i] = v[i].real(); out[2 * i + 1] = v[i].imag(); }
        if (stats) {
            stats[0] = r.nodes;
            stats[1] = (double)r.its;
            stats[2] = r.max_its;
            stats[3] = r.dp_max;
            stats[4] = r.eta;
            stats[5] = r.seconds;
            stats[6] = r.damped;
        }
    });
}

tdz_status tdz_tsurff_volkov(const tdz_tsurff *ts, double *abct) {
    return guarded([&] {
        TDZ_CHECK(ts && abct, TDZ_ERR_ARG, "null argument");
        for (int d = 0; d < 3; ++d) { abct[d] = ts->t.A[d]; abct[3 + d] = ts->t.B[d]; }
        abct[6] = ts->t.C;
        abct[7] = ts->t.vt;
    });
}

tdz_status tdz_tsurff_info(const tdz_tsurff *ts, double *info) {
    return guarded([&] {
        TDZ_CHECK(ts != nullptr && info != nullptr, TDZ_ERR_ARG, "null argument");
        const tdz::TSurff &t = ts->t;
        double points = 0.0;
        for (int a = 0; a < t.dim; ++a) {
            double face = 1.0;
            for (int b = 0; b < 3; ++b)
                if (b != a && b < t.dim) face *= (double)t.nodes[b].size();
            points += 2.0 * face;
        }
        info[0] = t.prevT;
        info[1] = t.R;
        info[2] = t.mass;
        info[3] = t.V0;
        info[4] = points;
        info[5] = (double)t.samples;
        info[6] = (double)t.nktot;
        info[7] = (double)t.dim;
    });
}

void tdz_tsurff_destroy(tdz_tsurff *ts) { delete ts; }

tdz_status tdz_cnn_create(int cin, int width, int cout, int layers, int D, int H, int W, int batch,
                          unsigned long long seed, tdz_cnn **out) {
    return guarded([&] {
        TDZ_CHECK(out, TDZ_ERR_ARG, "null argument");
        *out = nullptr;
        TDZ_CHECK(cin >= 1 && width >= 1 && cout >= 1 && layers >= 1 && D >= 1 && H >= 1 && W >= 1 && batch >= 1,
                  TDZ_ERR_ARG, "bad network shape");
        auto h = std::make_unique<tdz_cnn>();
        h->n.init(cin, width, cout, layers, D, H, W, batch, seed);
        *out = h.release();
    });
}

tdz_status tdz_cnn_forward(tdz_cnn *n, const float *in, float *out, int batch, void *stream) {
    return guarded([&] {
        TDZ_CHECK(n && in && out, TDZ_ERR_ARG, "null argument");
        n->n.forward(in, out, batch, static_cast<cudaStream_t>(stream), false);
    });
}

tdz_status tdz_cnn_train_step(tdz_cnn *n, const float *in, const float *target, int batch, float lr, void *stream) {
    return guarded([&] {
        TDZ_CHECK(n && in && target, TDZ_ERR_ARG, "null argument");
        TDZ_CHECK(batch >= 1 && batch <= n->n.batch, TDZ_ERR_ARG, "bad batch");
        n->n.train_step(in, target, batch, lr, static_cast<cudaStream_t>(stream));
    });
}

tdz_status tdz_cnn_loss(tdz_cnn *n, float *loss, void *stream) {
    return guarded([&] {
        TDZ_CHECK(n && loss, TDZ_ERR_ARG, "null argument");
        *loss = n->n.read_loss(static_cast<cudaStream_t>(stream));
    });
}

tdz_status tdz_cnn_num_params(const tdz_cnn *n, long long *count) {
    return guarded([&] {
        TDZ_CHECK(n && count, TDZ_ERR_ARG, "null argument");
        long long c = 0;
        for (int l = 0; l < n->n.layers; ++l) c += (long long)n->n.co[l] * n->n.ci[l] * 27 + n->n.co[l];
        *count = c;
    });
}

tdz_status tdz_cnn_get_params(const tdz_cnn *n, float *host) {
    return guarded([&] {
        TDZ_CHECK(n && host, TDZ_ERR_ARG, "null argument");
        std::vector<float> v;
        n->n.get_params(v);
        std::memcpy(host, v.data(), v.size() * sizeof(float));
    });
}

tdz_status tdz_cnn_set_params(tdz_cnn *n, const float *host) {
    return guarded([&] {
        TDZ_CHECK(n && host, TDZ_ERR_ARG, "null argument");
        long long c = 0;
        for (int l = 0; l < n->n.layers; ++l) c += (long long)n->n.co[l] * n->n.ci[l] * 27 + n->n.co[l];
        n->n.set_params(std::vector<float>(host, host + c));
    });
}

tdz_status tdz_cnn_get_grads(const tdz_cnn *n, float *host) {
    return guarded([&] {
        TDZ_CHECK(n && host, TDZ_ERR_ARG, "null argument");
        std::vector<float> v;
        n->n.get_grads(v);
        std::memcpy(host, v.data(), v.size() * sizeof(float));
    });
}

void tdz_cnn_destroy(tdz_cnn *n) { delete n; }

tdz_status tdz_h5_write(const char *path, int ndatasets, const char *const *names, const int *ranks,
                        const long long *dims, const double *const *data, int nattrs, const char *const *attr_names,
                        const long long *attr_lens, const double *const *attr_data) {
    return guarded([&] {
        TDZ_CHECK(path != nullptr && ndatasets >= 0 && nattrs >= 0, TDZ_ERR_ARG, "invalid arguments");
        TDZ_CHECK(ndatasets == 0 || (names && ranks && dims && data), TDZ_ERR_ARG, "dataset arrays missing");
        TDZ_CHECK(nattrs == 0 || (attr_names && attr_lens && attr_data), TDZ_ERR_ARG, "attribute arrays missing");
        std::vector<tdz::H5Array> ds(ndatasets), at(nattrs);
        const long long *d = dims;
        for (int i = 0; i < ndatasets; ++i) {
            TDZ_CHECK(names[i] != nullptr && ranks[i] >= 1 && ranks[i] <= 8, TDZ_ERR_ARG, "dataset name or rank");
            ds[i].name = names[i];
            for (int k = 0; k < ranks[i]; ++k) {
                TDZ_CHECK(d[k] >= 1, TDZ_ERR_ARG, std::string("dataset '") + names[i] + "' has an empty axis");
                ds[i].dims.push_back((uint64_t)d[k]);
            }
            d += ranks[i];
            ds[i].data = data[i];
        }
        for (int j = 0; j < nattrs; ++j) {
            TDZ_CHECK(attr_names[j] != nullptr && attr_lens[j] >= 1, TDZ_ERR_ARG, "attribute name or length");
            at[j].name = attr_names[j];
            at[j].dims = {(uint64_t)attr_lens[j]};
            at[j].data = attr_data[j];
        }
        tdz::h5_write_file(path, ds, at);
    });
}

tdz_status tdz_obsfile_open(const char *path, int dim, int n_bound, long long flush_rows, tdz_obsfile **out) {
    return guarded([&] {
        TDZ_CHECK(path != nullptr && out != nullptr, TDZ_ERR_ARG, "null argument");
        *out = new tdz_obsfile{tdz::ObsFile(path, dim, n_bound, flush_rows)};
    });
}

int tdz_obsfile_columns(const tdz_obsfile *f, int set) {
    if (!f || set < 0 || set >= tdz::ObsFile::kSets) return -1;
    return f->f.columns(set);
}

tdz_status tdz_obsfile_record(tdz_obsfile *f, double t, const double *const *rows) {
    return guarded([&] {
        TDZ_CHECK(f != nullptr, TDZ_ERR_ARG, "null file");
        f->f.record(t, rows);
    });
}

tdz_status tdz_obsfile_rows(const tdz_obsfile *f, long long *recorded, long long *written) {
    return guarded([&] {
        TDZ_CHECK(f != nullptr, TDZ_ERR_ARG, "null file");
        if (recorded) *recorded = f->f.rows();
        if (written) *written = f->f.written();
    });
}

tdz_status tdz_obsfile_flush(tdz_obsfile *f) {
    return guarded([&] {
        TDZ_CHECK(f != nullptr, TDZ_ERR_ARG, "null file");
        f->f.flush();
    });
}

tdz_status tdz_obsfile_close(tdz_obsfile *f) {
    const tdz_status st = guarded([&] {
        if (f) f->f.flush();
    });
    delete f;
    return st;
}

}  // extern "C"
