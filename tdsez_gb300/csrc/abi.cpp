// extern "C" boundary of the tdz library: every entry point catches the C++
// error of its body and returns a status code; the message is kept per thread
// for tdz_last_error(). Mirrors the PetscErrorCode / PetscCall convention of
// the reference (every call returns a code, no exception crosses the ABI).
#include <cmath>
#include <cstring>
#include <memory>

#include "oper.h"
#include "prop.h"

struct tdz_space {
    tdz::Space s;
};
struct tdz_op {
    tdz::Operator o;
};
struct tdz_solver {
    tdz::Solver s;
};
struct tdz_prop {
    tdz::Propagator p;
};

namespace tdz {
static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
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

long long tdz_operator_launches(const tdz_op *op) { return op ? op->o.launches : 0; }

void tdz_operator_destroy(tdz_op *op) { delete op; }

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
    so.mg.smooth = o->mg_smooth > 0 ? o->mg_smooth : 2;
    so.mg.coarse_its = o->mg_coarse_its > 0 ? o->mg_coarse_its : 12;
    return so;
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

void tdz_prop_destroy(tdz_prop *p) { delete p; }

}  // extern "C"
