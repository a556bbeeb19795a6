/* Oracle (test infrastructure only): the reference's CPU Crank-Nicolson solver
 * restated in C with OpenMP threads, for the CPU baseline leg of bench.py.
 *
 * Method as TDSE-Z runs it on P MPI ranks (src/propagator.cpp:125-243,
 * TDSEZConfigureStageKSP src/propagator.cpp:315-370): per step the CN matrix
 * A = M + i h/2 (H + sum_a c_a(t) D_a) is rebuilt on the assembled pattern
 * (src/monitor.cpp:273-331), rhs = M psi, GMRES(30) with right
 * preconditioning and a nonzero initial guess (the previous state) to a
 * relative true residual of rtol, then psi <- 2 X - psi. The preconditioner
 * is PETSc's parallel default, block Jacobi with ILU(0) on each rank's
 * diagonal block, built once from the first step's matrix and reused. Here
 * the blocks are contiguous row ranges, one per thread.
 *
 * All matrices share one CSR pattern (rowptr, col), column indices sorted.
 * Complex values are interleaved double pairs.
 */
#include <complex.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef double complex cplx;

static double now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

typedef struct {
    int n, nb;
    const int *rp, *ci;
    int *bstart;     /* nb + 1 row boundaries */
    int *diag;       /* index of the diagonal entry of each row */
    cplx *lu;        /* ILU(0) factors on the pattern, off-block entries unused */
} Pc;

/* ILU(0) of the diagonal block rows [r0, r1) (IKJ order, pattern-restricted) */
static int ilu0_block(Pc *pc, const cplx *a, int r0, int r1) {
    const int *rp = pc->rp, *ci = pc->ci;
    cplx *lu = pc->lu;
    int *pos = (int *)malloc(sizeof(int) * (size_t)(r1 - r0));
    if (!pos) return -1;
    for (int j = 0; j < r1 - r0; ++j) pos[j] = -1;
    for (int i = r0; i < r1; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) lu[k] = a[k];
    int bad = 0;
    for (int i = r0; i < r1; ++i) {
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] >= r0 && ci[k] < r1) pos[ci[k] - r0] = k;
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            if (j < r0 || j >= i) continue;
            const cplx piv = lu[pc->diag[j]];
            if (piv == 0) { bad = 1; continue; }
            const cplx f = lu[k] / piv;
            lu[k] = f;
            for (int kk = pc->diag[j] + 1; kk < rp[j + 1]; ++kk) {
                const int c = ci[kk];
                if (c >= r1) break;
                const int p = pos[c - r0];
                if (p >= 0) lu[p] -= f * lu[kk];
            }
        }
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] >= r0 && ci[k] < r1) pos[ci[k] - r0] = -1;
        if (lu[pc->diag[i]] == 0) bad = 1;
    }
    free(pos);
    return bad ? -2 : 0;
}

/* z = P^-1 r: per block L U z = r restricted to the block */
static void pc_apply(const Pc *pc, const cplx *r, cplx *z) {
    const int *rp = pc->rp, *ci = pc->ci;
    const cplx *lu = pc->lu;
#pragma omp parallel for schedule(static, 1)
    for (int b = 0; b < pc->nb; ++b) {
        const int r0 = pc->bstart[b], r1 = pc->bstart[b + 1];
        for (int i = r0; i < r1; ++i) {
            cplx s = r[i];
            for (int k = rp[i]; k < pc->diag[i]; ++k)
                if (ci[k] >= r0) s -= lu[k] * z[ci[k]];
            z[i] = s;
        }
        for (int i = r1 - 1; i >= r0; --i) {
            cplx s = z[i];
            for (int k = pc->diag[i] + 1; k < rp[i + 1]; ++k) {
                if (ci[k] >= r1) break;
                s -= lu[k] * z[ci[k]];
            }
            z[i] = s / lu[pc->diag[i]];
        }
    }
}

static void spmv(int n, const int *rp, const int *ci, const cplx *a, const cplx *x, cplx *y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        cplx s = 0;
        for (int k = rp[i]; k < rp[i + 1]; ++k) s += a[k] * x[ci[k]];
        y[i] = s;
    }
}

static cplx dotc(int n, const cplx *x, const cplx *y) {   /* sum conj(x) y */
    double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (int i = 0; i < n; ++i) {
        const cplx v = conj(x[i]) * y[i];
        re += creal(v);
        im += cimag(v);
    }
    return re + I * im;
}

static double nrm2(int n, const cplx *x) { return sqrt(creal(dotc(n, x, x))); }

/* GMRES(m), right preconditioned, modified Gram-Schmidt; x holds the guess.
 * Returns iterations, or -1 when maxit is reached. */
static int gmres(int n, const int *rp, const int *ci, const cplx *a, const Pc *pc, const cplx *b, cplx *x,
                 double rtol, int m, int maxit, cplx *work) {
    cplx *V = work, *Z = V + (size_t)(m + 1) * n, *w = Z + (size_t)m * n;
    cplx *H = (cplx *)calloc((size_t)(m + 1) * m, sizeof(cplx));
    cplx *g = (cplx *)calloc((size_t)(m + 1), sizeof(cplx));
    cplx *cs = (cplx *)calloc((size_t)m, sizeof(cplx)), *sn = (cplx *)calloc((size_t)m, sizeof(cplx));
    cplx *y = (cplx *)calloc((size_t)m, sizeof(cplx));
    const double target = rtol * nrm2(n, b);
    int total = 0, result = -1;
    for (;;) {
        spmv(n, rp, ci, a, x, V);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) V[i] = b[i] - V[i];
        const double beta = nrm2(n, V);
        if (beta <= target) { result = total; break; }
        if (total >= maxit) break;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) V[i] /= beta;
        memset(g, 0, sizeof(cplx) * (size_t)(m + 1));
        g[0] = beta;
        int j = 0, conv = 0;
        for (; j < m && total < maxit; ++j) {
            ++total;
            cplx *vj = V + (size_t)j * n, *zj = Z + (size_t)j * n;
            pc_apply(pc, vj, zj);
            spmv(n, rp, ci, a, zj, w);
            for (int i = 0; i <= j; ++i) {
                const cplx *vi = V + (size_t)i * n;
                const cplx h = dotc(n, vi, w);
                H[(size_t)i * m + j] = h;
#pragma omp parallel for schedule(static)
                for (int e = 0; e < n; ++e) w[e] -= h * vi[e];
            }
            const double hn = nrm2(n, w);
            for (int i = 0; i < j; ++i) {
                const cplx t0 = H[(size_t)i * m + j], t1 = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = conj(cs[i]) * t0 + conj(sn[i]) * t1;
                H[(size_t)(i + 1) * m + j] = -sn[i] * t0 + cs[i] * t1;
            }
            const cplx d = H[(size_t)j * m + j];
            const double r = sqrt(creal(d) * creal(d) + cimag(d) * cimag(d) + hn * hn);
            if (r == 0) { cs[j] = 1; sn[j] = 0; }
            else { cs[j] = d / r; sn[j] = hn / r; }
            H[(size_t)j * m + j] = r;
            g[j + 1] = -sn[j] * g[j];
            g[j] = conj(cs[j]) * g[j];
            if (cabs(g[j + 1]) <= target || hn == 0) { ++j; conv = 1; break; }
            cplx *vn = V + (size_t)(j + 1) * n;
#pragma omp parallel for schedule(static)
            for (int e = 0; e < n; ++e) vn[e] = w[e] / hn;
        }
        for (int i = j - 1; i >= 0; --i) {
            cplx s = g[i];
            for (int l = i + 1; l < j; ++l) s -= H[(size_t)i * m + l] * y[l];
            y[i] = s / H[(size_t)i * m + i];
        }
#pragma omp parallel for schedule(static)
        for (int e = 0; e < n; ++e) {
            cplx s = 0;
            for (int i = 0; i < j; ++i) s += y[i] * Z[(size_t)i * n + e];
            x[e] += s;
        }
        (void)conv;   /* the restart recomputes the true residual and decides */
    }
    free(H);
    free(g);
    free(cs);
    free(sn);
    free(y);
    return result;
}

/* Crank-Nicolson steps on the shared pattern. vals: M, H, then nd dipoles
 * (interleaved complex, nnz each); coef: nd field coefficients s E_a per
 * step (steps_max rows); psi: state in/out. threads: OpenMP threads (0: all);
 * blocks: block-Jacobi blocks (0: one per thread; 1: ILU(0) of the whole
 * matrix, whose triangular solves then run on one thread while the rest is
 * threaded). Runs at least min_steps and until `seconds` have passed (or
 * steps_max). out[0] = steps, out[1] = seconds, out[2] = Krylov iterations,
 * out[3] = threads, out[4] = blocks. Returns 0, or < 0 on failure. */
int cn_bjilu_run(int n, const int *rp, const int *ci, const double *vals, int nd, const double *coef, double dt,
                 double rtol, int threads, int blocks, double seconds, int min_steps, int steps_max, double *psi_io,
                 double *out) {
    if (threads > 0) omp_set_num_threads(threads);
    int nthr = 1;
#pragma omp parallel
    {
#pragma omp single
        nthr = omp_get_num_threads();
    }
    const int nnz = rp[n];
    const cplx *Mv = (const cplx *)vals, *Hv = Mv + nnz, *Dv = Hv + nnz;
    cplx *psi = (cplx *)psi_io;
    cplx *A = (cplx *)malloc(sizeof(cplx) * (size_t)nnz);
    cplx *rhs = (cplx *)malloc(sizeof(cplx) * (size_t)n), *X = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    const int m = 30;
    cplx *work = (cplx *)malloc(sizeof(cplx) * (size_t)n * (2 * m + 2));
    const int nb = blocks > 0 ? (blocks < n ? blocks : n) : nthr;
    Pc pc;
    pc.n = n;
    pc.nb = nb;
    pc.rp = rp;
    pc.ci = ci;
    pc.bstart = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
    pc.diag = (int *)malloc(sizeof(int) * (size_t)n);
    pc.lu = (cplx *)malloc(sizeof(cplx) * (size_t)nnz);
    if (!A || !rhs || !X || !work || !pc.bstart || !pc.diag || !pc.lu) return -1;
    for (int b = 0; b <= nb; ++b) pc.bstart[b] = (int)((long long)n * b / nb);
    for (int i = 0; i < n; ++i) {
        pc.diag[i] = -1;
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i) pc.diag[i] = k;
        if (pc.diag[i] < 0) return -3;
    }
    const cplx ih = 0.5 * dt * I;
    int steps = 0, status = 0;
    long long its = 0;
    double t0 = 0;
    while (steps < steps_max) {
        const double *c = coef + (size_t)steps * nd;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nnz; ++k) {
            cplx hv = Hv[k];
            for (int a = 0; a < nd; ++a) hv += c[a] * Dv[(size_t)a * nnz + k];
            A[k] = Mv[k] + ih * hv;
        }
        if (steps == 0) {   /* block Jacobi ILU(0) of the first step's matrix, reused */
            int bad = 0;
#pragma omp parallel for schedule(static, 1) reduction(| : bad)
            for (int b = 0; b < nb; ++b) bad |= ilu0_block(&pc, A, pc.bstart[b], pc.bstart[b + 1]) != 0;
            if (bad) { status = -4; break; }
            t0 = now();   /* the preconditioner setup is not timed */
        }
        spmv(n, rp, ci, Mv, psi, rhs);
        memcpy(X, psi, sizeof(cplx) * (size_t)n);
        const int it = gmres(n, rp, ci, A, &pc, rhs, X, rtol, m, 2000, work);
        if (it < 0) { status = -5; break; }
        its += it;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) psi[i] = 2.0 * X[i] - psi[i];
        ++steps;
        if (steps >= min_steps && now() - t0 >= seconds) break;
    }
    out[0] = steps;
    out[1] = now() - t0;
    out[2] = (double)its;
    out[3] = nthr;
    out[4] = nb;
    free(A);
    free(rhs);
    free(X);
    free(work);
    free(pc.bstart);
    free(pc.diag);
    free(pc.lu);
    return status;
}
