// Exact banded LU preconditioner for 1D stage operators (FP64 complex).
//
// The factorisation and the solves each run in one warp: a 1D operator has
// a few thousand rows and a band of 2p+1, so the work per elimination step
// (p rows times 2p columns) fits one warp, and the steps are sequential.
// The band is assembled on the host from the same base bands and stage
// scalars as the fused 1D apply (k_apply1d), so P A^-1 is the identity up to
// rounding; FGMRES then needs one iteration per solve.
#include "band.h"

#include <cmath>

namespace tdz {

namespace {

struct BandArgs {
    double2 *a;      // [n][3p+1]: row i holds columns i - p .. i + 2p
    int *piv;        // row interchanged with row k at step k
    int *err;        // 0, or 1 + the first step without a nonzero pivot
    int n, p;
};

__device__ __forceinline__ double2 &band_at(const BandArgs &f, int i, int j) {
    return f.a[(size_t)i * (3 * f.p + 1) + (j - i + f.p)];
}

__device__ __forceinline__ double2 cmul_d(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Gaussian elimination with partial pivoting down the band (one warp).
// Step k: the pivot is the entry of largest |re| + |im| among rows
// k .. k + p of column k (lowest row on ties); rows k and the pivot row swap
// their columns k .. k + 2p; the multipliers replace column k below the
// diagonal; the p x 2p trailing block takes the rank-one update.
__global__ void __launch_bounds__(32) k_band_factor(BandArgs f) {
    const int lane = threadIdx.x, n = f.n, p = f.p;
    for (int k = 0; k < n; ++k) {
        const int rmax = min(k + p, n - 1), cmax = min(k + 2 * p, n - 1);
        double best = -1.0;
        int bi = k;
        for (int r = k + lane; r <= rmax; r += 32) {
            const double2 v = band_at(f, r, k);
            const double m = fabs(v.x) + fabs(v.y);
            if (m > best) { best = m; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) f.piv[k] = bi;
        if (!(best > 0.0)) {
            // singular column: record it and leave the column as it is (the
            // host refuses the factorisation)
            if (lane == 0 && f.err[0] == 0) f.err[0] = k + 1;
            __syncwarp();
            continue;
        }
        if (bi != k)
            for (int j = k + lane; j <= cmax; j += 32) {
                const double2 t = band_at(f, k, j);
                band_at(f, k, j) = band_at(f, bi, j);
                band_at(f, bi, j) = t;
            }
        __syncwarp();
        const double2 d = band_at(f, k, k);
        const double dd = 1.0 / (d.x * d.x + d.y * d.y);
        const double2 inv = make_double2(d.x * dd, -d.y * dd);
        for (int r = k + 1 + lane; r <= rmax; r += 32) band_at(f, r, k) = cmul_d(band_at(f, r, k), inv);
        __syncwarp();
        const int nr = rmax - k, nc = cmax - k;
        for (int e = lane; e < nr * nc; e += 32) {
            const int r = k + 1 + e / nc, j = k + 1 + e % nc;
            const double2 l = band_at(f, r, k), u = band_at(f, k, j);
            double2 &t = band_at(f, r, j);
            t.x -= l.x * u.x - l.y * u.y;
            t.y -= l.x * u.y + l.y * u.x;
        }
        __syncwarp();
    }
}

// z = A^-1 r from the factors (one warp, the vector in shared memory):
// interchanges and L forward, then U backward.
__global__ void __launch_bounds__(32) k_band_solve(BandArgs f, const double2 *__restrict__ r, double2 *__restrict__ z) {
    extern __shared__ double2 xs[];
    const int lane = threadIdx.x, n = f.n, p = f.p;
    for (int i = lane; i < n; i += 32) xs[i] = r[i];
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        if (lane == 0) {
            const int q = f.piv[k];
            if (q != k) {
                const double2 t = xs[k];
                xs[k] = xs[q];
                xs[q] = t;
            }
        }
        __syncwarp();
        const double2 xk = xs[k];
        const int rmax = min(k + p, n - 1);
        for (int i = k + 1 + lane; i <= rmax; i += 32) {
            const double2 l = band_at(f, i, k);
            xs[i].x -= l.x * xk.x - l.y * xk.y;
            xs[i].y -= l.x * xk.y + l.y * xk.x;
        }
        __syncwarp();
    }
    for (int k = n - 1; k >= 0; --k) {
        const int cmax = min(k + 2 * p, n - 1);
        double sx = 0.0, sy = 0.0;
        for (int j = k + 1 + lane; j <= cmax; j += 32) {
            const double2 u = band_at(f, k, j), x = xs[j];
            sx += u.x * x.x - u.y * x.y;
            sy += u.x * x.y + u.y * x.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
        }
        if (lane == 0) {
            const double2 d = band_at(f, k, k);
            const double dd = 1.0 / (d.x * d.x + d.y * d.y);
            const double2 b = make_double2(xs[k].x - sx, xs[k].y - sy);
            xs[k] = make_double2((b.x * d.x + b.y * d.y) * dd, (b.y * d.x - b.x * d.y) * dd);
        }
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) z[i] = xs[i];
}

constexpr size_t kBandMaxRows = 12800;   // the solve keeps the vector in shared memory (200 KB)

}  // namespace

void PcBand::setup(Operator *op_) {
    op = op_;
    const Space &s = *op->sp;
    TDZ_CHECK(s.dim == 1, TDZ_ERR_UNSUPPORTED, "the banded LU preconditioner is for 1D operators");
    n = s.ax[0].n;
    p = s.ax[0].p;
    TDZ_CHECK((size_t)n <= kBandMaxRows, TDZ_ERR_UNSUPPORTED, "1D operator too large for the banded LU (n <= 12800)");
    exact = !op->quad.on;
    lu.alloc((size_t)n * (3 * p + 1) * sizeof(double2));
    piv.alloc((size_t)n * sizeof(int));
    err.alloc(sizeof(int));
    // the largest vector any instance may stage (the attribute is per kernel, not per launch)
    TDZ_CUDA(cudaFuncSetAttribute(k_band_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(kBandMaxRows * sizeof(double2))));
    stale = true;
}

void PcBand::factor(cudaStream_t st) {
    const Plan &pl = op->plan(TDZ_STAGE);
    const std::array<cd, 5> &sg = op->sigma;
    const int w = 3 * p + 1, bw = 2 * p + 1;
    std::vector<cd> a((size_t)n * w, cd(0.0));
    // the combination of stream A at the current stage (all terms of a 1D operator)
    for (int t = 0; t < pl.zA.n; ++t) {
        const cd c = pl.zA.factor[t] * sg[pl.zA.scalar[t]];
        const BandD &B = op->bases[0][pl.zA.base[t]];
        TDZ_CHECK(B.n == n && B.p == p, TDZ_ERR_INTERNAL, "1D base band of unexpected shape");
        for (int i = 0; i < n; ++i)
            for (int o = 0; o < bw; ++o) {
                const int j = i - p + o;
                if (j >= 0 && j < n) a[(size_t)i * w + o] += c * B.v[(size_t)i * bw + o];
            }
    }
    // Dirichlet walls as the 1D apply pins them: the wall rows keep their
    // diagonal only, and no other row reaches the wall columns
    if (pl.walls) {
        for (int side = 0; side < 2; ++side) {
            const int wr = side == 0 ? 0 : n - 1;
            cd d = 0.0;
            if (pl.wall_m >= 0) d += sg[pl.wall_m] * op->m_wall[side];
            if (pl.wall_h >= 0) d += sg[pl.wall_h] * op->h_wall[side];
            for (int o = 0; o < w; ++o) a[(size_t)wr * w + o] = 0.0;
            a[(size_t)wr * w + p] = d;
        }
        for (int i = 1; i + 1 < n; ++i)
            for (int wc : {0, n - 1}) {
                const int o = wc - i + p;
                if (o >= 0 && o < bw) a[(size_t)i * w + o] = 0.0;
            }
    }
    hband.resize(a.size());
    for (size_t e = 0; e < a.size(); ++e) hband[e] = make_double2(a[e].real(), a[e].imag());
    TDZ_CUDA(cudaMemcpyAsync(lu.ptr, hband.data(), hband.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    TDZ_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), st));
    BandArgs f{lu.as<double2>(), piv.as<int>(), err.as<int>(), n, p};
    k_band_factor<<<1, 32, 0, st>>>(f);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
    int herr = 0;
    TDZ_CUDA(cudaMemcpyAsync(&herr, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    TDZ_CHECK(herr == 0, TDZ_ERR_BREAKDOWN,
              "banded LU: the stage operator is singular (no pivot in column " + std::to_string(herr - 1) + ")");
    stale = false;
    ++factorizations;
}

void PcBand::apply(const double2 *r, double2 *z, cudaStream_t st) {
    if (stale) factor(st);
    BandArgs f{lu.as<double2>(), piv.as<int>(), err.as<int>(), n, p};
    k_band_solve<<<1, 32, (size_t)n * sizeof(double2), st>>>(f, r, z);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tdz
