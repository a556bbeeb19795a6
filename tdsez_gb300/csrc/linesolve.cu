// Banded Cholesky line solves (the exact Kronecker inverse of the overlap).
//
// Lines along y and z: one thread per line, consecutive threads on
// consecutive x, so every step of the recurrence is a coalesced load/store;
// the last p values of the recurrence stay in registers. Lines along x
// (contiguous rows): a CTA stages ROWS rows in shared memory with coalesced
// loads, one thread per row runs the recurrence there.
#include "linesolve.h"

#include <cmath>

#include "cplx.cuh"

namespace tdz {

void BandChol::factor(const BandD &A) {
    n = A.n;
    p = A.p;
    L.assign((size_t)n * (p + 1), 0.0);
    auto Lat = [&](int i, int j) -> double & { return L[(size_t)i * (p + 1) + (j - i + p)]; };
    for (int i = 0; i < n; ++i) {
        for (int j = std::max(0, i - p); j <= i; ++j) {
            double s = A.at(i, j);
            for (int k = std::max(std::max(0, i - p), j - p); k < j; ++k) s -= Lat(i, k) * Lat(j, k);
            if (i == j) {
                TDZ_CHECK(s > 0.0, TDZ_ERR_INTERNAL, "band is not positive definite");
                Lat(i, i) = std::sqrt(s);
            } else {
                Lat(i, j) = s / Lat(j, j);
            }
        }
    }
    for (int i = 0; i < n; ++i) Lat(i, i) = 1.0 / Lat(i, i);
}

void BandChol::upload() {
    std::vector<float> l32(L.begin(), L.end());
    tdz::upload(L64, L);
    tdz::upload(L32, l32);
}

namespace {

// strided lines: element k of line (a, b) at base + k*stride
template <class T, int P>
__global__ void k_line_strided(const T *__restrict__ L, int n, typename CT<T>::type *x, int nx_lines, int nb,
                               size_t stride, size_t bstride) {
    using C = typename CT<T>::type;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (a >= nx_lines || b >= nb) return;
    C *line = x + (size_t)b * bstride + a;
    C win[P + 1];
#pragma unroll
    for (int k = 0; k <= P; ++k) win[k] = czero<C>();
    // forward: y_i = (b_i - sum_k L(i, i-k) y_{i-k}) / L(i, i); win[0] is y_{i-1}
    for (int i = 0; i < n; ++i) {
        C v = line[(size_t)i * stride];
        const T *Li = L + (size_t)i * (P + 1);
#pragma unroll
        for (int k = 1; k <= P; ++k)
            if (i - k >= 0) rfma(v, -Li[P - k], win[k - 1]);
        const T d = Li[P];
        v.x *= d;
        v.y *= d;
#pragma unroll
        for (int k = P; k > 0; --k) win[k] = win[k - 1];
        win[0] = v;
        line[(size_t)i * stride] = v;
    }
    // backward: x_i = (y_i - sum_k L(i+k, i) x_{i+k}) / L(i, i)
#pragma unroll
    for (int k = 0; k <= P; ++k) win[k] = czero<C>();
    for (int i = n - 1; i >= 0; --i) {
        C v = line[(size_t)i * stride];
#pragma unroll
        for (int k = 1; k <= P; ++k)
            if (i + k < n) rfma(v, -L[(size_t)(i + k) * (P + 1) + (P - k)], win[k - 1]);
        const T d = L[(size_t)i * (P + 1) + P];
        v.x *= d;
        v.y *= d;
#pragma unroll
        for (int k = P; k > 0; --k) win[k] = win[k - 1];
        win[0] = v;
        line[(size_t)i * stride] = v;
    }
}

// contiguous rows of length n (axis x): stage ROWS rows in shared memory
template <class T, int P>
__global__ void k_line_rows(const T *__restrict__ L, int n, typename CT<T>::type *x, int nrows) {
    using C = typename CT<T>::type;
    extern __shared__ unsigned char smem_raw[];
    C *tile = reinterpret_cast<C *>(smem_raw);
    const int rows = blockDim.x;
    const int r0 = blockIdx.x * rows;
    const int nr = min(rows, nrows - r0);
    // coalesced load of nr rows
    for (int e = threadIdx.x; e < nr * n; e += blockDim.x) tile[e] = x[(size_t)r0 * n + e];
    __syncthreads();
    if (threadIdx.x < nr) {
        C *line = tile + (size_t)threadIdx.x * n;
        C win[P + 1];
#pragma unroll
        for (int k = 0; k <= P; ++k) win[k] = czero<C>();
        for (int i = 0; i < n; ++i) {
            C v = line[i];
            const T *Li = L + (size_t)i * (P + 1);
#pragma unroll
            for (int k = 1; k <= P; ++k)
                if (i - k >= 0) rfma(v, -Li[P - k], win[k - 1]);
            const T d = Li[P];
            v.x *= d;
            v.y *= d;
#pragma unroll
            for (int k = P; k > 0; --k) win[k] = win[k - 1];
            win[0] = v;
            line[i] = v;
        }
#pragma unroll
        for (int k = 0; k <= P; ++k) win[k] = czero<C>();
        for (int i = n - 1; i >= 0; --i) {
            C v = line[i];
#pragma unroll
            for (int k = 1; k <= P; ++k)
                if (i + k < n) rfma(v, -L[(size_t)(i + k) * (P + 1) + (P - k)], win[k - 1]);
            const T d = L[(size_t)i * (P + 1) + P];
            v.x *= d;
            v.y *= d;
#pragma unroll
            for (int k = P; k > 0; --k) win[k] = win[k - 1];
            win[0] = v;
            line[i] = v;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nr * n; e += blockDim.x) x[(size_t)r0 * n + e] = tile[e];
}

template <class T, int P>
void run_axis(const T *L, int axis, typename CT<T>::type *x, int n0, int n1, int n2, cudaStream_t st) {
    using C = typename CT<T>::type;
    if (axis == 0) {
        int rows = 32;
        while (rows > 1 && (size_t)rows * n0 * sizeof(C) > 96 * 1024) rows /= 2;
        const size_t smem = (size_t)rows * n0 * sizeof(C);
        TDZ_CHECK(smem <= 200 * 1024, TDZ_ERR_UNSUPPORTED, "axis too long for the row line solve");
        // set once to the largest size (a per-kernel limit: concurrent solves of
        // other lengths must not lower it under this launch)
        static const bool attr = [] {
            TDZ_CUDA(cudaFuncSetAttribute(k_line_rows<T, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            return true;
        }();
        (void)attr;
        const int nrows = n1 * n2;
        k_line_rows<T, P><<<(nrows + rows - 1) / rows, rows, smem, st>>>(L, n0, x, nrows);
    } else if (axis == 1) {
        // lines along y: a = x index, b = z index; stride n0, line base b*n0*n1 + a
        dim3 grid((n0 + 127) / 128, n2);
        k_line_strided<T, P><<<grid, 128, 0, st>>>(L, n1, x, n0, n2, (size_t)n0, (size_t)n0 * n1);
    } else {
        // lines along z: a = x + n0 y, stride n0 n1
        const int nl = n0 * n1;
        dim3 grid((nl + 127) / 128, 1);
        k_line_strided<T, P><<<grid, 128, 0, st>>>(L, n2, x, nl, 1, (size_t)n0 * n1, 0);
    }
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

template <class T>
void run_axis_p(int p, const T *L, int axis, typename CT<T>::type *x, int n0, int n1, int n2, cudaStream_t st) {
    switch (p) {
    case 1: run_axis<T, 1>(L, axis, x, n0, n1, n2, st); break;
    case 2: run_axis<T, 2>(L, axis, x, n0, n1, n2, st); break;
    case 3: run_axis<T, 3>(L, axis, x, n0, n1, n2, st); break;
    case 4: run_axis<T, 4>(L, axis, x, n0, n1, n2, st); break;
    case 5: run_axis<T, 5>(L, axis, x, n0, n1, n2, st); break;
    case 6: run_axis<T, 6>(L, axis, x, n0, n1, n2, st); break;
    case 7: run_axis<T, 7>(L, axis, x, n0, n1, n2, st); break;
    default: throw Error(TDZ_ERR_UNSUPPORTED, "line solves support degrees 1..7");
    }
}

}  // namespace

void line_solve(const BandChol &F, int axis, void *x, int n0, int n1, int n2, int prec, cudaStream_t st) {
    if (prec == TDZ_FP64) run_axis_p<double>(F.p, F.L64.as<double>(), axis, static_cast<double2 *>(x), n0, n1, n2, st);
    else run_axis_p<float>(F.p, F.L32.as<float>(), axis, static_cast<float2 *>(x), n0, n1, n2, st);
}

void KronSolve::setup(const std::array<const BandD *, 3> &bands, int dim_) {
    dim = dim_;
    for (int d = 0; d < 3; ++d) n[d] = 1;
    for (int d = 0; d < dim; ++d) {
        f[d].factor(*bands[d]);
        f[d].upload();
        n[d] = bands[d]->n;
    }
}

void KronSolve::apply(void *x, int prec, cudaStream_t st) const {
    for (int d = 0; d < dim; ++d) line_solve(f[d], d, x, n[0], n[1], n[2], prec, st);
}

}  // namespace tdz
