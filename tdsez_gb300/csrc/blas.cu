// Device vector operations for the Krylov solvers. Reductions (dot products
// and norms) accumulate in FP64 with warp-shuffle + shared-memory block sums
// into per-block partials, then one block per result sums the partials in a
// fixed order: the result does not depend on scheduling (bit-reproducible).
#include "blas.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <type_traits>

#include "cplx.cuh"

namespace tdz {
namespace blas {

namespace {

constexpr int kThreads = 256;
// about 8 CTAs per SM: latency hiding for the double-float dots
inline int red_blocks() { return 8 * sm_count(); }

inline int grid_for(size_t n) {
    const size_t b = (n + kThreads - 1) / kThreads;
    return (int)std::min<size_t>(std::max<size_t>(b, 1), (size_t)red_blocks());
}

template <class C> __device__ __forceinline__ C cmk(double re, double im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}

template <class T>
__global__ void k_scale(typename CT<T>::type *x, double ar, double ai, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        auto v = x[i];
        const T re = (T)ar * v.x - (T)ai * v.y, im = (T)ar * v.y + (T)ai * v.x;
        v.x = re;
        v.y = im;
        x[i] = v;
    }
}

template <class T>
__global__ void k_axpbypcz(typename CT<T>::type *y, double ar, double ai, const typename CT<T>::type *x, double br,
                           double bi, const typename CT<T>::type *z, double cr, double ci, size_t n) {
    using C = typename CT<T>::type;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        C acc = czero<C>();
        if (ar != 0.0 || ai != 0.0) cfma(acc, cmk<C>(ar, ai), x[i]);
        if (br != 0.0 || bi != 0.0) cfma(acc, cmk<C>(br, bi), y[i]);
        if (z && (cr != 0.0 || ci != 0.0)) cfma(acc, cmk<C>(cr, ci), z[i]);
        y[i] = acc;
    }
}

struct PtrPack {
    const void *p[kMaxDot];
};
struct CoefPack {
    double re[kMaxDot], im[kMaxDot];
};

// ---- FP64 vectors in double-float arithmetic. GB300's FP64 pipe (which also
// runs FP64 <-> FP32 conversions) issues 2 instructions per clock per SM, so
// FP64 BLAS written with double arithmetic is bound by that pipe, not by HBM.
// The multi-dot and multi-axpy (and complex-scalar updates) split each FP64
// element into an FP32 pair with integer operations and compute on the FP32
// pipes (about 48 significant bits, relative error near 1e-14); results that
// update a stored FP64 vector are added to it in FP64, so the vector keeps
// its 53 bits. Updates with real scalars (residuals, the CN state update,
// normalisations) stay in FP64: two FMAs per term and element.
struct CoefDF {
    dff re[kMaxDot], im[kMaxDot];
};

inline CoefDF coef_df(const CoefPack &cp, int k) {
    CoefDF c{};
    for (int i = 0; i < k; ++i) {
        c.re[i] = dff_from(cp.re[i]);
        c.im[i] = dff_from(cp.im[i]);
    }
    return c;
}

__device__ __forceinline__ cdff ld_df(const double2 &v) { return load_c<cdff>(v); }
__device__ __forceinline__ double2 st_df(const cdff &c) { return store_c<double2>(c); }
__host__ __device__ inline cdff mk_df(dff re, dff im) {
    cdff c;
    c.x = re;
    c.y = im;
    return c;
}

template <int K>
__global__ void __launch_bounds__(kThreads) k_mdot_df(PtrPack V, const double2 *w, size_t n, double2 *partial) {
    cdff acc[K];
#pragma unroll
    for (int i = 0; i < K; ++i) acc[i] = czero<cdff>();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const cdff wv = ld_df(w[e]);
#pragma unroll
        for (int i = 0; i < K; ++i) cfma_conj(acc[i], ld_df(static_cast<const double2 *>(V.p[i])[e]), wv);
    }
    __shared__ double2 red[kThreads / 32][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        double re = dff_to_double(acc[i].x), im = dff_to_double(acc[i].y);
        for (int off = 16; off > 0; off >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, off);
            im += __shfl_down_sync(0xffffffffu, im, off);
        }
        if (lane == 0) red[warp][i] = make_double2(re, im);
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double re = 0.0, im = 0.0;
        for (int w2 = 0; w2 < kThreads / 32; ++w2) { re += red[w2][threadIdx.x].x; im += red[w2][threadIdx.x].y; }
        partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = make_double2(re, im);
    }
}

// w += sum_i a_i V_i: the increment in double-float, the final add in FP64,
// so w keeps all 53 bits (it is the solution or the Arnoldi vector)
template <int K>
__global__ void k_maxpy_df(double2 *w, PtrPack V, CoefDF a, size_t n) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        cdff acc = czero<cdff>();
#pragma unroll
        for (int i = 0; i < K; ++i) cfma(acc, mk_df(a.re[i], a.im[i]), ld_df(static_cast<const double2 *>(V.p[i])[e]));
        double2 v = w[e];
        v.x += dff_to_double(acc.x);
        v.y += dff_to_double(acc.y);
        w[e] = v;
    }
}

// y = a x + b y + c z with real scalars: native FP64, two FMAs per term and element
__global__ void k_axpbypcz_r64(double2 *y, double a, const double2 *x, double b, const double2 *z, double c, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        if (a != 0.0) { const double2 v = x[i]; acc.x = a * v.x; acc.y = a * v.y; }
        if (b != 0.0) { const double2 v = y[i]; acc.x = fma(b, v.x, acc.x); acc.y = fma(b, v.y, acc.y); }
        if (z && c != 0.0) { const double2 v = z[i]; acc.x = fma(c, v.x, acc.x); acc.y = fma(c, v.y, acc.y); }
        y[i] = acc;
    }
}

// psi = 2 x - psi + c z: the CN state update fused with the last FGMRES
// correction (c z in double-float, the rest in FP64)
__global__ void k_cn_combine(double2 *psi, const double2 *x, const double2 *z, cdff c, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        cdff t = czero<cdff>();
        cfma(t, c, ld_df(z[i]));
        const double2 xv = x[i], pv = psi[i];
        psi[i] = make_double2(fma(2.0, xv.x, -pv.x) + dff_to_double(t.x), fma(2.0, xv.y, -pv.y) + dff_to_double(t.y));
    }
}

__global__ void k_scale_r64(double2 *x, double a, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double2 v = x[i];
        v.x *= a;
        v.y *= a;
        x[i] = v;
    }
}

// y = a x + b y + c z (zero scalars are skipped; z may be null)
__global__ void k_axpbypcz_df(double2 *y, cdff a, const double2 *x, cdff b, const double2 *z, cdff c, int use_a,
                              int use_b, int use_c, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        cdff acc = czero<cdff>();
        if (use_a) cfma(acc, a, ld_df(x[i]));
        if (use_b) cfma(acc, b, ld_df(y[i]));
        if (use_c) cfma(acc, c, ld_df(z[i]));
        y[i] = st_df(acc);
    }
}

__global__ void k_scale_df(double2 *x, cdff a, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        cdff acc = czero<cdff>();
        cfma(acc, a, ld_df(x[i]));
        x[i] = st_df(acc);
    }
}

__global__ void k_cast64to32_df(const double2 *x, float2 *y, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const cdff v = ld_df(x[i]);
        y[i] = make_float2(__fadd_rn(v.x.hi, v.x.lo), __fadd_rn(v.y.hi, v.y.lo));
    }
}

__global__ void k_cast32to64_df(const float2 *x, double2 *y, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = x[i];
        y[i] = make_double2(f2d_exact(v.x), f2d_exact(v.y));
    }
}

__global__ void k_add_cast_df(double2 *y, cdff a, const float2 *x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = x[i];
        cdff acc = ld_df(y[i]);
        cfma(acc, a, mk_df(dff(v.x), dff(v.y)));
        y[i] = st_df(acc);
    }
}

inline cdff cdf_host(cd a) { return mk_df(dff_from(a.real()), dff_from(a.imag())); }

// Fused Gram-Schmidt pass on an Arnoldi vector: w += sum_i a_i V_i (the
// result kept to 48 bits, the precision of the basis), then in the same pass
// the dots conj(V_i) w (MODE 0: partial slots 0..K-1), |w|^2 (MODE 1: slot 0)
// or both (MODE 2: slots 0..K-1 and K): one read of V and w instead of two.
template <int K, int MODE>
__global__ void __launch_bounds__(kThreads) k_gs_df(double2 *w, PtrPack V, CoefDF a, size_t n, double2 *partial) {
    constexpr int R = MODE == 1 ? 1 : (MODE == 2 ? K + 1 : K);
    cdff acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = czero<cdff>();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        cdff v[K];
        cdff x = ld_df(w[e]);
#pragma unroll
        for (int i = 0; i < K; ++i) {
            v[i] = ld_df(static_cast<const double2 *>(V.p[i])[e]);
            cfma(x, mk_df(a.re[i], a.im[i]), v[i]);
        }
        x = cnorm(x);
        w[e] = st_df(x);
        if constexpr (MODE != 1) {
#pragma unroll
            for (int i = 0; i < K; ++i) cfma_conj(acc[i], v[i], x);
        }
        if constexpr (MODE != 0) cfma_conj(acc[R - 1], x, x);
    }
    __shared__ double2 red[kThreads / 32][R];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        double re = dff_to_double(acc[i].x), im = dff_to_double(acc[i].y);
        for (int off = 16; off > 0; off >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, off);
            im += __shfl_down_sync(0xffffffffu, im, off);
        }
        if (lane == 0) red[warp][i] = make_double2(re, im);
    }
    __syncthreads();
    if (threadIdx.x < R) {
        double re = 0.0, im = 0.0;
        for (int w2 = 0; w2 < kThreads / 32; ++w2) { re += red[w2][threadIdx.x].x; im += red[w2][threadIdx.x].y; }
        partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = make_double2(re, im);
    }
}

// per-block partial sums of conj(V_i) w, i < k; partial layout [i][block]
template <class T, int K>
__global__ void __launch_bounds__(kThreads) k_mdot(PtrPack V, const typename CT<T>::type *w, size_t n,
                                                   double2 *partial) {
    using C = typename CT<T>::type;
    double2 acc[K];
#pragma unroll
    for (int i = 0; i < K; ++i) acc[i] = make_double2(0.0, 0.0);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const C wv = w[e];
        const double wr = wv.x, wi = wv.y;
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const C v = static_cast<const C *>(V.p[i])[e];
            const double vr = v.x, vi = v.y;
            acc[i].x += vr * wr + vi * wi;
            acc[i].y += vr * wi - vi * wr;
        }
    }
    __shared__ double2 red[kThreads / 32][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        double re = acc[i].x, im = acc[i].y;
        for (int off = 16; off > 0; off >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, off);
            im += __shfl_down_sync(0xffffffffu, im, off);
        }
        if (lane == 0) red[warp][i] = make_double2(re, im);
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double re = 0.0, im = 0.0;
        for (int w2 = 0; w2 < kThreads / 32; ++w2) { re += red[w2][threadIdx.x].x; im += red[w2][threadIdx.x].y; }
        partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = make_double2(re, im);
    }
}

// result[i] = sum over blocks of partial[i][block] (one block per i, fixed order)
__global__ void k_finish(const double2 *partial, int blocks, double2 *result) {
    __shared__ double2 red[kThreads];
    const int i = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) {
        re += partial[(size_t)i * blocks + b].x;
        im += partial[(size_t)i * blocks + b].y;
    }
    red[threadIdx.x] = make_double2(re, im);
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[threadIdx.x].x += red[threadIdx.x + s].x;
            red[threadIdx.x].y += red[threadIdx.x + s].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) result[i] = red[0];
}

template <class T, int K>
__global__ void k_maxpy(typename CT<T>::type *w, PtrPack V, CoefPack a, size_t n) {
    using C = typename CT<T>::type;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        C acc = w[e];
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const C v = static_cast<const C *>(V.p[i])[e];
            acc.x += (T)a.re[i] * v.x - (T)a.im[i] * v.y;
            acc.y += (T)a.re[i] * v.y + (T)a.im[i] * v.x;
        }
        w[e] = acc;
    }
}

template <class T, int K>
void mdot_k(const PtrPack &pp, const void *w, size_t n, double2 *partial, int blocks, cudaStream_t st) {
    if constexpr (std::is_same<T, double>::value)
        k_mdot_df<K><<<blocks, kThreads, 0, st>>>(pp, static_cast<const double2 *>(w), n, partial);
    else
        k_mdot<T, K><<<blocks, kThreads, 0, st>>>(pp, static_cast<const typename CT<T>::type *>(w), n, partial);
}

template <class T>
void mdot_dispatch(int k, const PtrPack &pp, const void *w, size_t n, double2 *partial, int blocks,
                   cudaStream_t st) {
    switch (k) {
#define TDZ_CASE(K) case K: mdot_k<T, K>(pp, w, n, partial, blocks, st); break;
        TDZ_CASE(1) TDZ_CASE(2) TDZ_CASE(3) TDZ_CASE(4) TDZ_CASE(5) TDZ_CASE(6) TDZ_CASE(7) TDZ_CASE(8)
        TDZ_CASE(9) TDZ_CASE(10) TDZ_CASE(11) TDZ_CASE(12) TDZ_CASE(13) TDZ_CASE(14) TDZ_CASE(15) TDZ_CASE(16)
#undef TDZ_CASE
    default: throw Error(TDZ_ERR_INTERNAL, "bad multi-dot width");
    }
}

template <class T>
void maxpy_dispatch(int k, void *w, const PtrPack &pp, const CoefPack &cp, size_t n, cudaStream_t st) {
    using C = typename CT<T>::type;
    C *wp = static_cast<C *>(w);
    const int g = grid_for(n);
    switch (k) {
#define TDZ_CASE(K)                                                                            \
    case K:                                                                                    \
        if constexpr (std::is_same<T, double>::value)                                          \
            k_maxpy_df<K><<<g, kThreads, 0, st>>>(reinterpret_cast<double2 *>(wp), pp, coef_df(cp, K), n); \
        else                                                                                   \
            k_maxpy<T, K><<<g, kThreads, 0, st>>>(wp, pp, cp, n);                              \
        break;
        TDZ_CASE(1) TDZ_CASE(2) TDZ_CASE(3) TDZ_CASE(4) TDZ_CASE(5) TDZ_CASE(6) TDZ_CASE(7) TDZ_CASE(8)
        TDZ_CASE(9) TDZ_CASE(10) TDZ_CASE(11) TDZ_CASE(12) TDZ_CASE(13) TDZ_CASE(14) TDZ_CASE(15) TDZ_CASE(16)
#undef TDZ_CASE
    default: throw Error(TDZ_ERR_INTERNAL, "bad multi-axpy width");
    }
}

}  // namespace

void copy(const void *x, void *y, size_t n, int prec, cudaStream_t st) {
    const size_t bytes = n * (prec == TDZ_FP64 ? 16 : 8);
    if (x != y) TDZ_CUDA(cudaMemcpyAsync(y, x, bytes, cudaMemcpyDeviceToDevice, st));
}

void zero(void *x, size_t n, int prec, cudaStream_t st) {
    TDZ_CUDA(cudaMemsetAsync(x, 0, n * (prec == TDZ_FP64 ? 16 : 8), st));
}

void scale(void *x, cd a, size_t n, int prec, cudaStream_t st) {
    const int g = grid_for(n);
    if (prec == TDZ_FP64 && a.imag() == 0.0) k_scale_r64<<<g, kThreads, 0, st>>>(static_cast<double2 *>(x), a.real(), n);
    else if (prec == TDZ_FP64) k_scale_df<<<g, kThreads, 0, st>>>(static_cast<double2 *>(x), cdf_host(a), n);
    else k_scale<float><<<g, kThreads, 0, st>>>(static_cast<float2 *>(x), a.real(), a.imag(), n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void axpbypcz(void *y, cd a, const void *x, cd b, const void *z, cd c, size_t n, int prec, cudaStream_t st) {
    const int g = grid_for(n);
    if (prec == TDZ_FP64 && a.imag() == 0.0 && b.imag() == 0.0 && c.imag() == 0.0)
        k_axpbypcz_r64<<<g, kThreads, 0, st>>>(static_cast<double2 *>(y), a.real(), static_cast<const double2 *>(x),
                                               b.real(), static_cast<const double2 *>(z), c.real(), n);
    else if (prec == TDZ_FP64)
        k_axpbypcz_df<<<g, kThreads, 0, st>>>(static_cast<double2 *>(y), cdf_host(a), static_cast<const double2 *>(x),
                                              cdf_host(b), static_cast<const double2 *>(z), cdf_host(c),
                                              a != 0.0, b != 0.0, z != nullptr && c != 0.0, n);
    else
        k_axpbypcz<float><<<g, kThreads, 0, st>>>(static_cast<float2 *>(y), a.real(), a.imag(),
                                                  static_cast<const float2 *>(x), b.real(), b.imag(),
                                                  static_cast<const float2 *>(z), c.real(), c.imag(), n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void axpby(void *y, cd a, const void *x, cd b, size_t n, int prec, cudaStream_t st) {
    axpbypcz(y, a, x, b, nullptr, 0.0, n, prec, st);
}

void cast(const void *x, int px, void *y, int py, size_t n, cudaStream_t st) {
    const int g = grid_for(n);
    if (px == py) { copy(x, y, n, px, st); return; }
    if (px == TDZ_FP64)
        k_cast64to32_df<<<g, kThreads, 0, st>>>(static_cast<const double2 *>(x), static_cast<float2 *>(y), n);
    else k_cast32to64_df<<<g, kThreads, 0, st>>>(static_cast<const float2 *>(x), static_cast<double2 *>(y), n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

namespace {
__global__ void k_keep_real(double2 *x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        x[i].y = 0.0;
}
}  // namespace

void keep_real(void *x, size_t n, cudaStream_t st) {
    k_keep_real<<<grid_for(n), kThreads, 0, st>>>(static_cast<double2 *>(x), n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void add_cast(double2 *y, cd a, const float2 *x, size_t n, cudaStream_t st) {
    k_add_cast_df<<<grid_for(n), kThreads, 0, st>>>(y, cdf_host(a), x, n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void Reducer::init() {
    if (blocks) return;
    const int nb = red_blocks();
    partial.alloc(sizeof(double2) * (kMaxDot + 1) * nb);
    result.alloc(sizeof(double2) * (kMaxDot + 1));
    if (!host) TDZ_CUDA(cudaMallocHost(reinterpret_cast<void **>(&host), sizeof(double2) * (kMaxDot + 1)));
    blocks = nb;   // last: a Reducer with blocks != 0 has all its buffers
}

Reducer::~Reducer() {
    if (host) cudaFreeHost(host);
}

void mdot(Reducer &r, const void *const *V, int k, const void *w, size_t n, int prec, cd *out, cudaStream_t st) {
    r.init();
    for (int c0 = 0; c0 < k; c0 += kMaxDot) {
        const int kk = std::min(kMaxDot, k - c0);
        PtrPack pp{};
        for (int i = 0; i < kk; ++i) pp.p[i] = V[c0 + i];
        if (prec == TDZ_FP64) mdot_dispatch<double>(kk, pp, w, n, r.partial.as<double2>(), r.blocks, st);
        else mdot_dispatch<float>(kk, pp, w, n, r.partial.as<double2>(), r.blocks, st);
        k_finish<<<kk, kThreads, 0, st>>>(r.partial.as<double2>(), r.blocks, r.result.as<double2>());
        TDZ_CUDA(cudaGetLastError());
    count_launch();
        TDZ_CUDA(cudaMemcpyAsync(r.host, r.result.ptr, sizeof(double2) * kk, cudaMemcpyDeviceToHost, st));
        TDZ_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < kk; ++i) out[c0 + i] = cd(r.host[i].x, r.host[i].y);
    }
}

void dot_device(Reducer &r, const void *x, const void *y, size_t n, int prec, double2 *out, cudaStream_t st) {
    r.init();
    PtrPack pp{};
    pp.p[0] = x;
    if (prec == TDZ_FP64) mdot_dispatch<double>(1, pp, y, n, r.partial.as<double2>(), r.blocks, st);
    else mdot_dispatch<float>(1, pp, y, n, r.partial.as<double2>(), r.blocks, st);
    k_finish<<<1, kThreads, 0, st>>>(r.partial.as<double2>(), r.blocks, out);
    TDZ_CUDA(cudaGetLastError());
    count_launch(2);
}

void mdot_partials(const void *const *V, int k, const void *w, size_t n, int prec, double2 *partial, int blocks,
                   double2 *out, cudaStream_t st) {
    TDZ_CHECK(k >= 1 && k <= kMaxDot, TDZ_ERR_INTERNAL, "bad multi-dot width");
    PtrPack pp{};
    for (int i = 0; i < k; ++i) pp.p[i] = V[i];
    if (prec == TDZ_FP64) mdot_dispatch<double>(k, pp, w, n, partial, blocks, st);
    else mdot_dispatch<float>(k, pp, w, n, partial, blocks, st);
    k_finish<<<k, kThreads, 0, st>>>(partial, blocks, out);
    TDZ_CUDA(cudaGetLastError());
    count_launch(2);
}

void maxpy(void *w, int k, const void *const *V, const cd *a, size_t n, int prec, cudaStream_t st) {
    for (int c0 = 0; c0 < k; c0 += kMaxDot) {
        const int kk = std::min(kMaxDot, k - c0);
        PtrPack pp{};
        CoefPack cp{};
        for (int i = 0; i < kk; ++i) {
            pp.p[i] = V[c0 + i];
            cp.re[i] = a[c0 + i].real();
            cp.im[i] = a[c0 + i].imag();
        }
        if (prec == TDZ_FP64) maxpy_dispatch<double>(kk, w, pp, cp, n, st);
        else maxpy_dispatch<float>(kk, w, pp, cp, n, st);
        TDZ_CUDA(cudaGetLastError());
    count_launch();
    }
}

void gs_update(Reducer &r, void *w, int k, const void *const *V, const cd *a, size_t n, cd *dots, double *norm,
               cudaStream_t st) {
    TDZ_CHECK(k >= 1 && k <= kMaxDot, TDZ_ERR_INTERNAL, "fused Gram-Schmidt width");
    TDZ_CHECK(dots != nullptr || norm != nullptr, TDZ_ERR_INTERNAL, "dots or norm");
    r.init();
    PtrPack pp{};
    CoefPack cp{};
    for (int i = 0; i < k; ++i) {
        pp.p[i] = V[i];
        cp.re[i] = a[i].real();
        cp.im[i] = a[i].imag();
    }
    const CoefDF cd_ = coef_df(cp, k);
    double2 *wp = static_cast<double2 *>(w);
    double2 *part = r.partial.as<double2>();
    switch (k) {
#define TDZ_CASE(K)                                                                                       \
    case K:                                                                                               \
        if (dots && norm) k_gs_df<K, 2><<<r.blocks, kThreads, 0, st>>>(wp, pp, cd_, n, part);             \
        else if (norm) k_gs_df<K, 1><<<r.blocks, kThreads, 0, st>>>(wp, pp, cd_, n, part);               \
        else k_gs_df<K, 0><<<r.blocks, kThreads, 0, st>>>(wp, pp, cd_, n, part);                         \
        break;
        TDZ_CASE(1) TDZ_CASE(2) TDZ_CASE(3) TDZ_CASE(4) TDZ_CASE(5) TDZ_CASE(6) TDZ_CASE(7) TDZ_CASE(8)
        TDZ_CASE(9) TDZ_CASE(10) TDZ_CASE(11) TDZ_CASE(12) TDZ_CASE(13) TDZ_CASE(14) TDZ_CASE(15) TDZ_CASE(16)
#undef TDZ_CASE
    default: break;
    }
    const int nres = (dots ? k : 0) + (norm ? 1 : 0);
    k_finish<<<nres, kThreads, 0, st>>>(part, r.blocks, r.result.as<double2>());
    TDZ_CUDA(cudaGetLastError());
    count_launch(2);
    TDZ_CUDA(cudaMemcpyAsync(r.host, r.result.ptr, sizeof(double2) * nres, cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    if (dots)
        for (int i = 0; i < k; ++i) dots[i] = cd(r.host[i].x, r.host[i].y);
    if (norm) {
        const double v = r.host[nres - 1].x;
        *norm = std::isfinite(v) ? std::sqrt(std::max(0.0, v)) : std::numeric_limits<double>::quiet_NaN();
    }
}

void cn_combine(void *psi, const void *x, const void *z, cd c, size_t n, cudaStream_t st) {
    const int g = (int)std::min<size_t>((n + kThreads - 1) / kThreads, (size_t)red_blocks());
    k_cn_combine<<<g, kThreads, 0, st>>>(static_cast<double2 *>(psi), static_cast<const double2 *>(x),
                                         static_cast<const double2 *>(z), cdf_host(c), n);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

double nrm2(Reducer &r, const void *x, size_t n, int prec, cudaStream_t st) {
    cd v;
    const void *V[1] = {x};
    mdot(r, V, 1, x, n, prec, &v, st);
    if (!std::isfinite(v.real())) return std::numeric_limits<double>::quiet_NaN();
    return std::sqrt(std::max(0.0, v.real()));
}

}  // namespace blas
}  // namespace tdz
