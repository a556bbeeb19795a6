// Fast-diagonalisation preconditioner (Lynch-Rice-Thomas) for the z-layered
// operator family: dense eigenvector transforms along x and y and one banded
// complex LU solve per (x, y) line along z with the live stage coefficients.
// Exact inverse (up to FP32 rounding) when the inner axes carry only mass and
// stiffness, which is the heterostructure's case. 3D with n_x, n_y <= 256:
// the transforms run on the tensor cores (tgemm.cu) over row-planar FP32
// buffers; otherwise (2D, wider axes) on the smem-tiled FP32 GEMMs below.
#include "fdm.h"

#include <cmath>

#include "apply_kernels.cuh"

namespace tdz {

// ---------------------------------------------------------------- host eigen
void gen_eig(const BandD &S, const BandD &M, std::vector<double> &V, std::vector<double> &lam) {
    const int n = S.n, p = S.p;
    std::vector<double> L((size_t)n * n, 0.0), C((size_t)n * n, 0.0);
    auto m = [&](int i, int j) { return std::abs(i - j) <= p ? M.at(i, j) : 0.0; };
    auto s = [&](int i, int j) { return std::abs(i - j) <= p ? S.at(i, j) : 0.0; };
    // Cholesky M = L L^T (banded)
    for (int i = 0; i < n; ++i)
        for (int j = std::max(0, i - p); j <= i; ++j) {
            double v = m(i, j);
            for (int k = std::max(0, i - p); k < j; ++k) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            if (i == j) {
                TDZ_CHECK(v > 0, TDZ_ERR_INTERNAL, "mass band not positive definite");
                L[(size_t)i * n + i] = std::sqrt(v);
            } else L[(size_t)i * n + j] = v / L[(size_t)j * n + j];
        }
    // C = L^-1 S L^-T : first W = L^-1 S (columns), then C = W L^-T
    std::vector<double> W((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            double v = s(i, c);
            for (int k = std::max(0, i - p); k < i; ++k) v -= L[(size_t)i * n + k] * W[(size_t)k * n + c];
            W[(size_t)i * n + c] = v / L[(size_t)i * n + i];
        }
    for (int r = 0; r < n; ++r)
        for (int i = 0; i < n; ++i) {
            double v = W[(size_t)r * n + i];
            for (int k = std::max(0, i - p); k < i; ++k) v -= L[(size_t)i * n + k] * C[(size_t)r * n + k];
            C[(size_t)r * n + i] = v / L[(size_t)i * n + i];
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            const double a = 0.5 * (C[(size_t)i * n + j] + C[(size_t)j * n + i]);
            C[(size_t)i * n + j] = C[(size_t)j * n + i] = a;
        }
    // cyclic Jacobi on C, accumulate Q
    std::vector<double> Q((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double v = C[(size_t)i * n + j] * C[(size_t)i * n + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * tot) break;
        for (int pi = 0; pi < n - 1; ++pi)
            for (int qi = pi + 1; qi < n; ++qi) {
                const double apq = C[(size_t)pi * n + qi];
                if (std::abs(apq) < 1e-300) continue;
                const double app = C[(size_t)pi * n + pi], aqq = C[(size_t)qi * n + qi];
                const double theta = 0.5 * (aqq - app) / apq;
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = C[(size_t)k * n + pi], akq = C[(size_t)k * n + qi];
                    C[(size_t)k * n + pi] = c * akp - sn * akq;
                    C[(size_t)k * n + qi] = sn * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = C[(size_t)pi * n + k], aqk = C[(size_t)qi * n + k];
                    C[(size_t)pi * n + k] = c * apk - sn * aqk;
                    C[(size_t)qi * n + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double qkp = Q[(size_t)k * n + pi], qkq = Q[(size_t)k * n + qi];
                    Q[(size_t)k * n + pi] = c * qkp - sn * qkq;
                    Q[(size_t)k * n + qi] = sn * qkp + c * qkq;
                }
            }
    }
    lam.assign(n, 0.0);
    for (int i = 0; i < n; ++i) lam[i] = C[(size_t)i * n + i];
    // V = L^-T Q (back substitution with L^T, column by column)
    V.assign((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int i = n - 1; i >= 0; --i) {
            double v = Q[(size_t)i * n + c];
            for (int k = i + 1; k <= std::min(n - 1, i + p); ++k) v -= L[(size_t)k * n + i] * V[(size_t)k * n + c];
            V[(size_t)i * n + c] = v / L[(size_t)i * n + i];
        }
}

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

// multiply-accumulate of the transforms: complex data times a real or complex
// matrix entry (FP32, or FP64 for the FP64 preconditioner)
template <class C, class R> __device__ __forceinline__ void gmac(C &acc, C a, R b) {
    acc.x = fma(a.x, b, acc.x);
    acc.y = fma(a.y, b, acc.y);
}
template <class C, class R> __device__ __forceinline__ void gmac_r(C &acc, R a, C b) {
    acc.x = fma(a, b.x, acc.x);
    acc.y = fma(a, b.y, acc.y);
}
template <class C> __device__ __forceinline__ void gmac_c(C &acc, C a, C b) {
    acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
    acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
__device__ __forceinline__ void gmac2(float2 &acc, float2 a, float b) { gmac(acc, a, b); }
__device__ __forceinline__ void gmac2(float2 &acc, float a, float2 b) { gmac_r(acc, a, b); }
__device__ __forceinline__ void gmac2(float2 &acc, float2 a, float2 b) { gmac_c(acc, a, b); }
__device__ __forceinline__ void gmac2(double2 &acc, double2 a, double b) { gmac(acc, a, b); }
__device__ __forceinline__ void gmac2(double2 &acc, double a, double2 b) { gmac_r(acc, a, b); }
__device__ __forceinline__ void gmac2(double2 &acc, double2 a, double2 b) { gmac_c(acc, a, b); }
template <class T> __device__ __forceinline__ T gzero();
template <> __device__ __forceinline__ float gzero<float>() { return 0.f; }
template <> __device__ __forceinline__ float2 gzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double gzero<double>() { return 0.0; }
template <> __device__ __forceinline__ double2 gzero<double2>() { return make_double2(0.0, 0.0); }

// C[M][N] (complex C2) = A[M][K] (complex, row-major) . B[K][N] (real, or
// complex for complex axis pencils)
template <class C2, class TB>
__global__ void __launch_bounds__(256) k_gemm_cr(const C2 *__restrict__ A, const TB *__restrict__ B,
                                                 C2 *__restrict__ Cm, int M, int N, int K) {
    __shared__ C2 As[BK][BM + 1];
    __shared__ TB Bs[BK][BN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    C2 acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = gzero<C2>();
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int i = threadIdx.x; i < BM * BK; i += 256) {
            const int r = i / BK, k = i % BK;
            const int gm = m0 + r, gk = k0 + k;
            As[k][r] = (gm < M && gk < K) ? A[(size_t)gm * K + gk] : gzero<C2>();
        }
        for (int i = threadIdx.x; i < BK * BN; i += 256) {
            const int k = i / BN, c = i % BN;
            const int gk = k0 + k, gn = n0 + c;
            Bs[k][c] = (gk < K && gn < N) ? B[(size_t)gk * N + gn] : gzero<TB>();
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            C2 a[4];
            TB b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[k][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[k][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) gmac2(acc[r][c], a[r], b[c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int gm = m0 + ty * 4 + r, gn = n0 + tx * 4 + c;
            if (gm < M && gn < N) Cm[(size_t)gm * N + gn] = acc[r][c];
        }
}

// per plane z: C_z[M][N] (complex C2) = A[M][K] (real, or complex for
// complex axis pencils; row-major) . B_z[K][N] (complex)
template <class C2, class TA>
__global__ void __launch_bounds__(256) k_gemm_rc(const TA *__restrict__ A, const C2 *__restrict__ B,
                                                 C2 *__restrict__ Cm, int M, int N, int K) {
    __shared__ TA As[BK][BM + 4];
    __shared__ C2 Bs[BK][BN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const size_t plane = (size_t)blockIdx.z;
    const C2 *Bz = B + plane * (size_t)K * N;
    C2 *Cz = Cm + plane * (size_t)M * N;
    C2 acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = gzero<C2>();
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int i = threadIdx.x; i < BM * BK; i += 256) {
            const int r = i / BK, k = i % BK;
            const int gm = m0 + r, gk = k0 + k;
            As[k][r] = (gm < M && gk < K) ? A[(size_t)gm * K + gk] : gzero<TA>();
        }
        for (int i = threadIdx.x; i < BK * BN; i += 256) {
            const int k = i / BN, c = i % BN;
            const int gk = k0 + k, gn = n0 + c;
            Bs[k][c] = (gk < K && gn < N) ? Bz[(size_t)gk * N + gn] : gzero<C2>();
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            TA a[4];
            C2 b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[k][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[k][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) gmac2(acc[r][c], a[r], b[c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int gm = m0 + ty * 4 + r, gn = n0 + tx * 4 + c;
            if (gm < M && gn < N) Cz[(size_t)gm * N + gn] = acc[r][c];
        }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 crecf(float2 a) {
    const float d = 1.f / (a.x * a.x + a.y * a.y);
    return make_float2(a.x * d, -a.y * d);
}

// natural-order complex FP64 -> row-planar FP32 [z][y][c][x] (row pitch ld)
__global__ void k_to_planar(const double2 *__restrict__ r, float *__restrict__ a, int n0, size_t rows, int ld) {
    const size_t total = rows * (size_t)n0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t row = e / n0;
        const int x = (int)(e % n0);
        const double2 v = r[e];   // FP64 -> FP32 without the (slow) FP64 pipe
        const dff re = dff_split(v.x), im = dff_split(v.y);
        a[(row * 2) * ld + x] = __fadd_rn(re.hi, re.lo);
        a[(row * 2 + 1) * ld + x] = __fadd_rn(im.hi, im.lo);
    }
}

// the same with ||z||^2: FP32 sums per thread (a few dozen squares of FP32
// values), FP64 per block into part[block]
__global__ void __launch_bounds__(256) k_from_planar_norm(const float *__restrict__ a, double2 *__restrict__ z, int n0,
                                                          size_t rows, int ld, double *__restrict__ part) {
    const size_t total = rows * (size_t)n0;
    float acc = 0.f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t row = e / n0;
        const int x = (int)(e % n0);
        const float re = a[(row * 2) * ld + x], im = a[(row * 2 + 1) * ld + x];
        z[e] = make_double2(f2d_exact(re), f2d_exact(im));
        acc = fmaf(re, re, fmaf(im, im, acc));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = (double)acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        part[blockIdx.x] = t;
    }
}

// *out = sum of part[0 .. n) in a fixed order (one block)
__global__ void __launch_bounds__(256) k_sum_parts(const double *__restrict__ part, int n, double *out) {
    __shared__ double ws[256];
    double t = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) t += part[i];
    ws[threadIdx.x] = t;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) ws[threadIdx.x] += ws[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = ws[0];
}

__global__ void k_from_planar(const float *__restrict__ a, double2 *__restrict__ z, int n0, size_t rows, int ld) {
    const size_t total = rows * (size_t)n0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t row = e / n0;
        const int x = (int)(e % n0);
        z[e] = make_double2(f2d_exact(a[(row * 2) * ld + x]), f2d_exact(a[(row * 2 + 1) * ld + x]));
    }
}

struct ZSolveParams {
    float *x;               // in/out: real part of (line (i, j), row k) at x[k ks + j js + i is], imaginary at + cs
    size_t ks;
    int js, is, cs;
    float2 *ck;             // scratch: elimination state at the start of each row block, [b][e][line]
    float2 *zb;             // scratch: the band rows of Bc, then of Cc, [2][n2][bw]
    const float *bands;     // outer base bands [nb][n2][bw]
    const float *lx, *ly;   // inner eigenvalues
    const float *lxi, *lyi; // their imaginary parts (complex axis pencils), else null
    int n0, n1, n2;
    CombP<float> Bc, Cc;    // A_z(s) = Bc + s Cc
};

// One banded complex LU (no pivoting) + solve per line (i, j), one thread
// per line, lines contiguous in memory (coalesced across the warp).
//
// The U factor is not stored. The forward pass runs the elimination and the
// forward substitution down the line and saves only the elimination state
// (the last P rows of U with their reciprocal pivots, and the last P entries
// of L^-1 r) at the start of every block of ZBlk::B rows. The backward pass
// walks the blocks bottom-up: from the block's saved state it redoes the
// block's elimination (U rows into shared memory, L^-1 r into registers), then
// back-substitutes the block and writes the solution in place. Per row that
// is 8 bytes read and the state in the forward pass, 8 bytes read, 8 written
// and the state in the backward pass (about 40 bytes for P = 3, against
// 96 with a stored U), and no stores in the forward pass at all. The block's
// right-hand side and state are prefetched into registers one block ahead;
// the forward pass streams its rows kZDist ahead through asynchronous copies
// into shared memory. The band rows of Bc and Cc are evaluated once per solve
// (k_zbands) and copied into each CTA's shared memory.
constexpr int kZDist = 32, kZThreads = 128;
template <int P> struct ZBlk {
    static constexpr int B = P <= 3 ? 16 : 8;        // rows per block (divides kZDist)
    static constexpr int NS = P * (P + 1) + P;       // complex entries of the saved state
    static_assert(B * (P + 1) >= kZDist, "the U block doubles as the forward pass's row ring");
};

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int P> size_t zsolve_smem(int n2) {
    return ((size_t)2 * n2 * (2 * P + 1) + (size_t)ZBlk<P>::B * (P + 1) * kZThreads) * sizeof(float2);
}

// the band rows of A_z(s) = Bc + s Cc for the current stage: [2][n2][2P+1]
__global__ void k_zbands(const ZSolveParams prm, int bw) {
    const int n = prm.n2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * bw; e += gridDim.x * blockDim.x) {
        const int k = e / bw, o = e % bw;
        prm.zb[e] = comb_at<float, float2>(prm.Bc, prm.bands, n, bw, k, o);
        prm.zb[(size_t)n * bw + e] = comb_at<float, float2>(prm.Cc, prm.bands, n, bw, k, o);
    }
}

template <int P, bool CI>
__global__ void __launch_bounds__(kZThreads) k_zsolve(const ZSolveParams prm) {
    constexpr int BWd = 2 * P + 1, B = ZBlk<P>::B, NS = ZBlk<P>::NS;
    static_assert(kZDist % B == 0, "row blocks must tile the prefetch ring");
    extern __shared__ float2 zs_smem[];
    const int n = prm.n2;
    float2 *sB = zs_smem, *sC = zs_smem + (size_t)n * BWd;          // band rows of Bc and Cc
    float2 *sU = zs_smem + (size_t)2 * n * BWd;                      // [row of block][q][thread]
    for (int e = threadIdx.x; e < 2 * n * BWd; e += blockDim.x) sB[e] = prm.zb[e];
    __syncthreads();
    const int nl = prm.n0 * prm.n1;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    const int i = l % prm.n0, j = l / prm.n0;
    const float s = prm.lx[i] + (prm.ly ? prm.ly[j] : 0.f);
    const float si = CI ? prm.lxi[i] + (prm.lyi ? prm.lyi[j] : 0.f) : 0.f;
    float *xl = prm.x + (size_t)j * prm.js + (size_t)i * prm.is;
    const size_t ks = prm.ks;
    const int cs = prm.cs;
    auto ldx = [&](int k) { const float *q = xl + (size_t)k * ks; return make_float2(q[0], q[cs]); };
    auto stx = [&](int k, float2 v) { float *q = xl + (size_t)k * ks; q[0] = v.x; q[cs] = v.y; };
    float2 *ck = prm.ck + l;
    const size_t cst = (size_t)nl;

    float2 Uw[P][P + 1];     // U rows k-1 .. k-P; [0] holds the reciprocal pivot
    float2 yw[P];            // L^-1 r at rows k-1 .. k-P
    auto reset = [&]() {
#pragma unroll
        for (int d = 0; d < P; ++d) {
            yw[d] = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q <= P; ++q) Uw[d][q] = make_float2(1.f, 0.f);
        }
    };
    // row k: eliminate columns k-P .. k-1 with the U rows in Uw; shifts the
    // new U row into Uw[0] and L^-1 r into yw[0]
    auto eliminate = [&](int k, float2 rhs) {
        float2 a[BWd];
#pragma unroll
        for (int o = 0; o < BWd; ++o) {
            const float2 b = sB[k * BWd + o], c = sC[k * BWd + o];
            a[o] = CI ? make_float2(fmaf(-si, c.y, fmaf(s, c.x, b.x)), fmaf(si, c.x, fmaf(s, c.y, b.y)))
                      : make_float2(fmaf(s, c.x, b.x), fmaf(s, c.y, b.y));
        }
#pragma unroll
        for (int d = P; d >= 1; --d) {
            if (k - d < 0) continue;
            const float2 *Ur = Uw[d - 1];   // row k-d: Ur[q] = U(k-d, k-d+q), Ur[0] = 1 / U(k-d, k-d)
            const float2 f = cmulf(a[P - d], Ur[0]);
#pragma unroll
            for (int q = 1; q <= P; ++q) {
                const float2 t = cmulf(f, Ur[q]);
                a[P - d + q].x -= t.x;
                a[P - d + q].y -= t.y;
            }
            const float2 t = cmulf(f, yw[d - 1]);
            rhs.x -= t.x;
            rhs.y -= t.y;
        }
        a[P] = crecf(a[P]);
#pragma unroll
        for (int d = P - 1; d > 0; --d) {
            yw[d] = yw[d - 1];
#pragma unroll
            for (int q = 0; q <= P; ++q) Uw[d][q] = Uw[d - 1][q];
        }
#pragma unroll
        for (int q = 0; q <= P; ++q) Uw[0][q] = a[P + q];
        yw[0] = rhs;
    };

    // forward pass: the state at the start of blocks 1 .. nb-1. The rows
    // stream through a kZDist-deep ring in shared memory (this thread's
    // column of the U block, free until the backward pass) filled by
    // asynchronous copies, one commit group per row, so kZDist rows are
    // always in flight whatever the compiler's schedule.
    reset();
    {
        float *ring = reinterpret_cast<float *>(sU + threadIdx.x);   // slot u: ring[2 u kZThreads + {0, 1}]
        auto issue = [&](int k, int u) {
            if (k < n) {
                const float *q = xl + (size_t)k * ks;
                cp_async4(ring + (size_t)2 * u * kZThreads, q);
                cp_async4(ring + (size_t)2 * u * kZThreads + 1, q + cs);
            }
            cp_async_commit();
        };
#pragma unroll
        for (int u = 0; u < kZDist; ++u) issue(u, u);
        for (int k0 = 0; k0 < n; k0 += kZDist) {
#pragma unroll
            for (int u = 0; u < kZDist; ++u) {
                const int k = k0 + u;
                if (k < n) {
                    if (u % B == 0 && k > 0) {
                        float2 *c = ck + (size_t)(k / B) * NS * cst;
#pragma unroll
                        for (int d = 0; d < P; ++d) {
#pragma unroll
                            for (int q = 0; q <= P; ++q) c[(size_t)(d * (P + 1) + q) * cst] = Uw[d][q];
                            c[(size_t)(P * (P + 1) + d) * cst] = yw[d];
                        }
                    }
                    cp_async_wait<kZDist - 1>();   // row k has landed
                    const float2 rhs = *reinterpret_cast<const float2 *>(ring + (size_t)2 * u * kZThreads);
                    issue(k + kZDist, u);
                    eliminate(k, rhs);
                }
            }
        }
        cp_async_wait<0>();
    }

    // backward pass, blocks nb-1 .. 0; a block's rows and saved state are
    // loaded into registers one block ahead
    const int nb = (n + B - 1) / B;
    float2 nr[B], nst[NS];
    auto fetch = [&](int b) {
#pragma unroll
        for (int r = 0; r < B; ++r) {
            const int k = b * B + r;
            nr[r] = k < n ? ldx(k) : make_float2(0.f, 0.f);
        }
        if (b > 0) {
            const float2 *c = ck + (size_t)b * NS * cst;
#pragma unroll
            for (int e = 0; e < NS; ++e) nst[e] = c[(size_t)e * cst];
        }
    };
    float2 xw[P];
#pragma unroll
    for (int d = 0; d < P; ++d) xw[d] = make_float2(0.f, 0.f);
    float2 *su = sU + threadIdx.x;
    fetch(nb - 1);
    for (int b = nb - 1; b >= 0; --b) {
        float2 rr[B];
#pragma unroll
        for (int r = 0; r < B; ++r) rr[r] = nr[r];
        if (b > 0) {
#pragma unroll
            for (int d = 0; d < P; ++d) {
#pragma unroll
                for (int q = 0; q <= P; ++q) Uw[d][q] = nst[d * (P + 1) + q];
                yw[d] = nst[P * (P + 1) + d];
            }
        } else {
            reset();
        }
        if (b > 0) fetch(b - 1);
        // redo the block's elimination
        float2 yb[B];
#pragma unroll
        for (int r = 0; r < B; ++r) {
            const int k = b * B + r;
            yb[r] = make_float2(0.f, 0.f);
            if (k < n) {
                eliminate(k, rr[r]);
                yb[r] = yw[0];
#pragma unroll
                for (int q = 0; q <= P; ++q) su[(size_t)(r * (P + 1) + q) * kZThreads] = Uw[0][q];
            }
        }
        // back substitution of the block
#pragma unroll
        for (int r = B - 1; r >= 0; --r) {
            const int k = b * B + r;
            if (k < n) {
                float2 v = yb[r];
#pragma unroll
                for (int q = 1; q <= P; ++q) {
                    if (k + q >= n) continue;
                    const float2 t = cmulf(su[(size_t)(r * (P + 1) + q) * kZThreads], xw[q - 1]);
                    v.x -= t.x;
                    v.y -= t.y;
                }
                v = cmulf(v, su[(size_t)(r * (P + 1)) * kZThreads]);
#pragma unroll
                for (int d = P - 1; d > 0; --d) xw[d] = xw[d - 1];
                xw[0] = v;
                stx(k, v);
            }
        }
    }
}

// ---- twisted line solve: two threads per line
// The line is cut at the twist m (a multiple of the block length). One thread
// factors rows 0 .. m-1 from the top, its partner rows n-1 .. m from the
// bottom (the same elimination on the reversed line: for a complex-symmetric
// band matrix, row k read backwards). Each half's elimination runs over the
// band's columns past its end too, so its last P rows of U carry the
// coupling to the other half. The two final elimination states meet in shared
// memory, where both threads solve the same 2P x 2P system for the P unknowns
// on either side of the twist: with the tail rows scaled by the reciprocal
// pivots, U1 T1 + W1 T2 = c1 and U2 T2 + W2 T1 = c2 (U unit upper
// triangular), so S T2 = c2 - W2 U1^-1 c1 with S = U2 - W2 U1^-1 W1, and
// T1 = U1^-1 (c1 - W1 T2). Each thread then back-substitutes its half from the
// partner's tail values. This doubles the threads of the latency-bound
// recursion and halves its length.
constexpr int kZ2Lines = 64;                     // lines per CTA (two threads each)
template <int P> struct ZBlk2 {
    static constexpr int B = P == 2 ? 16 : 8;    // rows per block
    static constexpr int NS = P * (P + 1) + P;
    static_assert(B * (P + 1) >= kZDist, "the U block doubles as the row ring");
    static_assert(NS <= B * (P + 1), "the U block doubles as the exchange buffer");
};

template <int P> size_t zsolve2_smem(int n2) {
    return ((size_t)2 * n2 * (2 * P + 1) + (size_t)ZBlk2<P>::B * (P + 1) * 2 * kZ2Lines) * sizeof(float2);
}
__host__ __device__ inline int zsolve2_twist(int n2, int B) { return B * ((n2 + B) / (2 * B)); }

__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

template <int P, bool CI>
__global__ void __launch_bounds__(2 * kZ2Lines) k_zsolve2(const ZSolveParams prm) {
    constexpr int BWd = 2 * P + 1, B = ZBlk2<P>::B, NS = ZBlk2<P>::NS, T = 2 * kZ2Lines;
    static_assert(kZDist % B == 0, "row blocks must tile the prefetch ring");
    extern __shared__ float2 zs_smem[];
    const int n = prm.n2;
    float2 *sB = zs_smem, *sC = zs_smem + (size_t)n * BWd;
    float2 *sU = zs_smem + (size_t)2 * n * BWd;   // [slot][thread]: row ring, exchange, U block
    for (int e = threadIdx.x; e < 2 * n * BWd; e += blockDim.x) sB[e] = prm.zb[e];
    __syncthreads();
    const int half = threadIdx.x / kZ2Lines;       // 0: rows 0 .. m-1, 1: rows n-1 .. m
    const int li = threadIdx.x % kZ2Lines;
    const int nl = prm.n0 * prm.n1;
    const int lraw = blockIdx.x * kZ2Lines + li;
    const bool valid = lraw < nl;
    const int l = valid ? lraw : nl - 1;           // idle threads shadow a real line, store nothing
    const int m = zsolve2_twist(n, B);
    const int L = half ? n - m : m;                // rows of this half
    const int i = l % prm.n0, j = l / prm.n0;
    const float s = prm.lx[i] + (prm.ly ? prm.ly[j] : 0.f);
    const float si = CI ? prm.lxi[i] + (prm.lyi ? prm.lyi[j] : 0.f) : 0.f;
    float *xl = prm.x + (size_t)j * prm.js + (size_t)i * prm.is;
    const size_t ks = prm.ks;
    const int cs = prm.cs;
    auto phys = [&](int k) { return half ? n - 1 - k : k; };
    auto ldx = [&](int k) { const float *q = xl + (size_t)phys(k) * ks; return make_float2(q[0], q[cs]); };
    auto stx = [&](int k, float2 v) {
        if (valid) {
            float *q = xl + (size_t)phys(k) * ks;
            q[0] = v.x;
            q[cs] = v.y;
        }
    };
    const size_t cst = (size_t)nl;
    float2 *ck = prm.ck + (size_t)(half ? (m + B - 1) / B : 0) * NS * cst + l;

    float2 Uw[P][P + 1];
    float2 yw[P];
    auto reset = [&]() {
#pragma unroll
        for (int d = 0; d < P; ++d) {
            yw[d] = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q <= P; ++q) Uw[d][q] = make_float2(1.f, 0.f);
        }
    };
    // local row k of this half (its band row read backwards in the bottom half)
    auto eliminate = [&](int k, float2 rhs) {
        float2 a[BWd];
        const int pr = phys(k);
#pragma unroll
        for (int o = 0; o < BWd; ++o) {
            const int oo = half ? 2 * P - o : o;
            const float2 b = sB[pr * BWd + oo], c = sC[pr * BWd + oo];
            a[o] = CI ? make_float2(fmaf(-si, c.y, fmaf(s, c.x, b.x)), fmaf(si, c.x, fmaf(s, c.y, b.y)))
                      : make_float2(fmaf(s, c.x, b.x), fmaf(s, c.y, b.y));
        }
#pragma unroll
        for (int d = P; d >= 1; --d) {
            if (k - d < 0) continue;
            const float2 *Ur = Uw[d - 1];
            const float2 f = cmulf(a[P - d], Ur[0]);
#pragma unroll
            for (int q = 1; q <= P; ++q) {
                const float2 t = cmulf(f, Ur[q]);
                a[P - d + q].x -= t.x;
                a[P - d + q].y -= t.y;
            }
            const float2 t = cmulf(f, yw[d - 1]);
            rhs.x -= t.x;
            rhs.y -= t.y;
        }
        a[P] = crecf(a[P]);
#pragma unroll
        for (int d = P - 1; d > 0; --d) {
            yw[d] = yw[d - 1];
#pragma unroll
            for (int q = 0; q <= P; ++q) Uw[d][q] = Uw[d - 1][q];
        }
#pragma unroll
        for (int q = 0; q <= P; ++q) Uw[0][q] = a[P + q];
        yw[0] = rhs;
    };

    // forward pass of this half, rows streamed through the ring
    reset();
    {
        float *ring = reinterpret_cast<float *>(sU + threadIdx.x);
        auto issue = [&](int k, int u) {
            if (k < L) {
                const float *q = xl + (size_t)phys(k) * ks;
                cp_async4(ring + (size_t)2 * u * T, q);
                cp_async4(ring + (size_t)2 * u * T + 1, q + cs);
            }
            cp_async_commit();
        };
#pragma unroll
        for (int u = 0; u < kZDist; ++u) issue(u, u);
        for (int k0 = 0; k0 < L; k0 += kZDist) {
#pragma unroll
            for (int u = 0; u < kZDist; ++u) {
                const int k = k0 + u;
                if (k < L) {
                    if (u % B == 0 && k > 0 && valid) {
                        float2 *c = ck + (size_t)(k / B) * NS * cst;
#pragma unroll
                        for (int d = 0; d < P; ++d) {
#pragma unroll
                            for (int q = 0; q <= P; ++q) c[(size_t)(d * (P + 1) + q) * cst] = Uw[d][q];
                            c[(size_t)(P * (P + 1) + d) * cst] = yw[d];
                        }
                    }
                    cp_async_wait<kZDist - 1>();
                    const float2 rhs = *reinterpret_cast<const float2 *>(ring + (size_t)2 * u * T);
                    issue(k + kZDist, u);
                    eliminate(k, rhs);
                }
            }
        }
        cp_async_wait<0>();
    }

    // exchange the final states and solve the twist system (same arithmetic in both threads)
    float2 *ex = sU;   // [e][thread]
#pragma unroll
    for (int d = 0; d < P; ++d) {
#pragma unroll
        for (int q = 0; q <= P; ++q) ex[(size_t)(d * (P + 1) + q) * T + threadIdx.x] = Uw[d][q];
        ex[(size_t)(P * (P + 1) + d) * T + threadIdx.x] = yw[d];
    }
    __syncthreads();
    float2 U1[P][P], W1[P][P], c1[P], U2[P][P], W2[P][P], c2[P];
    auto tail = [&](int col, float2 (&U)[P][P], float2 (&W)[P][P], float2 (&c)[P]) {
        auto st = [&](int e) { return ex[(size_t)e * T + col]; };
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const int d = P - 1 - r;
            const float2 rp = st(d * (P + 1));
#pragma unroll
            for (int k = 0; k < P; ++k) {
                U[r][k] = k > r ? cmulf(rp, st(d * (P + 1) + (k - r))) : make_float2(0.f, 0.f);
                W[r][k] = k >= P - 1 - r ? cmulf(rp, st(d * (P + 1) + (2 * P - 1 - r - k))) : make_float2(0.f, 0.f);
            }
            c[r] = cmulf(rp, st(P * (P + 1) + d));
        }
    };
    tail(li, U1, W1, c1);
    tail(li + kZ2Lines, U2, W2, c2);
    __syncthreads();   // the exchange buffer is this thread's U block from here on
    // z1 = U1^-1 c1, M1 = U1^-1 W1 (unit upper triangular)
    float2 z1[P], M1[P][P];
#pragma unroll
    for (int r = P - 1; r >= 0; --r) {
        z1[r] = c1[r];
#pragma unroll
        for (int k = 0; k < P; ++k) M1[r][k] = W1[r][k];
#pragma unroll
        for (int q = r + 1; q < P; ++q) {
            z1[r] = csubf(z1[r], cmulf(U1[r][q], z1[q]));
#pragma unroll
            for (int k = 0; k < P; ++k) M1[r][k] = csubf(M1[r][k], cmulf(U1[r][q], M1[q][k]));
        }
    }
    // S = U2 + I - W2 M1 (U2 holds the strict upper part), g = c2 - W2 z1
    float2 S[P][P], g[P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
        g[r] = c2[r];
#pragma unroll
        for (int k = 0; k < P; ++k) S[r][k] = k == r ? make_float2(1.f, 0.f) : U2[r][k];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            g[r] = csubf(g[r], cmulf(W2[r][q], z1[q]));
#pragma unroll
            for (int k = 0; k < P; ++k) S[r][k] = csubf(S[r][k], cmulf(W2[r][q], M1[q][k]));
        }
    }
    // S T2 = g: Gaussian elimination without pivoting, then T1 = z1 - M1 T2
#pragma unroll
    for (int c = 0; c < P; ++c) {
        const float2 inv = crecf(S[c][c]);
#pragma unroll
        for (int r = c + 1; r < P; ++r) {
            const float2 f = cmulf(S[r][c], inv);
#pragma unroll
            for (int k = c + 1; k < P; ++k) S[r][k] = csubf(S[r][k], cmulf(f, S[c][k]));
            g[r] = csubf(g[r], cmulf(f, g[c]));
        }
        S[c][c] = inv;
    }
    float2 T2[P], T1[P];
#pragma unroll
    for (int r = P - 1; r >= 0; --r) {
        float2 v = g[r];
#pragma unroll
        for (int k = r + 1; k < P; ++k) v = csubf(v, cmulf(S[r][k], T2[k]));
        T2[r] = cmulf(v, S[r][r]);
    }
#pragma unroll
    for (int r = 0; r < P; ++r) {
        T1[r] = z1[r];
#pragma unroll
        for (int k = 0; k < P; ++k) T1[r] = csubf(T1[r], cmulf(M1[r][k], T2[k]));
    }

    // backward pass of this half; row L + c of this half is the partner's tail row P-1-c
    const int nb = (L + B - 1) / B;
    float2 nr[B], nst[NS];
    auto fetch = [&](int b) {
#pragma unroll
        for (int r = 0; r < B; ++r) {
            const int k = b * B + r;
            nr[r] = k < L ? ldx(k) : make_float2(0.f, 0.f);
        }
        if (b > 0) {
            const float2 *c = ck + (size_t)b * NS * cst;
#pragma unroll
            for (int e = 0; e < NS; ++e) nst[e] = c[(size_t)e * cst];
        }
    };
    float2 xw[P];
#pragma unroll
    for (int c = 0; c < P; ++c) xw[c] = half ? T1[P - 1 - c] : T2[P - 1 - c];
    float2 *su = sU + threadIdx.x;
    fetch(nb - 1);
    for (int b = nb - 1; b >= 0; --b) {
        float2 rr[B];
#pragma unroll
        for (int r = 0; r < B; ++r) rr[r] = nr[r];
        if (b > 0) {
#pragma unroll
            for (int d = 0; d < P; ++d) {
#pragma unroll
                for (int q = 0; q <= P; ++q) Uw[d][q] = nst[d * (P + 1) + q];
                yw[d] = nst[P * (P + 1) + d];
            }
        } else {
            reset();
        }
        if (b > 0) fetch(b - 1);
        float2 yb[B];
#pragma unroll
        for (int r = 0; r < B; ++r) {
            const int k = b * B + r;
            yb[r] = make_float2(0.f, 0.f);
            if (k < L) {
                eliminate(k, rr[r]);
                yb[r] = yw[0];
#pragma unroll
                for (int q = 0; q <= P; ++q) su[(size_t)(r * (P + 1) + q) * T] = Uw[0][q];
            }
        }
#pragma unroll
        for (int r = B - 1; r >= 0; --r) {
            const int k = b * B + r;
            if (k < L) {
                float2 v = yb[r];
#pragma unroll
                for (int q = 1; q <= P; ++q) v = csubf(v, cmulf(su[(size_t)(r * (P + 1) + q) * T], xw[q - 1]));
                v = cmulf(v, su[(size_t)(r * (P + 1)) * T]);
#pragma unroll
                for (int d = P - 1; d > 0; --d) xw[d] = xw[d - 1];
                xw[0] = v;
                stx(k, v);
            }
        }
    }
}

template <int P, bool CI> void launch_zsolve_t(const ZSolveParams &zp, cudaStream_t st) {
    constexpr size_t kMax = 220 * 1024;
    // the dynamic shared-memory limit is a property of the kernel, not of a
    // launch: set it once to the largest size any line length may use, so
    // that solves of different lengths from several host threads cannot
    // lower it under each other's launches
    static const bool attr = [] {
        TDZ_CUDA(cudaFuncSetAttribute(k_zsolve2<P, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMax));
        TDZ_CUDA(cudaFuncSetAttribute(k_zsolve<P, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMax));
        return true;
    }();
    (void)attr;
    const int nl = zp.n0 * zp.n1;
    k_zbands<<<(zp.n2 * (2 * P + 1) + 255) / 256, 256, 0, st>>>(zp, 2 * P + 1);
    if (zp.n2 >= 4 * ZBlk2<P>::B) {
        const size_t smem = zsolve2_smem<P>(zp.n2);
        TDZ_CHECK(smem <= kMax, TDZ_ERR_UNSUPPORTED, "outer axis too long for the FDM line solve");
        k_zsolve2<P, CI><<<(nl + kZ2Lines - 1) / kZ2Lines, 2 * kZ2Lines, smem, st>>>(zp);
        return;
    }
    const size_t smem = zsolve_smem<P>(zp.n2);
    TDZ_CHECK(smem <= kMax, TDZ_ERR_UNSUPPORTED, "outer axis too long for the FDM line solve");
    k_zsolve<P, CI><<<(nl + kZThreads - 1) / kZThreads, kZThreads, smem, st>>>(zp);
}

// complex eigenvalues (complex axis pencils) take the variant with the
// imaginary part of the line shift
template <int P> void launch_zsolve(const ZSolveParams &zp, cudaStream_t st) {
    if (zp.lxi) launch_zsolve_t<P, true>(zp, st);
    else launch_zsolve_t<P, false>(zp, st);
}

// saved-state scratch of the line solves (float2 entries): the larger of the
// one-thread and the two-thread layouts
size_t zsolve_state_size(int P, int n2, size_t lines) {
    auto sz = [&](int B, int NS, int B2) {
        const int m = zsolve2_twist(n2, B2);
        const size_t one = (size_t)((n2 + B - 1) / B) * NS * lines;
        const size_t two = (size_t)((m + B2 - 1) / B2 + (n2 - m + B2 - 1) / B2) * NS * lines;
        return std::max(one, two);
    };
    switch (P) {
    case 2: return sz(ZBlk<2>::B, ZBlk<2>::NS, ZBlk2<2>::B);
    case 3: return sz(ZBlk<3>::B, ZBlk<3>::NS, ZBlk2<3>::B);
    case 4: return sz(ZBlk<4>::B, ZBlk<4>::NS, ZBlk2<4>::B);
    default: return sz(ZBlk<5>::B, ZBlk<5>::NS, ZBlk2<5>::B);
    }
}

}  // namespace

void PcFDM::setup(Operator *op_, int prec) {
    op = op_;
    TDZ_CHECK(prec == TDZ_FP32 || prec == TDZ_FP64, TDZ_ERR_ARG, "FDM precision must be FP32 or FP64");
    f64 = prec == TDZ_FP64;
    const Space &s = *op->sp;
    dim = s.dim;
    TDZ_CHECK(dim >= 2, TDZ_ERR_UNSUPPORTED, "the FDM preconditioner needs 2D or 3D");
    P = s.ax[0].p;
    TDZ_CHECK(P >= 2 && P <= 5, TDZ_ERR_UNSUPPORTED, "the FDM preconditioner supports degrees 2..5");
    const Plan &pl = op->plan(TDZ_STAGE);
    // Inner-axis pencils. With only stiffness on the inner axes the
    // eigenvectors are those of (S_d, M_d) and the stage factor comes from
    // the stiffness terms (this also diagonalises stream C). Otherwise, with
    // no stream C, the pencil is S_d = sum_t f_t B_t over the inner one-axis
    // terms on the stiffness's stage scalar g (kinetic, potential and
    // absorbing layer of axis d), with stage factor g: complex symmetric when
    // the axis has an absorbing layer. Inner terms on other scalars (a field
    // along an inner axis) are left out of the fast inverse.
    exact = true;
    pencil = 0;
    cplx = false;
    dropped.clear();
    auto pure_s = [&](const Comb &c) {
        for (int i = 0; i < c.n; ++i)
            if (c.base[i] != kS) return false;
        return true;
    };
    const Comb *inner[2] = {&pl.xT, &pl.yT};
    if (pl.hasB && (!pure_s(pl.xT) || (dim == 3 && !pure_s(pl.yT)))) {
        if (pl.hasC) {
            exact = false;
        } else {
            pencil = 1;
            pencil_scalar = -1;
            for (int t = 0; t < pl.xT.n; ++t)
                if (pl.xT.base[t] == kS) pencil_scalar = pl.xT.scalar[t];
            TDZ_CHECK(pencil_scalar >= 0, TDZ_ERR_INTERNAL, "inner axis without a stiffness term");
            for (int d = 0; d < dim - 1; ++d)
                for (int t = 0; t < inner[d]->n; ++t)
                    if (inner[d]->scalar[t] != pencil_scalar) {
                        exact = false;
                        dropped.push_back(inner[d]->scalar[t]);
                    }
        }
    }
    if (op->quad.on) exact = false;   // the non-separable term is left out of the fast inverse
    for (int d = 0; d < 3; ++d) n[d] = d < dim ? s.ax[d].n : 1;
    N = (size_t)s.ndof();
    // axis pencils: real (S_d, M_d) eigenvectors, or complex ones
    std::vector<double> Vr[2], lr[2];
    std::vector<cd> Vc[2], lc[2];
    bool is_c[2] = {false, false};
    for (int d = 0; d < dim - 1; ++d) {
        if (pencil == 0) {
            gen_eig(op->bases[d][kS], op->bases[d][kM], Vr[d], lr[d]);
            continue;
        }
        const int bw = 2 * P + 1;
        std::vector<cd> band((size_t)n[d] * bw, cd(0.0));
        for (int t = 0; t < inner[d]->n; ++t) {
            if (inner[d]->scalar[t] != pencil_scalar) continue;
            const BandD &B = op->bases[d][inner[d]->base[t]];
            for (size_t e = 0; e < band.size(); ++e) band[e] += inner[d]->factor[t] * B.v[e];
        }
        bool imag = false;
        for (const cd &v : band) imag = imag || v.imag() != 0.0;
        if (!imag) {
            BandD re(n[d], P);
            for (size_t e = 0; e < band.size(); ++e) re.v[e] = band[e].real();
            gen_eig(re, op->bases[d][kM], Vr[d], lr[d]);
        } else if (gen_eig_complex(band, P, op->bases[d][kM], Vc[d], lc[d])) {
            is_c[d] = true;
        } else {
            // no complex-orthogonal eigenbasis: fall back to the stiffness pencil
            pencil = 0;
            exact = false;
            dropped.clear();
            for (int e = 0; e < dim - 1; ++e) {
                is_c[e] = false;
                gen_eig(op->bases[e][kS], op->bases[e][kM], Vr[e], lr[e]);
            }
            break;
        }
    }
    cplx = is_c[0] || is_c[1];
    tensor = !f64 && !cplx && dim == 3 && transform_supported(n[0]) && transform_supported(n[1]);
    // transform matrices and eigenvalues in the preconditioner's precision
    auto up = [&](DevBuf &b, const std::vector<double> &v) {
        if (f64) upload(b, v);
        else upload(b, std::vector<float>(v.begin(), v.end()));
    };
    auto upc = [&](DevBuf &b, const std::vector<cd> &v) {
        if (f64) {
            std::vector<double2> h(v.size());
            for (size_t e = 0; e < v.size(); ++e) h[e] = make_double2(v[e].real(), v[e].imag());
            upload(b, h);
        } else {
            std::vector<float2> h(v.size());
            for (size_t e = 0; e < v.size(); ++e) h[e] = make_float2((float)v[e].real(), (float)v[e].imag());
            upload(b, h);
        }
    };
    for (int d = 0; d < dim - 1; ++d) {
        const int nd = n[d];
        if (cplx) {
            // complex transforms (SIMT): V and V^T complex, eigenvalues split into parts
            const std::vector<cd> vc = is_c[d] ? Vc[d] : std::vector<cd>(Vr[d].begin(), Vr[d].end());
            const std::vector<cd> l = is_c[d] ? lc[d] : std::vector<cd>(lr[d].begin(), lr[d].end());
            std::vector<cd> vt((size_t)nd * nd);
            for (int i = 0; i < nd; ++i)
                for (int j = 0; j < nd; ++j) vt[(size_t)j * nd + i] = vc[(size_t)i * nd + j];
            std::vector<double> lre(nd), lim(nd);
            for (int i = 0; i < nd; ++i) { lre[i] = l[i].real(); lim[i] = l[i].imag(); }
            upc(V[d], vc);
            upc(VT[d], vt);
            up(lam[d], lre);
            up(lami[d], lim);
            continue;
        }
        const std::vector<double> &Vd = Vr[d], &ld = lr[d];
        std::vector<double> VTd((size_t)nd * nd);
        for (int i = 0; i < nd; ++i)
            for (int j = 0; j < nd; ++j) VTd[(size_t)j * nd + i] = Vd[(size_t)i * nd + j];
        up(lam[d], ld);
        if (tensor) {
            // 3D: eigenvector transforms on the tensor cores (forward with V, inverse with V^T)
            Tf[d].build(Vd, nd, nd);
            Ti[d].build(VTd, nd, nd);
        } else {
            up(V[d], Vd);
            up(VT[d], VTd);
        }
    }
    if (f64) {
        ufac.alloc(N * (3 * P + 1) * sizeof(double2));
        piv64.alloc(N * sizeof(int));
        b1.alloc(N * sizeof(double2));
        b2.alloc(N * sizeof(double2));
        return;
    }
    ufac.alloc(zsolve_state_size(P, n[dim - 1], N / n[dim - 1]) * sizeof(float2));
    zb.alloc((size_t)2 * n[dim - 1] * (2 * P + 1) * sizeof(float2));
    if (tensor) {
        npart.alloc((size_t)16 * sm_count() * sizeof(double));
        ldx = (n[0] + 3) / 4 * 4;
        ldy = (n[1] + 3) / 4 * 4;
        pa.alloc((size_t)n[2] * n[1] * 2 * ldx * sizeof(float));
        pb.alloc((size_t)n[2] * n[0] * 2 * ldy * sizeof(float));
    } else {
        b1.alloc(N * sizeof(float2));
        b2.alloc(N * sizeof(float2));
    }
}

bool PcFDM::exact_now() const {
    if (op->quad.on) return false;
    if (pencil == 0) return exact;
    for (int sc : dropped)
        if (op->sigma[sc] != cd(0.0)) return false;
    return true;
}

namespace {

// line solve parameters of the current stage (bands and eigenvalues; the
// caller sets the data layout)
// stage coefficients of the line matrices A_z(s) = Bc + s Cc of the current
// (or pole) stage, as CombP of the precision T
template <class T> void line_combs(const PcFDM &f, CombP<T> &Bc, CombP<T> &Cc) {
    const Operator *op = f.op;
    const Plan &pl = const_cast<Operator *>(op)->plan(TDZ_STAGE);
    const std::array<cd, 5> &sg = f.pole ? f.pole_sigma : op->sigma;
    auto eval = [&](const Comb &c) {
        CombP<T> out{};
        out.n = c.n;
        for (int i = 0; i < c.n; ++i) {
            const cd v = c.factor[i] * sg[c.scalar[i]];
            out.base[i] = c.base[i];
            out.re[i] = (T)v.real();
            out.im[i] = (T)v.imag();
        }
        return out;
    };
    Bc = eval(pl.zA);
    Comb cc = pl.zC;
    if (f.pencil == 1) {
        // stream B in the eigenbasis: g (lam_x + lam_y) M_out (no stream C)
        Comb gm;
        gm.add(kM, f.pencil_scalar, 1.0);
        Cc = eval(gm);
    } else if (pl.hasB && pl.xT.n > 0) {
        // stream B: M_out (x) (M_y (x) beta S_x + beta S_y (x) M_x) -> beta M_out
        cd beta = 0.0;
        for (int t = 0; t < pl.xT.n; ++t)
            if (pl.xT.base[t] == kS) beta += pl.xT.factor[t] * sg[pl.xT.scalar[t]];
        cc.add(kM, 0, 0.0);
        CombP<T> c = eval(cc);
        for (int t = 0; t < c.n; ++t)
            if (c.base[t] == kM) { c.re[t] += (T)beta.real(); c.im[t] += (T)beta.imag(); }
        Cc = c;
    } else {
        Cc = eval(cc);
    }
}

ZSolveParams line_params(const PcFDM &f) {
    const Operator *op = f.op;
    const int dim = f.dim;
    const int *n = f.n;
    const int outer = dim - 1;
    ZSolveParams zp{};
    zp.ck = f.ufac.as<float2>();
    zp.zb = f.zb.as<float2>();
    zp.bands = op->dev32[outer].as<float>();
    zp.lx = f.lam[0].as<float>();
    zp.ly = dim == 3 ? f.lam[1].as<float>() : nullptr;
    if (f.cplx) {
        zp.lxi = f.lami[0].as<float>();
        zp.lyi = dim == 3 ? f.lami[1].as<float>() : nullptr;
    }
    zp.n0 = n[0];
    zp.n1 = dim == 3 ? n[1] : 1;
    zp.n2 = n[outer];
    line_combs<float>(f, zp.Bc, zp.Cc);
    return zp;
}

// FP64 line solves (the FP64 preconditioner): one thread per line, banded LU
// with partial pivoting (the lines of the end term's indefinite stages need
// it), the line matrix evaluated from the FP64 bands into a global scratch
// whose row r holds columns r - P .. r + 2P, lines interleaved (coalesced)
struct Line64Params {
    double2 *x;               // line (i, j), row k at x[k ks + j js + i]
    size_t ks;
    int js;
    int n0, n1, n2;
    const double *bands;      // outer base bands [nb][n2][2P+1] (FP64)
    const double *lx, *ly, *lxi, *lyi;
    CombP<double> Bc, Cc;
    double2 *U;               // [n2][3P + 1][lines]: the line's LU factors
    int *piv;                 // [n2][lines]: row interchanged with row k at step k
};

template <int P> __global__ void __launch_bounds__(128) k_line64(const Line64Params prm) {
    constexpr int BW = 2 * P + 1, W = 3 * P + 1;
    const int nl = prm.n0 * prm.n1;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    const int i = l % prm.n0, j = l / prm.n0;
    const double sr = prm.lx[i] + (prm.ly ? prm.ly[j] : 0.0);
    const double si = (prm.lxi ? prm.lxi[i] : 0.0) + (prm.lyi ? prm.lyi[j] : 0.0);
    double2 *xl = prm.x + (size_t)j * prm.js + i;
    const int n = prm.n2;
    const size_t ks = prm.ks;
    // entry (r, c) of the line matrix, |c - r| within the widened band
    auto A = [&](int r, int c) -> double2 & { return prm.U[((size_t)r * W + (c - r + P)) * nl + l]; };
    auto cm = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    for (int r = 0; r < n; ++r)
        for (int o = 0; o < W; ++o) {
            double2 v = make_double2(0.0, 0.0);
            if (o < BW) {
                const double2 b = comb_at<double, double2>(prm.Bc, prm.bands, n, BW, r, o);
                const double2 c = comb_at<double, double2>(prm.Cc, prm.bands, n, BW, r, o);
                v = make_double2(b.x + sr * c.x - si * c.y, b.y + sr * c.y + si * c.x);
            }
            prm.U[((size_t)r * W + o) * nl + l] = v;
        }
    for (int k = 0; k < n; ++k) {
        const int rmax = min(k + P, n - 1), cmax = min(k + 2 * P, n - 1);
        int bi = k;
        double best = fabs(A(k, k).x) + fabs(A(k, k).y);
        for (int r = k + 1; r <= rmax; ++r) {
            const double m = fabs(A(r, k).x) + fabs(A(r, k).y);
            if (m > best) { best = m; bi = r; }
        }
        prm.piv[(size_t)k * nl + l] = bi;
        if (!(best > 0.0)) continue;   // singular column: the solve returns non-finite values
        if (bi != k)
            for (int c = k; c <= cmax; ++c) {
                const double2 t = A(k, c);
                A(k, c) = A(bi, c);
                A(bi, c) = t;
            }
        const double2 d = A(k, k);
        const double dd = 1.0 / (d.x * d.x + d.y * d.y);
        const double2 inv = make_double2(d.x * dd, -d.y * dd);
        for (int r = k + 1; r <= rmax; ++r) {
            const double2 f = cm(A(r, k), inv);
            A(r, k) = f;
            for (int c = k + 1; c <= cmax; ++c) {
                const double2 u = cm(f, A(k, c));
                double2 &t = A(r, c);
                t.x -= u.x;
                t.y -= u.y;
            }
        }
    }
    for (int k = 0; k < n; ++k) {
        const int q = prm.piv[(size_t)k * nl + l];
        if (q != k) {
            const double2 t = xl[(size_t)k * ks];
            xl[(size_t)k * ks] = xl[(size_t)q * ks];
            xl[(size_t)q * ks] = t;
        }
        const double2 xk = xl[(size_t)k * ks];
        for (int r = k + 1; r <= min(k + P, n - 1); ++r) {
            const double2 u = cm(A(r, k), xk);
            xl[(size_t)r * ks].x -= u.x;
            xl[(size_t)r * ks].y -= u.y;
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        double2 v = xl[(size_t)k * ks];
        for (int c = k + 1; c <= min(k + 2 * P, n - 1); ++c) {
            const double2 u = cm(A(k, c), xl[(size_t)c * ks]);
            v.x -= u.x;
            v.y -= u.y;
        }
        const double2 d = A(k, k);
        const double dd = 1.0 / (d.x * d.x + d.y * d.y);
        xl[(size_t)k * ks] = make_double2((v.x * d.x + v.y * d.y) * dd, (v.y * d.x - v.x * d.y) * dd);
    }
}

void line_solve64(const PcFDM &f, double2 *x, cudaStream_t st) {
    const int dim = f.dim, outer = dim - 1;
    Line64Params lp{};
    lp.x = x;
    lp.n0 = f.n[0];
    lp.n1 = dim == 3 ? f.n[1] : 1;
    lp.n2 = f.n[outer];
    lp.ks = (size_t)lp.n0 * lp.n1;
    lp.js = lp.n0;
    lp.bands = f.op->dev64[outer].as<double>();
    lp.lx = f.lam[0].as<double>();
    lp.ly = dim == 3 ? f.lam[1].as<double>() : nullptr;
    if (f.cplx) {
        lp.lxi = f.lami[0].as<double>();
        lp.lyi = dim == 3 ? f.lami[1].as<double>() : nullptr;
    }
    line_combs<double>(f, lp.Bc, lp.Cc);
    lp.U = f.ufac.as<double2>();
    lp.piv = f.piv64.as<int>();
    const int nl = lp.n0 * lp.n1, blocks = (nl + 127) / 128;
    switch (f.P) {
    case 2: k_line64<2><<<blocks, 128, 0, st>>>(lp); break;
    case 3: k_line64<3><<<blocks, 128, 0, st>>>(lp); break;
    case 4: k_line64<4><<<blocks, 128, 0, st>>>(lp); break;
    case 5: k_line64<5><<<blocks, 128, 0, st>>>(lp); break;
    }
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void line_solve(int P, const ZSolveParams &zp, cudaStream_t st) {
    switch (P) {
    case 2: launch_zsolve<2>(zp, st); break;
    case 3: launch_zsolve<3>(zp, st); break;
    case 4: launch_zsolve<4>(zp, st); break;
    case 5: launch_zsolve<5>(zp, st); break;
    }
    TDZ_CUDA(cudaGetLastError());
    count_launch(2);
}

}  // namespace

void PcFDM::apply_norm(const double2 *r, double2 *z, double *norm2, cudaStream_t st) {
    TDZ_CHECK(tensor, TDZ_ERR_INTERNAL, "fused norm only on the tensor-core path");
    norm_out = norm2;
    apply(r, z, st);
    norm_out = nullptr;
}

void PcFDM::apply(const double2 *r, double2 *z, cudaStream_t st) {
    const size_t rows = (size_t)n[1] * n[2];
    if (tensor) {
        // [z][y][c][x] -> [z][x'][c][y] -> [z][y'][c][x'] -> line solves -> [z][x][c][y'] -> [z][y][c][x]
        float *a = pa.as<float>(), *b = pb.as<float>();
        const int blocks = (int)std::min<size_t>((N + 255) / 256, (size_t)16 * sm_count());
        k_to_planar<<<blocks, 256, 0, st>>>(r, a, n[0], rows, ldx);
        transform(Tf[0], a, n[2], n[1], ldx, b, ldy, st);
        transform(Tf[1], b, n[2], n[0], ldy, a, ldx, st);
        ZSolveParams zp = line_params(*this);
        zp.x = a;
        zp.ks = (size_t)2 * n[1] * ldx;
        zp.js = 2 * ldx;
        zp.is = 1;
        zp.cs = ldx;
        line_solve(P, zp, st);
        transform(Ti[0], a, n[2], n[1], ldx, b, ldy, st);
        transform(Ti[1], b, n[2], n[0], ldy, a, ldx, st);
        if (norm_out) {
            k_from_planar_norm<<<blocks, 256, 0, st>>>(a, z, n[0], rows, ldx, npart.as<double>());
            k_sum_parts<<<1, 256, 0, st>>>(npart.as<double>(), blocks, norm_out);
            count_launch();
        } else {
            k_from_planar<<<blocks, 256, 0, st>>>(a, z, n[0], rows, ldx);
        }
        TDZ_CUDA(cudaGetLastError());
        count_launch(2);
        ++applies;
        return;
    }
    const int grows = (int)rows;
    if (f64) {
        // FP64 preconditioner (SIMT transforms, FP64 line solves)
        double2 *y1 = b1.as<double2>(), *y2 = b2.as<double2>();
        auto x64 = [&](const DevBuf &Mx, const double2 *in, double2 *out) {
            const dim3 g((n[0] + BN - 1) / BN, (grows + BM - 1) / BM);
            if (cplx) k_gemm_cr<double2, double2><<<g, 256, 0, st>>>(in, Mx.as<double2>(), out, grows, n[0], n[0]);
            else k_gemm_cr<double2, double><<<g, 256, 0, st>>>(in, Mx.as<double>(), out, grows, n[0], n[0]);
        };
        auto y64 = [&](const DevBuf &My, const double2 *in, double2 *out) {
            const dim3 g((n[0] + BN - 1) / BN, (n[1] + BM - 1) / BM, n[2]);
            if (cplx) k_gemm_rc<double2, double2><<<g, 256, 0, st>>>(My.as<double2>(), in, out, n[1], n[0], n[1]);
            else k_gemm_rc<double2, double><<<g, 256, 0, st>>>(My.as<double>(), in, out, n[1], n[0], n[1]);
        };
        x64(V[0], r, y2);
        double2 *cur = y2, *oth = y1;
        if (dim == 3) {
            y64(VT[1], y2, y1);
            std::swap(cur, oth);
        }
        TDZ_CUDA(cudaGetLastError());
        line_solve64(*this, cur, st);
        if (dim == 3) {
            y64(V[1], cur, oth);
            std::swap(cur, oth);
        }
        x64(VT[0], cur, z);
        TDZ_CUDA(cudaGetLastError());
        count_launch(dim == 3 ? 4 : 2);
        ++applies;
        return;
    }
    float2 *x1 = b1.as<float2>(), *x2 = b2.as<float2>();
    blas::cast(r, TDZ_FP64, x1, TDZ_FP32, N, st);
    // transforms along x (rows of n0) and along y (planes of n1 x n0) with a
    // real or complex FP32 matrix
    auto along_x = [&](const DevBuf &Mx, const float2 *in, float2 *out) {
        const dim3 g((n[0] + BN - 1) / BN, (grows + BM - 1) / BM);
        if (cplx) k_gemm_cr<float2, float2><<<g, 256, 0, st>>>(in, Mx.as<float2>(), out, grows, n[0], n[0]);
        else k_gemm_cr<float2, float><<<g, 256, 0, st>>>(in, Mx.as<float>(), out, grows, n[0], n[0]);
    };
    auto along_y = [&](const DevBuf &My, const float2 *in, float2 *out) {
        const dim3 g((n[0] + BN - 1) / BN, (n[1] + BM - 1) / BM, n[2]);
        if (cplx) k_gemm_rc<float2, float2><<<g, 256, 0, st>>>(My.as<float2>(), in, out, n[1], n[0], n[1]);
        else k_gemm_rc<float2, float><<<g, 256, 0, st>>>(My.as<float>(), in, out, n[1], n[0], n[1]);
    };
    // forward transforms: along x with V (t_i = sum_i' V[i'][i] r_i'), along y with V^T
    along_x(V[0], x1, x2);
    float2 *cur = x2, *oth = x1;
    if (dim == 3) {
        along_y(VT[1], x2, x1);
        cur = x1;
        oth = x2;
    }
    TDZ_CUDA(cudaGetLastError());
    // line solves along the outer axis: A_z(s) = zA + s (beta M + zC), interleaved complex
    ZSolveParams zp = line_params(*this);
    zp.x = reinterpret_cast<float *>(cur);
    zp.ks = (size_t)2 * n[0] * (dim == 3 ? n[1] : 1);
    zp.js = 2 * n[0];
    zp.is = 2;
    zp.cs = 1;
    line_solve(P, zp, st);
    // inverse transforms: along y with V, along x with V^T
    if (dim == 3) {
        along_y(V[1], cur, oth);
        std::swap(cur, oth);
    }
    along_x(VT[0], cur, oth);
    TDZ_CUDA(cudaGetLastError());
    count_launch(dim == 3 ? 4 : 2);
    blas::cast(oth, TDZ_FP32, z, TDZ_FP64, N, st);
    ++applies;
}

}  // namespace tdz
