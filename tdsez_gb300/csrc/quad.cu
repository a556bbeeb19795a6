// Non-separable soft-core potential term by per-element quadrature (quad.h).
// One CTA per element: gather the (p+1)^d coefficients, interpolate to the
// Q^d Gauss points axis by axis (sum factorisation, shared memory ping-pong),
// multiply by w V with V from the closed form, project back axis by axis and
// add coef * result to y with atomics (neighbouring elements share
// coefficients). Work per element 2 d Q (p+1)^d (d-dimensional sum
// factorisation): the per-element tensor-contraction flops of this term.
#include "quad.h"

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "cplx.cuh"

namespace tdz {

namespace {

constexpr int kMaxQ = 10;      // Gauss points per element and axis
constexpr int kQThreads = 64;

template <class T> struct QuadParams {
    const void *x;
    void *y;
    int n[3], nel[3], nq;
    const int *off[3];
    const T *N[3], *w[3], *xq[3];
    int nsoft;
    T soft[kMaxSoft][5];
    T cre, cim;
    double cre_d, cim_d;
};

__device__ __forceinline__ void atomic_add_c(float2 *p, float2 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void atomic_add_c(double2 *p, double2 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}

template <class T> __device__ __forceinline__ T rsqrt_t(T v);
template <> __device__ __forceinline__ float rsqrt_t<float>(float v) { return rsqrtf(v); }
template <> __device__ __forceinline__ double rsqrt_t<double>(double v) { return 1.0 / sqrt(v); }

template <class T, int P, int DIM>
__global__ void __launch_bounds__(kQThreads) k_quad(const QuadParams<T> prm) {
    using C = typename CT<T>::type;
    constexpr int NP = P + 1;
    constexpr int M = NP > kMaxQ ? NP : kMaxQ;
    constexpr int CAP = DIM == 3 ? M * M * M : M * M;
    __shared__ C bufA[CAP], bufB[CAP];
    __shared__ T sN[3][kMaxQ * NP], sW[3][kMaxQ], sX[3][kMaxQ];
    const int Q = prm.nq, tid = threadIdx.x;
    int e = blockIdx.x;
    int el[3] = {0, 0, 0};
    for (int d = 0; d < DIM; ++d) { el[d] = e % prm.nel[d]; e /= prm.nel[d]; }
    int o[3] = {0, 0, 0};
    for (int d = 0; d < DIM; ++d) o[d] = prm.off[d][el[d]];
    for (int d = 0; d < DIM; ++d)
        for (int i = tid; i < Q * NP; i += kQThreads) sN[d][i] = prm.N[d][(size_t)el[d] * Q * NP + i];
    for (int d = 0; d < DIM; ++d)
        for (int i = tid; i < Q; i += kQThreads) {
            sW[d][i] = prm.w[d][(size_t)el[d] * Q + i];
            sX[d][i] = prm.xq[d][(size_t)el[d] * Q + i];
        }
    const C *X = static_cast<const C *>(prm.x);
    C *Y = static_cast<C *>(prm.y);
    // extents of the local tensor [z][y][x] during the passes
    if constexpr (DIM == 3) {
        for (int i = tid; i < NP * NP * NP; i += kQThreads) {
            const int kx = i % NP, ky = (i / NP) % NP, kz = i / (NP * NP);
            bufA[i] = X[((size_t)(o[2] + kz) * prm.n[1] + (o[1] + ky)) * prm.n[0] + o[0] + kx];
        }
        __syncthreads();
        // x: A[kz][ky][kx] -> B[kz][ky][qx]
        for (int i = tid; i < NP * NP * Q; i += kQThreads) {
            const int qx = i % Q, r = i / Q;
            C acc = czero<C>();
            for (int k = 0; k < NP; ++k) rfma(acc, sN[0][qx * NP + k], bufA[r * NP + k]);
            bufB[i] = acc;
        }
        __syncthreads();
        // y: B[kz][ky][qx] -> A[kz][qy][qx]
        for (int i = tid; i < NP * Q * Q; i += kQThreads) {
            const int qx = i % Q, qy = (i / Q) % Q, kz = i / (Q * Q);
            C acc = czero<C>();
            for (int k = 0; k < NP; ++k) rfma(acc, sN[1][qy * NP + k], bufB[(kz * NP + k) * Q + qx]);
            bufA[i] = acc;
        }
        __syncthreads();
        // z: A[kz][qy][qx] -> B[qz][qy][qx], times w V
        for (int i = tid; i < Q * Q * Q; i += kQThreads) {
            const int qx = i % Q, qy = (i / Q) % Q, qz = i / (Q * Q);
            C acc = czero<C>();
            for (int k = 0; k < NP; ++k) rfma(acc, sN[2][qz * NP + k], bufA[(k * Q + qy) * Q + qx]);
            T v = T(0);
            for (int c = 0; c < prm.nsoft; ++c) {
                const T dx = sX[0][qx] - prm.soft[c][1], dy = sX[1][qy] - prm.soft[c][2], dz = sX[2][qz] - prm.soft[c][3];
                v -= prm.soft[c][0] * rsqrt_t<T>(dx * dx + dy * dy + dz * dz + prm.soft[c][4]);
            }
            const T f = sW[0][qx] * sW[1][qy] * sW[2][qz] * v;
            acc.x *= f;
            acc.y *= f;
            bufB[i] = acc;
        }
        __syncthreads();
        // back z: B[qz][qy][qx] -> A[kz][qy][qx]
        for (int i = tid; i < NP * Q * Q; i += kQThreads) {
            const int qx = i % Q, qy = (i / Q) % Q, kz = i / (Q * Q);
            C acc = czero<C>();
            for (int q = 0; q < Q; ++q) rfma(acc, sN[2][q * NP + kz], bufB[(q * Q + qy) * Q + qx]);
            bufA[i] = acc;
        }
        __syncthreads();
        // back y: A[kz][qy][qx] -> B[kz][ky][qx]
        for (int i = tid; i < NP * NP * Q; i += kQThreads) {
            const int qx = i % Q, ky = (i / Q) % NP, kz = i / (Q * NP);
            C acc = czero<C>();
            for (int q = 0; q < Q; ++q) rfma(acc, sN[1][q * NP + ky], bufA[(kz * Q + q) * Q + qx]);
            bufB[i] = acc;
        }
        __syncthreads();
        // back x and scatter: B[kz][ky][qx] -> y
        for (int i = tid; i < NP * NP * NP; i += kQThreads) {
            const int kx = i % NP, r = i / NP, ky = r % NP, kz = r / NP;
            C acc = czero<C>();
            for (int q = 0; q < Q; ++q) rfma(acc, sN[0][q * NP + kx], bufB[r * Q + q]);
            C out;
            out.x = prm.cre * acc.x - prm.cim * acc.y;
            out.y = prm.cre * acc.y + prm.cim * acc.x;
            atomic_add_c(&Y[((size_t)(o[2] + kz) * prm.n[1] + (o[1] + ky)) * prm.n[0] + o[0] + kx], out);
        }
    } else {
        for (int i = tid; i < NP * NP; i += kQThreads) {
            const int kx = i % NP, ky = i / NP;
            bufA[i] = X[(size_t)(o[1] + ky) * prm.n[0] + o[0] + kx];
        }
        __syncthreads();
        // x: A[ky][kx] -> B[ky][qx]
        for (int i = tid; i < NP * Q; i += kQThreads) {
            const int qx = i % Q, ky = i / Q;
            C acc = czero<C>();
            for (int k = 0; k < NP; ++k) rfma(acc, sN[0][qx * NP + k], bufA[ky * NP + k]);
            bufB[i] = acc;
        }
        __syncthreads();
        // y: B[ky][qx] -> A[qy][qx], times w V
        for (int i = tid; i < Q * Q; i += kQThreads) {
            const int qx = i % Q, qy = i / Q;
            C acc = czero<C>();
            for (int k = 0; k < NP; ++k) rfma(acc, sN[1][qy * NP + k], bufB[k * Q + qx]);
            T v = T(0);
            for (int c = 0; c < prm.nsoft; ++c) {
                const T dx = sX[0][qx] - prm.soft[c][1], dy = sX[1][qy] - prm.soft[c][2];
                v -= prm.soft[c][0] * rsqrt_t<T>(dx * dx + dy * dy + prm.soft[c][4]);
            }
            const T f = sW[0][qx] * sW[1][qy] * v;
            acc.x *= f;
            acc.y *= f;
            bufA[i] = acc;
        }
        __syncthreads();
        // back y: A[qy][qx] -> B[ky][qx]
        for (int i = tid; i < NP * Q; i += kQThreads) {
            const int qx = i % Q, ky = i / Q;
            C acc = czero<C>();
            for (int q = 0; q < Q; ++q) rfma(acc, sN[1][q * NP + ky], bufA[q * Q + qx]);
            bufB[i] = acc;
        }
        __syncthreads();
        // back x and scatter
        for (int i = tid; i < NP * NP; i += kQThreads) {
            const int kx = i % NP, ky = i / NP;
            C acc = czero<C>();
            for (int q = 0; q < Q; ++q) rfma(acc, sN[0][q * NP + kx], bufB[ky * Q + q]);
            C out;
            out.x = prm.cre * acc.x - prm.cim * acc.y;
            out.y = prm.cre * acc.y + prm.cim * acc.x;
            atomic_add_c(&Y[(size_t)(o[1] + ky) * prm.n[0] + o[0] + kx], out);
        }
    }
}

// ---------------------------------------------------------------- streaming 3D kernel
// For axes whose elements own consecutive coefficient windows (no repeated
// knots) and Q = p + 1 Gauss points. A CTA owns TE x TE elements in (x, y)
// and streams a chunk of their z column. Interpolation of a coefficient plane
// to the tile's (TE Q)^2 quadrature points (x, then y) is done once per
// plane and kept in a ring of p + 1 planes; per z element every quadrature
// column is interpolated along z, multiplied by w V (V from the closed form)
// and projected back along z into a ring of p + 1 accumulator planes; a
// coefficient plane whose elements are all done is projected back along y
// and x and added to y with one atomic per coefficient and tile (the tiles
// overlap by p coefficients per axis, chunk ends by p planes). Versus one CTA
// per element: each interpolated plane serves p + 1 elements and the
// coefficients receive (1 + p/TE)^2 atomic adds instead of (p+1)^3.
// FP32 arithmetic on FP32 vectors, or double-float arithmetic on FP64
// vectors (the FGMRES applies: 1/sqrt of the potential by rsqrtf and one
// Newton step in double-float, about 48 bits).
template <class A> struct QArith;
template <> struct QArith<float> {
    using C = float2;
    using MC = float2;
    using TT = float;
    __device__ static float from(TT v) { return v; }
    __device__ static float one() { return 1.f; }
    // -Z / sqrt(r2 + a) summed over the centres at (x, y, z)
    __device__ static float pot(const QuadParams<TT> &prm, float x, float y, float z) {
        float v = 0.f;
        for (int k = 0; k < prm.nsoft; ++k) {
            const float dx = x - prm.soft[k][1], dy = y - prm.soft[k][2], dz = z - prm.soft[k][3];
            v -= prm.soft[k][0] * rsqrtf(dx * dx + dy * dy + dz * dz + prm.soft[k][4]);
        }
        return v;
    }
    __device__ static float mul(float a, float b) { return a * b; }
    __device__ static void scale(float2 &f, float w) { f.x *= w; f.y *= w; }
    __device__ static void atomic_out(float2 *dst, float2 a, double cre, double cim) {
        atomicAdd(&dst->x, (float)cre * a.x - (float)cim * a.y);
        atomicAdd(&dst->y, (float)cre * a.y + (float)cim * a.x);
    }
};
template <> struct QArith<dff> {
    using C = cdff;
    using MC = double2;
    using TT = double;
    __device__ static dff from(TT v) { return dff_split(v); }
    __device__ static dff one() { return dff(1.f); }
    __device__ static dff mul(dff a, dff b) { return renorm(tfma(a, b, dff(0.f))); }
    __device__ static dff pot(const QuadParams<TT> &prm, dff x, dff y, dff z) {
        dff v(0.f);
        for (int k = 0; k < prm.nsoft; ++k) {
            const dff dx = renorm(tfma(dff(1.f), x, dff_split(-prm.soft[k][1])));
            const dff dy = renorm(tfma(dff(1.f), y, dff_split(-prm.soft[k][2])));
            const dff dz = renorm(tfma(dff(1.f), z, dff_split(-prm.soft[k][3])));
            const dff r2 = renorm(tfma(dx, dx, tfma(dy, dy, tfma(dz, dz, dff_split(prm.soft[k][4])))));
            // 1/sqrt(r2): rsqrtf, then one Newton step y1 = y0 - y0 (r2 y0^2 - 1) / 2 in double-float
            const float y0 = rsqrtf(r2.hi);
            const dff t = renorm(tfma(dff(y0), dff(y0), dff(0.f)));            // y0^2, exact
            const dff u = renorm(tfma(r2, t, dff(-1.f)));                       // r2 y0^2 - 1
            const dff yi = renorm(tfma(dff(-0.5f * y0), u, dff(y0)));
            v = renorm(tfma(dff_split(-prm.soft[k][0]), yi, v));
        }
        return v;
    }
    __device__ static void scale(cdff &f, dff w) {
        f.x = renorm(tfma(f.x, w, dff(0.f)));
        f.y = renorm(tfma(f.y, w, dff(0.f)));
    }
    __device__ static void atomic_out(double2 *dst, cdff a, double cre, double cim) {
        const double ax = dff_to_double(a.x), ay = dff_to_double(a.y);
        atomicAdd(&dst->x, cre * ax - cim * ay);
        atomicAdd(&dst->y, cre * ay + cim * ax);
    }
};

template <class A, int P, int TE> struct QStream {
    using C = typename QArith<A>::C;
    static constexpr int NP = P + 1, Q = P + 1, TQ = TE * Q, TC = TE + P, PL = TQ * TQ;
    static constexpr size_t smem = sizeof(C) * ((size_t)2 * NP * PL + TC * TC + TC * TQ);
};
constexpr int kQsThreads = 512;
// tile side in elements: the two rings of (TE (p+1))^2 points fit the 227 KB of shared memory
template <class A, int P> constexpr int qs_te() {
    return std::is_same<A, float>::value ? (P <= 4 ? 8 : 6) : (P <= 3 ? 7 : (P == 4 ? 6 : 4));
}

template <class A, int P, int TE>
__global__ void __launch_bounds__(kQsThreads) k_quad3_stream(const QuadParams<typename QArith<A>::TT> prm,
                                                             int zchunk) {
    using Q3 = QArith<A>;
    using C = typename Q3::C;
    using MC = typename Q3::MC;
    using S = QStream<A, P, TE>;
    constexpr int NP = S::NP, Q = S::Q, TQ = S::TQ, TC = S::TC, PL = S::PL;
    extern __shared__ __align__(16) unsigned char qs_raw[];
    C *sV = reinterpret_cast<C *>(qs_raw);   // [NP][PL] x,y-interpolated coefficient planes (ring, row qy, column qx)
    C *sG = sV + NP * PL;                    // [NP][PL] z-projected accumulators (ring)
    C *sX = sG + NP * PL;                    // [TC][TC] staged coefficient plane
    C *sU = sX + TC * TC;                    // [TC][TQ] x-interpolated rows, then the back-y rows
    __shared__ A sNx[TE * Q * NP], sNy[TE * Q * NP], sNz[Q * NP];
    __shared__ A sWx[TQ], sWy[TQ], sXx[TQ], sXy[TQ], sWz[Q], sXz[Q];
    const int tid = threadIdx.x;
    const int nelx = prm.nel[0], nely = prm.nel[1], nelz = prm.nel[2];
    const int tilesX = (nelx + TE - 1) / TE;
    const int ex0 = (blockIdx.x % tilesX) * TE, ey0 = (blockIdx.x / tilesX) * TE;
    const int ez0 = blockIdx.y * zchunk, ez1 = min(nelz, ez0 + zchunk);
    if (ez0 >= ez1) return;
    const int n0 = prm.n[0], n1 = prm.n[1], n2 = prm.n[2];
    const int cx0 = prm.off[0][ex0], cy0 = prm.off[1][ey0];
    const A zero = A(0.f);
    // per-tile tables (elements past the grid: zero rows, no contribution)
    for (int i = tid; i < TE * Q * NP; i += kQsThreads) {
        const int e = i / (Q * NP), r = i % (Q * NP);
        sNx[i] = ex0 + e < nelx ? Q3::from(prm.N[0][(size_t)(ex0 + e) * Q * NP + r]) : zero;
        sNy[i] = ey0 + e < nely ? Q3::from(prm.N[1][(size_t)(ey0 + e) * Q * NP + r]) : zero;
    }
    for (int i = tid; i < TQ; i += kQsThreads) {
        const int e = i / Q;
        const bool inx = ex0 + e < nelx, iny = ey0 + e < nely;
        sWx[i] = inx ? Q3::from(prm.w[0][(size_t)ex0 * Q + i]) : zero;
        sXx[i] = inx ? Q3::from(prm.xq[0][(size_t)ex0 * Q + i]) : zero;
        sWy[i] = iny ? Q3::from(prm.w[1][(size_t)ey0 * Q + i]) : zero;
        sXy[i] = iny ? Q3::from(prm.xq[1][(size_t)ey0 * Q + i]) : zero;
    }
    for (int i = tid; i < NP * PL; i += kQsThreads) sG[i] = czero<C>();
    const MC *X = static_cast<const MC *>(prm.x);
    MC *Y = static_cast<MC *>(prm.y);
    __syncthreads();

    // coefficient plane kz -> sV[kz % NP]
    auto interpolate_plane = [&](int kz) {
        for (int i = tid; i < TC * TC; i += kQsThreads) {
            const int iy = i / TC, ix = i % TC, gy = cy0 + iy, gx = cx0 + ix;
            sX[i] = (gy < n1 && gx < n0 && kz < n2) ? load_c<C, MC>(X[((size_t)kz * n1 + gy) * n0 + gx]) : czero<C>();
        }
        __syncthreads();
        for (int i = tid; i < TC * TQ; i += kQsThreads) {   // x: sU[iy][qx]
            const int iy = i / TQ, qx = i % TQ, e = qx / Q;
            const A *nx = sNx + qx * NP;
            C a = czero<C>();
#pragma unroll
            for (int c = 0; c < NP; ++c) rfma(a, nx[c], sX[iy * TC + e + c]);
            sU[i] = cnorm(a);
        }
        __syncthreads();
        C *v = sV + (size_t)(kz % NP) * PL;
        for (int i = tid; i < PL; i += kQsThreads) {        // y: v[qy][qx]
            const int qy = i / TQ, qx = i % TQ, e = qy / Q;
            const A *ny = sNy + qy * NP;
            C a = czero<C>();
#pragma unroll
            for (int c = 0; c < NP; ++c) rfma(a, ny[c], sU[(e + c) * TQ + qx]);
            v[i] = cnorm(a);
        }
        __syncthreads();
    };
    // complete coefficient plane kz in sG[kz % NP]: back along y and x, add to y, clear
    auto flush_plane = [&](int kz) {
        C *g = sG + (size_t)(kz % NP) * PL;
        for (int i = tid; i < TC * TQ; i += kQsThreads) {   // back y: sU[iy][qx]
            const int iy = i / TQ, qx = i % TQ;
            C a = czero<C>();
#pragma unroll
            for (int c = 0; c < NP; ++c) {
                const int e = iy - c;
                if (e < 0 || e >= TE) continue;
#pragma unroll
                for (int q = 0; q < Q; ++q) rfma(a, sNy[(e * Q + q) * NP + c], g[(e * Q + q) * TQ + qx]);
            }
            sU[i] = cnorm(a);
        }
        __syncthreads();
        for (int i = tid; i < TC * TC; i += kQsThreads) {   // back x, add to y
            const int iy = i / TC, ix = i % TC, gy = cy0 + iy, gx = cx0 + ix;
            C a = czero<C>();
#pragma unroll
            for (int c = 0; c < NP; ++c) {
                const int e = ix - c;
                if (e < 0 || e >= TE) continue;
#pragma unroll
                for (int q = 0; q < Q; ++q) rfma(a, sNx[(e * Q + q) * NP + c], sU[iy * TQ + e * Q + q]);
            }
            if (gy < n1 && gx < n0 && kz < n2)
                Q3::atomic_out(&Y[((size_t)kz * n1 + gy) * n0 + gx], cnorm(a), prm.cre_d, prm.cim_d);
        }
        for (int i = tid; i < PL; i += kQsThreads) g[i] = czero<C>();
        __syncthreads();
    };

    const int cz0 = prm.off[2][ez0];
    for (int c = 0; c < P; ++c) interpolate_plane(cz0 + c);
    for (int ez = ez0; ez < ez1; ++ez) {
        const int cz = prm.off[2][ez];
        interpolate_plane(cz + P);
        for (int i = tid; i < Q * NP; i += kQsThreads) sNz[i] = Q3::from(prm.N[2][(size_t)ez * Q * NP + i]);
        for (int i = tid; i < Q; i += kQsThreads) {
            sWz[i] = Q3::from(prm.w[2][(size_t)ez * Q + i]);
            sXz[i] = Q3::from(prm.xq[2][(size_t)ez * Q + i]);
        }
        __syncthreads();
        // z: interpolate, times w V, project back, per quadrature column
        for (int i = tid; i < PL; i += kQsThreads) {
            const int qy = i / TQ, qx = i % TQ;
            C v[NP], g[NP];
#pragma unroll
            for (int c = 0; c < NP; ++c) {
                v[c] = sV[(size_t)((cz + c) % NP) * PL + i];
                g[c] = czero<C>();
            }
            const A wxy = Q3::mul(sWx[qx], sWy[qy]);
#pragma unroll
            for (int qz = 0; qz < Q; ++qz) {
                C f = czero<C>();
#pragma unroll
                for (int c = 0; c < NP; ++c) rfma(f, sNz[qz * NP + c], v[c]);
                f = cnorm(f);
                const A wv = Q3::mul(Q3::mul(wxy, sWz[qz]), Q3::pot(prm, sXx[qx], sXy[qy], sXz[qz]));
                Q3::scale(f, wv);
#pragma unroll
                for (int c = 0; c < NP; ++c) rfma(g[c], sNz[qz * NP + c], f);
            }
#pragma unroll
            for (int c = 0; c < NP; ++c) {
                C &d = sG[(size_t)((cz + c) % NP) * PL + i];
                rfma(d, Q3::one(), cnorm(g[c]));
                d = cnorm(d);
            }
        }
        __syncthreads();
        flush_plane(cz);   // no later element of the chunk touches plane cz
    }
    // planes with contributions from the chunk's last elements
    const int czl = prm.off[2][ez1 - 1];
    for (int c = 1; c <= P; ++c) flush_plane(czl + c);
}

// the streaming kernel applies: 3D, Q = p + 1, consecutive element offsets on every axis
bool stream_ok(const QuadTerm &q) { return q.dim == 3 && q.nq == q.p + 1 && q.consecutive; }

template <class A, int P>
void launch_q3s(const QuadTerm &q, const QuadParams<typename QArith<A>::TT> &prm, cudaStream_t st) {
    constexpr int TE = qs_te<A, P>();
    using S = QStream<A, P, TE>;
    auto kern = k_quad3_stream<A, P, TE>;
    static_assert(S::smem <= 200 * 1024, "quadrature rings larger than the shared memory");
    static const bool attr = [&] {
        TDZ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem));
        return true;
    }();
    (void)attr;
    const int tiles = ((q.nel[0] + TE - 1) / TE) * ((q.nel[1] + TE - 1) / TE);
    // about two CTAs per SM in total, z chunks no shorter than 4 (p + 1) elements
    int chunks = std::max(1, (2 * sm_count() + tiles - 1) / tiles);
    chunks = std::max(1, std::min(chunks, q.nel[2] / (4 * (P + 1))));
    const int zchunk = (q.nel[2] + chunks - 1) / chunks;
    kern<<<dim3(tiles, (q.nel[2] + zchunk - 1) / zchunk), kQsThreads, S::smem, st>>>(prm, zchunk);
}

template <class T>
QuadParams<T> make_qparams(const QuadTerm &q, cd coef, const void *x, void *y) {
    QuadParams<T> prm{};
    const bool dbl = sizeof(T) == 8;
    prm.x = x;
    prm.y = y;
    prm.nq = q.nq;
    for (int d = 0; d < 3; ++d) {
        prm.n[d] = q.n[d];
        prm.nel[d] = q.nel[d];
        if (d < q.dim) {
            prm.off[d] = q.off[d].as<int>();
            prm.N[d] = static_cast<const T *>((dbl ? q.N64[d] : q.N32[d]).ptr);
            prm.w[d] = static_cast<const T *>((dbl ? q.w64[d] : q.w32[d]).ptr);
            prm.xq[d] = static_cast<const T *>((dbl ? q.x64[d] : q.x32[d]).ptr);
        }
    }
    prm.nsoft = q.nsoft;
    for (int c = 0; c < q.nsoft; ++c)
        for (int k = 0; k < 5; ++k) prm.soft[c][k] = (T)q.soft[c][k];
    prm.cre = (T)coef.real();
    prm.cim = (T)coef.imag();
    prm.cre_d = coef.real();
    prm.cim_d = coef.imag();
    return prm;
}

template <class T, int P>
void launch_q(const QuadTerm &q, const QuadParams<T> &prm, cudaStream_t st) {
    const long long nel = (long long)q.nel[0] * q.nel[1] * (q.dim == 3 ? q.nel[2] : 1);
    TDZ_CHECK(nel < (1LL << 31), TDZ_ERR_UNSUPPORTED, "too many elements for the quadrature term");
    if (q.dim == 3) k_quad<T, P, 3><<<(unsigned)nel, kQThreads, 0, st>>>(prm);
    else k_quad<T, P, 2><<<(unsigned)nel, kQThreads, 0, st>>>(prm);
}

template <class T>
void dispatch_q(const QuadTerm &q, cd coef, const void *x, void *y, cudaStream_t st) {
    const QuadParams<T> prm = make_qparams<T>(q, coef, x, y);
    if (stream_ok(q)) {   // FP32: FP32 arithmetic; FP64 vectors: double-float arithmetic
        using A = typename std::conditional<std::is_same<T, float>::value, float, dff>::type;
        switch (q.p) {
        case 2: launch_q3s<A, 2>(q, prm, st); return;
        case 3: launch_q3s<A, 3>(q, prm, st); return;
        case 4: launch_q3s<A, 4>(q, prm, st); return;
        case 5: launch_q3s<A, 5>(q, prm, st); return;
        default: break;
        }
    }
    switch (q.p) {
    case 2: launch_q<T, 2>(q, prm, st); break;
    case 3: launch_q<T, 3>(q, prm, st); break;
    case 4: launch_q<T, 4>(q, prm, st); break;
    case 5: launch_q<T, 5>(q, prm, st); break;
    default: throw Error(TDZ_ERR_UNSUPPORTED, "quadrature term supports degrees 2..5");
    }
}

}  // namespace

void QuadTerm::build(const Space &s, int nsoft_, const double *soft_) {
    on = nsoft_ > 0;
    if (!on) return;
    TDZ_CHECK(s.dim >= 2, TDZ_ERR_UNSUPPORTED, "soft-core centres need a 2D or 3D space");
    TDZ_CHECK(nsoft_ <= kMaxSoft, TDZ_ERR_UNSUPPORTED, "at most 8 soft-core centres");
    TDZ_CHECK(soft_ != nullptr, TDZ_ERR_ARG, "soft-core parameters missing");
    TDZ_CHECK(s.nquad >= 1 && s.nquad <= kMaxQ, TDZ_ERR_UNSUPPORTED, "quadrature term supports 1..10 Gauss points");
    nsoft = nsoft_;
    for (int c = 0; c < nsoft; ++c) {
        for (int k = 0; k < 5; ++k) soft[c][k] = soft_[5 * c + k];
        TDZ_CHECK(soft[c][4] > 0.0, TDZ_ERR_ARG, "soft-core parameter a must be positive");
    }
    dim = s.dim;
    p = s.ax[0].p;
    nq = s.nquad;
    consecutive = true;
    for (int d = 0; d < dim; ++d) {
        const Axis1D &a = s.ax[d];
        TDZ_CHECK(a.nq == nq && a.p == p, TDZ_ERR_INTERNAL, "axis tables disagree");
        for (int e = 0; e + 1 < a.nel; ++e)
            if (a.offset[e + 1] != a.offset[e] + 1) consecutive = false;
        nel[d] = a.nel;
        n[d] = a.n;
        std::vector<int> o(a.offset.begin(), a.offset.end());
        upload(off[d], o);
        upload(N64[d], a.N);
        upload(w64[d], a.wq);
        upload(x64[d], a.xq);
        upload(N32[d], std::vector<float>(a.N.begin(), a.N.end()));
        upload(w32[d], std::vector<float>(a.wq.begin(), a.wq.end()));
        upload(x32[d], std::vector<float>(a.xq.begin(), a.xq.end()));
    }
}

void QuadTerm::apply(cd coef, int prec, const void *x, void *y, cudaStream_t st) const {
    if (!on || coef == cd(0.0)) return;
    if (prec == TDZ_FP32) dispatch_q<float>(*this, coef, x, y, st);
    else dispatch_q<double>(*this, coef, x, y, st);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tdz
