// Fused matrix-free apply of the three-stream Kronecker form (see oper.h),
//   y = T_z (x) M_y (x) M_x x                                   stream A
//     + M_z (x) [M_y (x) T_x + T_y (x) M_x] x                   stream B
//     + Mm_z (x) [M_y (x) S_x + S_y (x) M_x] x                  stream C
// on sm_103a. Replaces MatMult on the assembled AIJ stage matrices and the
// three-pass TDSEZTensorOps::Term (src/tensorops.cpp:97-153).
//
// 3D kernel: a CTA owns a TX x TY column tile and streams the z planes of its
// z chunk. Per input plane it stages the (TY+2p) x (TX+2p) halo tile in
// shared memory, contracts along x (the band rows of its own column in
// registers), then along y (shared memory), and feeds the streams into a
// ring of 2p+1 output-plane accumulators held in registers: plane z
// contributes Z(m, z) w(z) to output planes m = z-p..z+p (the outer bands
// are symmetric, so that is row z of Z), and plane z-p is complete and
// stored once plane z has been added. The complex band combinations are
// formed from the real base bands and the stage scalars (kernel parameters),
// so a stage change needs no upload. Every coefficient is read from HBM once
// per apply (halo re-reads hit L2) and written once.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <type_traits>
#include <vector>

#include "cplx.cuh"
#include "oper.h"

namespace tdz {

template <class T> struct CombP {
    int n;
    int base[kMaxComb];
    T re[kMaxComb], im[kMaxComb];
};

template <class T> struct ApplyParams {
    const void *x;
    void *y;
    int n0, n1, n2;             // sizes along x, y, z (unused axes 1)
    const T *b0, *b1, *b2;      // base bands per axis [nbase][n][2p+1]
    CombP<T> xT, yT, zA, zC;
    int zchunk;
    int zchunk_planes;          // zchunk + 2p (rows of the precomputed outer bands)
    int p;                      // degree (1D kernel)
    T wall_re[2], wall_im[2];   // 1D walls: diagonal values, wall = 0 / n-1
    int walls;
    int za_kind, zc_kind;       // outer combinations: 0 complex, 1 real, 2 imaginary (fewer products)
    const void *sub;            // non-null: y = sub - op x (a residual), same layout as y
    // 3D only: per-CTA partial sums of the stored y, red[blockIdx.x] (FP64):
    // red_mode 1: sum |y|^2, 2: sum conj(dotv) y (dotv laid out as y)
    double2 *red;
    const void *dotv;
    int red_mode;
    int *err;                   // error word of bounded waits (device, library-owned)
};


// the value stored at output element e: op x, or sub[e] - op x
template <class T, class MC, class C>
__device__ __forceinline__ MC out_value(const ApplyParams<T> &prm, size_t e, C v) {
    if (prm.sub) {
        C r = load_c<C>(static_cast<const MC *>(prm.sub)[e]);
        rfma(r, T(-1.f), v);
        v = cnorm(r);
    }
    return store_c<MC>(v);
}
// the same with sub[e] already loaded
template <class T, class MC, class C>
__device__ __forceinline__ MC out_value_sub(const ApplyParams<T> &prm, MC b, C v) {
    if (prm.sub) {
        C r = load_c<C>(b);
        rfma(r, T(-1.f), v);
        v = cnorm(r);
    }
    return store_c<MC>(v);
}

// entry o of row i of a combination of base bands
template <class T, class C>
__device__ __forceinline__ C comb_at(const CombP<T> &cb, const T *bands, int n, int bw, int i, int o) {
    C z = czero<C>();
    for (int t = 0; t < cb.n; ++t) {
        const T b = bands[((size_t)cb.base[t] * n + i) * bw + o];
        z.x = tfma(cb.re[t], b, z.x);
        z.y = tfma(cb.im[t], b, z.y);
    }
    return cnorm(z);
}

// ---------------------------------------------------------------- 3D kernel
// Per z plane, one barrier: the x stage of the next plane and the y and
// outer stages of this plane, then the prefetched tile after next goes from
// registers to shared memory and the one after that is requested (its
// latency overlaps a whole plane of compute). The halo tile and the x-stage
// results are double-buffered.
constexpr int kLoadsPerThread3 = 4;   // covers (TY+2p)(TX+2p) / (TX TY) for p <= 5

// ring of output planes: unrolled with fixed slots (FP32) or shifted per plane
template <class T> constexpr bool kShiftRing = !std::is_same<T, float>::value;

// TX is the largest tile width; the launch may use a narrower one
// (blockDim.x = 16..TX) to fit n0 with less padding. KA / KC: the kind of the
// outer combinations fixed at compile time (0 complex, 1 real, 2 imaginary);
// the double-float CN stage (KC = 2) and mass (KA = 1) get their own
// instantiations, which save a quarter of the outer-stage products.
template <class T, int P, bool HB, bool HC, int TX, int TY, int KA, int KC>
__device__ __noinline__ double2 apply3d_run(const ApplyParams<T> &prm, int x0, int y0, int z0, int z1) {
    using C = typename CT<T>::type;
    constexpr int BW = 2 * P + 1, RY = TY + 2 * P, RX = TX + 2 * P;
    constexpr int NU = 1 + (HB ? 1 : 0) + (HC ? 1 : 0);
    constexpr int UT = 1, US = HB ? 2 : 1;    // slots of u_T and u_S in sU
    static_assert(RY * (16 + 2 * P) <= kLoadsPerThread3 * 16 * TY, "tile larger than the prefetch registers");
    const int txw = blockDim.x;               // tile width of this launch
    const int NT = txw * TY, RXw = txw + 2 * P;
    __shared__ T sYm[BW][TY];
    __shared__ T sYs[HC ? BW : 1][TY];
    __shared__ C sYt[HB ? BW : 1][TY];
    extern __shared__ unsigned char dyn_raw[];
    // dynamic: the double-buffered halo tile and x-stage results, then the
    // precomputed outer-band rows of the run: [plane][o] (A, C complex; M real)
    C (*sIn)[RY][RX] = reinterpret_cast<C (*)[RY][RX]>(dyn_raw);
    C (*sU)[NU][RY][TX] = reinterpret_cast<C (*)[NU][RY][TX]>(dyn_raw + sizeof(C) * 2 * RY * RX);
    C *sZA = reinterpret_cast<C *>(dyn_raw + sizeof(C) * (2 * RY * RX + 2 * NU * RY * TX));
    C *sZC = sZA + (size_t)prm.zchunk_planes * BW;
    T *sZM = reinterpret_cast<T *>(sZC + (HC ? (size_t)prm.zchunk_planes * BW : 0));

    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * txw + tx;
    const int n0 = prm.n0, n1 = prm.n1, n2 = prm.n2;
    using MC = typename MemC<T>::type;
    const MC *__restrict__ X = static_cast<const MC *>(prm.x);
    MC *__restrict__ Y = static_cast<MC *>(prm.y);
    const int gx = x0 + tx, gy = y0 + ty;
    const int zs = z0 - P;
    const int nplanes = (z1 - z0) + 2 * P;

    // band rows of this thread's x column
    T xm[BW], xs[HC ? BW : 1];
    C xt[HB ? BW : 1];
#pragma unroll
    for (int j = 0; j < BW; ++j) {
        const bool in = gx < n0;
        xm[j] = in ? prm.b0[((size_t)kM * n0 + gx) * BW + j] : T(0);
        if constexpr (HC) xs[j] = in ? prm.b0[((size_t)kS * n0 + gx) * BW + j] : T(0);
        if constexpr (HB) xt[j] = in ? comb_at<T, C>(prm.xT, prm.b0, n0, BW, gx, j) : czero<C>();
    }
    for (int i = tid; i < BW * TY; i += NT) {
        const int j = i / TY, r = i % TY, yy = y0 + r;
        const bool in = yy < n1;
        sYm[j][r] = in ? prm.b1[((size_t)kM * n1 + yy) * BW + j] : T(0);
        if constexpr (HC) sYs[j][r] = in ? prm.b1[((size_t)kS * n1 + yy) * BW + j] : T(0);
        if constexpr (HB) sYt[j][r] = in ? comb_at<T, C>(prm.yT, prm.b1, n1, BW, yy, j) : czero<C>();
    }
    for (int i = tid; i < nplanes * BW; i += NT) {
        const int pl = i / BW, o = i % BW, zin = zs + pl;
        const bool in = zin >= 0 && zin < n2;
        sZA[i] = in ? comb_at<T, C>(prm.zA, prm.b2, n2, BW, zin, o) : czero<C>();
        if constexpr (HC) sZC[i] = in ? comb_at<T, C>(prm.zC, prm.b2, n2, BW, zin, o) : czero<C>();
        if constexpr (HB) sZM[i] = in ? prm.b2[((size_t)kM * n2 + zin) * BW + o] : T(0);
    }

    // prefetch registers: element e = tid + q NT of the (RY x RX) tile. The
    // element's place in the plane and in sIn is the same for every plane, so
    // it is resolved once here (off: in-plane offset, -1 outside the grid or
    // the tile; so: slot in sIn, -1 outside the tile).
    C pre[kLoadsPerThread3];
    int off[kLoadsPerThread3], so[kLoadsPerThread3];
#pragma unroll
    for (int q = 0; q < kLoadsPerThread3; ++q) {
        const int e = tid + q * NT;
        off[q] = -1;
        so[q] = -1;
        if (e < RY * RXw) {
            const int r = e / RXw, c = e % RXw;
            so[q] = r * RX + c;
            const int yy = y0 - P + r, xx = x0 - P + c;
            if (yy >= 0 && yy < n1 && xx >= 0 && xx < n0) off[q] = yy * n0 + xx;
        }
    }
    const size_t plane = (size_t)n1 * n0;
    auto load_plane = [&](int zin) {
#pragma unroll
        for (int q = 0; q < kLoadsPerThread3; ++q)
            pre[q] = off[q] >= 0 ? load_c<C>(X[(size_t)zin * plane + off[q]]) : czero<C>();
    };
    // input planes it = lo .. hi-1 (zin = zs + it) lie inside the grid
    const int lo = max(0, -zs), hi = min(nplanes, n2 - zs);
    auto store_in = [&](int it) {
#pragma unroll
        for (int q = 0; q < kLoadsPerThread3; ++q)
            if (so[q] >= 0) (&sIn[it & 1][0][0])[so[q]] = pre[q];
    };
    auto fetch = [&](int it) {   // plane it into the prefetch registers, if it is in the grid
        if (it < hi) load_plane(zs + it);
    };
    // x stage of plane it: sIn[it & 1] -> sU[it & 1]
    auto xstage = [&](int it) {
        const int buf = it & 1;
        for (int r = ty; r < RY; r += TY) {
            C uM = czero<C>(), uT = czero<C>(), uS = czero<C>();
#pragma unroll
            for (int j = 0; j < BW; ++j) {
                const C v = sIn[buf][r][tx + j];
                rfma(uM, xm[j], v);
                if constexpr (HB) cfma(uT, xt[j], v);
                if constexpr (HC) rfma(uS, xs[j], v);
            }
            sU[buf][0][r][tx] = cnorm(uM);
            if constexpr (HB) sU[buf][UT][r][tx] = cnorm(uT);
            if constexpr (HC) sU[buf][US][r][tx] = cnorm(uS);
        }
    };
    // y and outer stages of plane it from sU[it & 1]; output plane
    // zs + it - P + o accumulates in acc[(ring + o) % BW]
    C acc[BW];
#pragma unroll
    for (int s = 0; s < BW; ++s) acc[s] = czero<C>();
    auto yzstage = [&](int it, int ring) {
        const int buf = it & 1;
        C wA = czero<C>(), wB = czero<C>(), wC = czero<C>();
#pragma unroll
        for (int j = 0; j < BW; ++j) {
            const T ym = sYm[j][ty];
            const C um = sU[buf][0][ty + j][tx];
            rfma(wA, ym, um);
            if constexpr (HB) {
                rfma(wB, ym, sU[buf][UT][ty + j][tx]);
                cfma(wB, sYt[j][ty], um);
            }
            if constexpr (HC) {
                rfma(wC, ym, sU[buf][US][ty + j][tx]);
                rfma(wC, sYs[j][ty], um);
            }
        }
        wA = cnorm(wA);
        if constexpr (HB) wB = cnorm(wB);
        if constexpr (HC) wC = cnorm(wC);
        const C *zA = sZA + (size_t)it * BW;
#pragma unroll
        for (int o = 0; o < BW; ++o) {
            C &a = acc[(ring + o) % BW];
            if constexpr (KA == 1) rfma(a, zA[o].x, wA);
            else if constexpr (KA == 2) ifma(a, zA[o].y, wA);
            else cfma(a, zA[o], wA);
            if constexpr (HB) rfma(a, sZM[(size_t)it * BW + o], wB);
            if constexpr (HC) {
                const C zc = sZC[(size_t)it * BW + o];
                if constexpr (KC == 1) rfma(a, zc.x, wC);
                else if constexpr (KC == 2) ifma(a, zc.y, wC);
                else cfma(a, zc, wC);
            }
        }
    };
    // Software pipeline, one barrier per plane. Step it (lo <= it < hi): the
    // x stage of plane it+1 and the y / outer stages of plane it (independent
    // work between two barriers), then plane it+2 from the registers into
    // sIn and the request of plane it+3. sIn and sU are double-buffered: the
    // buffer a step writes was last read before the previous barrier.
    auto step = [&](int it, int ring) {
        xstage(it + 1);                // a plane past hi leaves results that nobody reads
        yzstage(it, ring);
        store_in(it + 2);
        fetch(it + 3);
        __syncthreads();
    };
    if (lo < hi) {
        fetch(lo);
        store_in(lo);
        fetch(lo + 1);
        __syncthreads();
        xstage(lo);
        store_in(lo + 1);
        fetch(lo + 2);
        __syncthreads();
    }
    double2 racc = make_double2(0.0, 0.0);   // this thread's share of the requested sum
    // The side input of output plane zs + it - P (sub for a residual, else dotv
    // for a dot) is requested before the plane's step, so its latency overlaps
    // the step's compute.
    auto side_load = [&](int it) {
        MC sv{};
        if (it >= 2 * P && gx < n0 && gy < n1) {
            const size_t e = ((size_t)(zs + it - P) * n1 + gy) * n0 + gx;
            if (prm.sub) sv = static_cast<const MC *>(prm.sub)[e];
            else if (prm.red_mode == 2) sv = static_cast<const MC *>(prm.dotv)[e];
        }
        return sv;
    };
    auto finish = [&](int it, C &out, MC sv) {   // output plane zs + it - P is complete
        if (it >= 2 * P) {
            const int m = zs + it - P;
            if (gx < n0 && gy < n1) {
                const size_t e = ((size_t)m * n1 + gy) * n0 + gx;
                const MC v = out_value_sub<T, MC>(prm, sv, out);
                Y[e] = v;
                if (prm.red_mode == 1) {
                    racc.x = fma((double)v.x, (double)v.x, fma((double)v.y, (double)v.y, racc.x));
                } else if (prm.red_mode == 2) {
                    const MC d = prm.sub ? static_cast<const MC *>(prm.dotv)[e] : sv;
                    racc.x = fma((double)d.x, (double)v.x, fma((double)d.y, (double)v.y, racc.x));
                    racc.y = fma((double)d.x, (double)v.y, fma(-(double)d.y, (double)v.x, racc.y));
                }
            }
        }
    };

    if constexpr (kShiftRing<T>) {
        // FP64 / double-float: one copy of the step; the ring shifts down by one
        // slot per plane (a few register moves), which keeps the long
        // emulated-FP64 body inside the instruction cache
#pragma unroll 1
        for (int it = 0; it < nplanes; ++it) {
            const MC sv = side_load(it);
            if (it >= lo && it < hi) step(it, 0);
            finish(it, acc[0], sv);
#pragma unroll
            for (int s = 0; s + 1 < BW; ++s) acc[s] = acc[s + 1];
            acc[BW - 1] = czero<C>();
        }
    } else {
        // FP32: the plane loop unrolled by the ring length, fixed slots
        for (int base = 0; base < nplanes; base += BW) {
#pragma unroll
            for (int ph = 0; ph < BW; ++ph) {
                const int it = base + ph;
                if (it >= nplanes) break;
                const int ring = (ph - P + 2 * BW) % BW;
                const MC sv = side_load(it);
                if (it >= lo && it < hi) step(it, ring);
                finish(it, acc[ring], sv);
                acc[ring] = czero<C>();
            }
        }
    }
    return racc;
}

// This CTA owns planes [b L, (b + 1) L) of the (tile, z) order, z fastest
// (L = prm.zchunk): one or more runs of consecutive planes of one tile, each
// with its own 2p halo planes. An even split over a grid of about one wave
// keeps the halo small and leaves no tail wave. A run is a separate
// (not inlined) function, so the register allocation of its plane loop does
// not carry the run loop's state.
template <class T, int P, bool HB, bool HC, int TX, int TY, int KA = 0, int KC = 0>
__global__ void __launch_bounds__(TX *TY) k_apply3d(const __grid_constant__ ApplyParams<T> prm) {
    const int txw = blockDim.x;
    const int n0 = prm.n0, n1 = prm.n1, n2 = prm.n2;
    const int tilesX = (n0 + txw - 1) / txw;
    const long long total = (long long)tilesX * ((n1 + TY - 1) / TY) * n2;
    long long pos = (long long)blockIdx.x * prm.zchunk;
    const long long end = min(total, pos + prm.zchunk);
    double2 racc = make_double2(0.0, 0.0);
    for (bool first = true; pos < end; first = false) {
        const int tile = (int)(pos / n2);
        const int z0 = (int)(pos - (long long)tile * n2);
        const int z1 = (int)min((long long)n2, z0 + (end - pos));
        pos += z1 - z0;
        if (!first) __syncthreads();   // the last run's readers of the band rows are done
        const double2 r =
            apply3d_run<T, P, HB, HC, TX, TY, KA, KC>(prm, (tile % tilesX) * txw, (tile / tilesX) * TY, z0, z1);
        racc.x += r.x;
        racc.y += r.y;
    }
    if (prm.red_mode) {   // CTA sum -> red[blockIdx.x] (fixed order: deterministic)
        __shared__ double2 wsum[32];
        for (int off = 16; off > 0; off >>= 1) {
            racc.x += __shfl_down_sync(0xffffffffu, racc.x, off);
            racc.y += __shfl_down_sync(0xffffffffu, racc.y, off);
        }
        const int tid = threadIdx.y * blockDim.x + threadIdx.x, nw = (blockDim.x * blockDim.y + 31) / 32;
        if ((tid & 31) == 0) wsum[tid >> 5] = racc;
        __syncthreads();
        if (tid == 0) {
            double2 t = make_double2(0.0, 0.0);
            for (int w = 0; w < nw; ++w) { t.x += wsum[w].x; t.y += wsum[w].y; }
            prm.red[blockIdx.x] = t;
        }
    }
}

// ---------------------------------------------------------------- 2D kernel
// x stage on a TX-wide row tile, outer stage along y with the register ring.
template <class T, int P, bool HB, bool HC, int TX>
__global__ void __launch_bounds__(TX) k_apply2d(const ApplyParams<T> prm) {
    using C = typename CT<T>::type;
    constexpr int BW = 2 * P + 1, RX = TX + 2 * P;
    __shared__ C sIn[RX];
    __shared__ C sZA[BW], sZC[BW];
    __shared__ T sZM[BW];
    const int tx = threadIdx.x;
    const int n0 = prm.n0, n1 = prm.n1;
    const int x0 = blockIdx.x * TX, gx = x0 + tx;
    const int z0 = blockIdx.y * prm.zchunk;
    const int z1 = min(n1, z0 + prm.zchunk);
    if (z0 >= z1) return;
    using MC = typename MemC<T>::type;
    const MC *__restrict__ X = static_cast<const MC *>(prm.x);
    MC *__restrict__ Y = static_cast<MC *>(prm.y);
    T xm[BW], xs[HC ? BW : 1];
    C xt[HB ? BW : 1];
#pragma unroll
    for (int j = 0; j < BW; ++j) {
        const bool in = gx < n0;
        xm[j] = in ? prm.b0[((size_t)kM * n0 + gx) * BW + j] : T(0);
        if constexpr (HC) xs[j] = in ? prm.b0[((size_t)kS * n0 + gx) * BW + j] : T(0);
        if constexpr (HB) xt[j] = in ? comb_at<T, C>(prm.xT, prm.b0, n0, BW, gx, j) : czero<C>();
    }
    C acc[BW];
#pragma unroll
    for (int s = 0; s < BW; ++s) acc[s] = czero<C>();
    const int zs = z0 - P;
    const int nplanes = (z1 - z0) + 2 * P;
    for (int base = 0; base < nplanes; base += BW) {
#pragma unroll
        for (int ph = 0; ph < BW; ++ph) {
            const int it = base + ph;
            if (it >= nplanes) break;
            const int zin = zs + it;
            if (zin >= 0 && zin < n1) {
                __syncthreads();
                for (int c = tx; c < RX; c += TX) {
                    const int xx = x0 - P + c;
                    sIn[c] = (xx >= 0 && xx < n0) ? load_c<C>(X[(size_t)zin * n0 + xx]) : czero<C>();
                }
                if (tx < BW) {
                    sZA[tx] = comb_at<T, C>(prm.zA, prm.b1, n1, BW, zin, tx);
                    if constexpr (HB) sZM[tx] = prm.b1[((size_t)kM * n1 + zin) * BW + tx];
                    if constexpr (HC) sZC[tx] = comb_at<T, C>(prm.zC, prm.b1, n1, BW, zin, tx);
                }
                __syncthreads();
                C uM = czero<C>(), uT = czero<C>(), uS = czero<C>();
#pragma unroll
                for (int j = 0; j < BW; ++j) {
                    const C v = sIn[tx + j];
                    rfma(uM, xm[j], v);
                    if constexpr (HB) cfma(uT, xt[j], v);
                    if constexpr (HC) rfma(uS, xs[j], v);
                }
                uM = cnorm(uM);
                if constexpr (HB) uT = cnorm(uT);
                if constexpr (HC) uS = cnorm(uS);
#pragma unroll
                for (int o = 0; o < BW; ++o) {
                    C &a = acc[(ph - P + o + 2 * BW) % BW];
                    kfma(a, sZA[o], uM, prm.za_kind);
                    if constexpr (HB) rfma(a, sZM[o], uT);
                    if constexpr (HC) kfma(a, sZC[o], uS, prm.zc_kind);
                }
            }
            if (it >= 2 * P) {
                const int m = zin - P;
                if (gx < n0) Y[(size_t)m * n0 + gx] = out_value<T, MC>(prm, (size_t)m * n0 + gx, acc[(ph - P + 2 * BW) % BW]);
            }
            acc[(ph - P + 2 * BW) % BW] = czero<C>();
        }
    }
}

// ---------------------------------------------------------------- 1D kernel
template <class T>
__global__ void k_apply1d(const ApplyParams<T> prm) {
    using C = typename CT<T>::type;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = prm.n0, p = prm.p, bw = 2 * p + 1;
    if (i >= n) return;
    const C *__restrict__ X = static_cast<const C *>(prm.x);
    C *__restrict__ Y = static_cast<C *>(prm.y);
    const bool wall_i = prm.walls && (i == 0 || i == n - 1);
    C acc = czero<C>();
    if (wall_i) {
        const int s = i == 0 ? 0 : 1;
        C d;
        d.x = prm.wall_re[s];
        d.y = prm.wall_im[s];
        cfma(acc, d, X[i]);
    } else {
        for (int o = 0; o < bw; ++o) {
            const int j = i - p + o;
            if (j < 0 || j >= n) continue;
            if (prm.walls && (j == 0 || j == n - 1)) continue;
            cfma(acc, comb_at<T, C>(prm.zA, prm.b0, n, bw, i, o), X[j]);
        }
    }
    if (prm.sub) {
        const C b = static_cast<const C *>(prm.sub)[i];
        acc.x = b.x - acc.x;
        acc.y = b.y - acc.y;
    }
    Y[i] = acc;
}

// ---------------------------------------------------------------- launch helpers
constexpr int kTX3 = 32, kTY3 = 8, kTX2 = 128;
// tile height: 8 rows for FP32; 16 for FP64 and double-float, which recompute
// the 2p halo rows of the x stage (ratio (16 + 2p) / 16 instead of (8 + 2p) / 8),
// except with all three streams, whose registers need the smaller CTA
template <class T, bool HB, bool HC> struct TileY {
    static constexpr int v = std::is_same<T, float>::value || (HB && HC) ? 8 : 16;
};

// z chunk per CTA: about `target` CTAs in total (0: 8 per SM), chunks no
// shorter than 4p planes (the 2p halo planes of a chunk are re-read)
inline int pick_chunk(int tiles, int n_outer, int P, int target = 0) {
    if (target <= 0) target = 8 * sm_count();
    int chunks = (target + tiles - 1) / tiles;
    chunks = std::max(1, std::min(chunks, n_outer / std::max(1, 4 * P)));
    return (n_outer + chunks - 1) / chunks;
}

// tile width 16..32 (multiple of 4) with the least padding of n0; ties go to the wider
inline int pick_tile_x(int n0) {
    int best = kTX3, pad = (n0 + kTX3 - 1) / kTX3 * kTX3;
    for (int t = kTX3 - 4; t >= 16; t -= 4) {
        const int p = (n0 + t - 1) / t * t;
        if (p < pad) { pad = p; best = t; }
    }
    return best;
}

// ---------------------------------------------------------------- autotuner
// Launch shape (tile width, z chunk) of the 3D apply, chosen per kernel
// instantiation and grid size by timing the candidates on the first launch
// (CUDA events on the caller's stream, one warm-up and two timed launches
// each, about 30 ms once for the double-float apply). Off: the heuristic
// shape. Switched by tdz_set_autotune (default on).
struct TuneKey {
    const void *kern;
    int n0, n1, n2;
    bool operator<(const TuneKey &o) const {
        if (kern != o.kern) return kern < o.kern;
        if (n0 != o.n0) return n0 < o.n0;
        if (n1 != o.n1) return n1 < o.n1;
        return n2 < o.n2;
    }
};
bool autotune_enabled();
bool tune_verbose();   // TDZ_AUTOTUNE_VERBOSE set: the autotuner prints each candidate's time
// a fixed launch shape for every 3D apply (no autotuning): TDZ_APPLY3D_SHAPE="tile_x,run"
// in the environment at load time, or tdz_set_apply3d_shape
bool forced_shape(int *txw, int *run);
void set_forced_shape(int txw, int run);
bool tune_lookup(const TuneKey &k, int *txw, int *zchunk);
void tune_store(const TuneKey &k, int txw, int zchunk);

template <class T, int P, bool HB, bool HC, int KA = 0, int KC = 0>
inline void run3d(const ApplyParams<T> &prm0, cudaStream_t st) {
    using C = typename CT<T>::type;
    constexpr int TY = TileY<T, HB, HC>::v, NU = 1 + (HB ? 1 : 0) + (HC ? 1 : 0);
    auto kern = k_apply3d<T, P, HB, HC, kTX3, TY, KA, KC>;
    const bool fp32 = std::is_same<T, float>::value;
    const size_t tile_smem = sizeof(C) * ((size_t)2 * (TY + 2 * P) * (kTX3 + 2 * P) + 2 * NU * (TY + 2 * P) * kTX3);
    auto smem_for = [&](int zchunk) {
        const size_t rows = (size_t)(zchunk + 2 * P) * (2 * P + 1);
        return tile_smem + rows * sizeof(C) * (HC ? 2 : 1) + (HB ? rows * sizeof(T) : 0);
    };
    // shared memory grows with the run length (its band rows, at most n2 + 2p
    // planes): one opt-in to the largest size, occupancy at the largest size
    constexpr size_t kMaxDyn = 200 * 1024;
    static const int nsm = [&] {   // once per instantiation (thread-safe static initialisation)
        TDZ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDyn));
        int dev = 0, n = 0;
        TDZ_CUDA(cudaGetDevice(&dev));
        TDZ_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        return n;
    }();
    const int n2 = prm0.n2;
    TDZ_CHECK(smem_for(n2) <= kMaxDyn, TDZ_ERR_UNSUPPORTED, "outer axis too long for the 3D apply");
    thread_local int occ_n2 = -1, occ_slots = 0;   // resident CTAs at the last n2 seen
    if (occ_n2 != n2) {
        int per_sm = 0;
        TDZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTX3 * TY, smem_for(n2)));
        occ_slots = std::max(1, per_sm) * nsm;
        occ_n2 = n2;
    }
    const int slots = occ_slots;
    auto tiles_for = [&](int txw) { return ((prm0.n0 + txw - 1) / txw) * ((prm0.n1 + TY - 1) / TY); };
    // run length L for a grid of about g CTAs (no shorter than 4p planes)
    auto seg_for = [&](int txw, long long g) {
        const long long total = (long long)tiles_for(txw) * n2;
        return (int)std::min<long long>(total, std::max<long long>(4 * P, (total + g - 1) / g));
    };
    // (tuning candidates run without the fused reduction; the final launch
    // keeps its grid within the reduction's partial-sum slots)
    auto launch = [&](int txw, int seg, bool candidate = false) {
        ApplyParams<T> prm = prm0;
        const long long total = (long long)tiles_for(txw) * n2;
        if (candidate) prm.red_mode = 0;
        if (prm.red_mode) seg = (int)std::max<long long>(seg, (total + kApplyRedCap - 1) / kApplyRedCap);
        prm.zchunk = seg;
        prm.zchunk_planes = std::min(seg, n2) + 2 * P;
        const unsigned grid = (unsigned)((total + seg - 1) / seg);
        TDZ_CHECK(smem_for(std::min(seg, n2)) <= kMaxDyn, TDZ_ERR_UNSUPPORTED, "outer axis too long for the 3D apply");
        kern<<<grid, dim3(txw, TY), smem_for(std::min(seg, n2)), st>>>(prm);
    };
    // heuristic: one wave of persistent CTAs; FP32 full warps along x and two
    // waves, FP64 and double-float the least x padding
    int txw = fp32 ? kTX3 : pick_tile_x(prm0.n0);
    int zchunk = seg_for(txw, (long long)slots * (fp32 ? 2 : 1));
    const TuneKey key{reinterpret_cast<const void *>(kern), prm0.n0, prm0.n1, prm0.n2};
    if (forced_shape(&txw, &zchunk)) {
        txw = std::max(16, std::min(kTX3, txw / 4 * 4));
        zchunk = std::max(4 * P, zchunk);
    } else if (autotune_enabled() && !tune_lookup(key, &txw, &zchunk)) {
        std::vector<std::pair<int, int>> cand;
        for (int t = kTX3; t >= 16; t -= 4) {
            if ((prm0.n0 + t - 1) / t * t > (prm0.n0 + kTX3 - 1) / kTX3 * kTX3) continue;   // more padding than 32
            for (int w : {1, 2, 3, 4, 8}) {
                const int z = seg_for(t, (long long)slots * w);
                if (std::find(cand.begin(), cand.end(), std::make_pair(t, z)) == cand.end()) cand.push_back({t, z});
            }
        }
        cudaEvent_t e0, e1;
        TDZ_CUDA(cudaEventCreate(&e0));
        TDZ_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (const auto &c : cand) {
            launch(c.first, c.second, true);
            TDZ_CUDA(cudaEventRecord(e0, st));
            launch(c.first, c.second, true);
            launch(c.first, c.second, true);
            TDZ_CUDA(cudaEventRecord(e1, st));
            TDZ_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            TDZ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (tune_verbose())
                std::fprintf(stderr, "tdz autotune apply3d<%s,p%d,B%d,C%d,%d%d> %dx%dx%d: tile %dx%d run %d grid %lld: %.1f us\n",
                             sizeof(T) == 4 ? "f32" : (std::is_same<T, double>::value ? "f64" : "df"), P, (int)HB,
                             (int)HC, KA, KC, prm0.n0, prm0.n1, n2, c.first, TY, c.second,
                             ((long long)tiles_for(c.first) * n2 + c.second - 1) / c.second, 500.f * ms);
            if (ms < best) { best = ms; txw = c.first; zchunk = c.second; }
        }
        TDZ_CUDA(cudaEventDestroy(e0));
        TDZ_CUDA(cudaEventDestroy(e1));
        tune_store(key, txw, zchunk);
    }
    launch(txw, zchunk);
}

template <class T, int P, bool HB, bool HC>
inline void run2d(const ApplyParams<T> &prm0, cudaStream_t st) {
    ApplyParams<T> prm = prm0;
    const int tiles = (prm.n0 + kTX2 - 1) / kTX2;
    prm.zchunk = pick_chunk(tiles, prm.n1, P);
    dim3 grid(tiles, (prm.n1 + prm.zchunk - 1) / prm.zchunk);
    k_apply2d<T, P, HB, HC, kTX2><<<grid, kTX2, 0, st>>>(prm);
}

// per-degree entry points (apply_p<P>.cu)
// (prec: TDZ_FP32, TDZ_FP64, TDZ_FP64_DF, or kPrecF32M64 with pf on FP64 vectors)
#define TDZ_APPLY_DECL(P)                                                                                  \
    void apply_p##P(int dim, bool hb, bool hc, const ApplyParams<float> &pf, const ApplyParams<double> &pd, \
                    const ApplyParams<dff> &pdf, int prec, cudaStream_t st);
TDZ_APPLY_DECL(2)
TDZ_APPLY_DECL(3)
TDZ_APPLY_DECL(4)
TDZ_APPLY_DECL(5)
#undef TDZ_APPLY_DECL

}  // namespace tdz
