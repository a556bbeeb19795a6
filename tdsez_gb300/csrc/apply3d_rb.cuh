// Register-blocked fused 3D apply of the three-stream Kronecker form (see
// oper.h and apply_kernels.cuh for the operator), FP32 or double-float
// arithmetic on FP32 or FP64 vectors. Replaces MatMult on the assembled AIJ
// stage matrices and the three band passes of TDSEZTensorOps::Term
// (src/tensorops.cpp:97-153) for every 3D apply that is not native FP64.
//
// A CTA of txw x NTY threads owns a txw x TY column tile (TY = NTY R) and
// streams the z planes of its run. Thread (tx, ty) owns output column
// x0 + tx and the R output rows y0 + ty R + r, so the z coefficients it
// reads once per plane and the x-stage rows it reads for the y contraction
// serve R outputs. Per input plane:
//   staging  the (TY + 2p) x (32 + 2p) halo tile arrives in shared memory
//            three planes ahead: by TMA (cp.async.bulk.tensor.3d, one
//            elected thread, completion on an mbarrier) for FP64 vectors,
//            whose rows are 16-byte multiples for any n_x; by cp.async
//            (8-byte copies, zero fill outside the grid) for FP32 vectors,
//            whose rows are not 16-byte multiples for odd n_x. FP64 input is
//            converted once per element to the arithmetic type (integer
//            splits, off the FP64 pipe) into a second buffer.
//   x stage  the band rows of the thread's column live in registers.
//   y stage  in registers from the x-stage rows in shared memory; the
//            y band rows of the thread's R rows live in registers for FP32
//            without the inner-axis stream, else in shared memory.
//   z stage  a ring of 2p+1 output-plane accumulators per output row in
//            registers: plane z adds Z(m, z) w(z) to output planes m =
//            z-p..z+p; plane z-p is then complete and stored.
// One barrier per plane: after it, plane it+3 is requested, the x stage of
// plane it+1 and the y / z stages of plane it run. Staging buffers are
// triple-buffered, converted tiles and x-stage results double-buffered.
// Every mbarrier wait is bounded (clock64); a time-out sets the library's
// error word (prm.err, read by take_apply_error()) and the CTA finishes
// without waiting again.
#pragma once
#include <cudaTypedefs.h>

#include <cstring>

#include "apply_kernels.cuh"

namespace tdz {

constexpr int kRbTX = 32;   // widest tile (blockDim.x = txw <= 32)
constexpr long long kRbWaitCycles = 4000000000LL;   // about 2 s at 2 GHz
// CTAs per SM the register allocation is fitted to (256-thread FP32 CTAs: two)
template <class T> struct RbMinBlocks { static constexpr int v = std::is_same<T, float>::value ? 2 : 1; };

template <class MC> struct IsF64Mem { static constexpr bool v = std::is_same<MC, double2>::value; };

// FP64 -> FP32 keeping the leading 24 significand bits (truncation, relative
// error below 2^-23) with integer operations; |v| < 2^-100 gives 0, values
// beyond the FP32 range a non-finite result
__device__ __forceinline__ float d2f_trunc(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const unsigned int h32 = (unsigned int)(u >> 32);
    const unsigned int sign = h32 & 0x80000000u;
    const int e = (int)((h32 >> 20) & 0x7FFu) - 1023;
    if (e < -100) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float(sign | 0x7F800000u | (e == 1024 && (u << 12) ? 0x400000u : 0u));
    const unsigned int m23 = ((h32 & 0xFFFFFu) << 3) | ((unsigned int)u >> 29);
    return __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | m23);
}

// memory complex -> arithmetic complex
template <class C, class MC> __device__ __forceinline__ C rb_load(const MC &m);
template <> __device__ __forceinline__ float2 rb_load<float2, float2>(const float2 &m) { return m; }
template <> __device__ __forceinline__ float2 rb_load<float2, double2>(const double2 &m) {
    return make_float2(d2f_trunc(m.x), d2f_trunc(m.y));
}
template <> __device__ __forceinline__ cdff rb_load<cdff, double2>(const double2 &m) {
    return load_c<cdff, double2>(m);
}
// arithmetic complex -> memory complex
template <class MC, class C> __device__ __forceinline__ MC rb_store(const C &c);
template <> __device__ __forceinline__ float2 rb_store<float2, float2>(const float2 &c) { return c; }
template <> __device__ __forceinline__ double2 rb_store<double2, float2>(const float2 &c) {
    return make_double2(f2d_exact(c.x), f2d_exact(c.y));
}
template <> __device__ __forceinline__ double2 rb_store<double2, cdff>(const cdff &c) {
    return store_c<double2, cdff>(c);
}
// sub - v in the arithmetic type (the residual of a fused b - A x)
template <class C, class MC> __device__ __forceinline__ C rb_sub(const MC &b, C v) {
    C r = rb_load<C, MC>(b);
    r.x = tfma(decltype(v.x)(-1.f), v.x, r.x);
    r.y = tfma(decltype(v.y)(-1.f), v.y, r.y);
    return cnorm(r);
}

__device__ __forceinline__ uint32_t rb_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool rb_mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; false (and the error word set) on time-out
__device__ __forceinline__ bool rb_mbar_wait(uint32_t bar, uint32_t parity, int *err) {
    if (rb_mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!rb_mbar_try(bar, parity)) {
        if (clock64() - t0 > kRbWaitCycles) {
            if (err) atomicExch(err, 1);
            return false;
        }
    }
    return true;
}

// shape and shared-memory layout of one instantiation
template <class T, class MC, int P, bool HB, bool HC, int NTY, int R> struct RbShape {
    using C = typename CT<T>::type;
    static constexpr int BW = 2 * P + 1, TY = NTY * R, RY = TY + 2 * P, RX = kRbTX + 2 * P;
    static constexpr int NU = 1 + (HB ? 1 : 0) + (HC ? 1 : 0);
    static constexpr bool kTma = IsF64Mem<MC>::v;
    static constexpr bool kConv = !std::is_same<MC, C>::value;   // staged tile converted before use
    static constexpr bool kYReg = std::is_same<T, float>::value && !HB;
    static constexpr size_t al(size_t b) { return (b + 127) / 128 * 128; }
    static constexpr size_t kLand = al(sizeof(MC) * RY * RX);     // one staged plane
    static constexpr size_t kConvB = kConv ? al(sizeof(C) * RY * RX) : 0;
    static constexpr size_t kU = al(sizeof(C) * NU * RY * kRbTX);
    static constexpr size_t oLand = 128;                         // after the mbarriers
    static constexpr size_t oConv = oLand + 3 * kLand;
    static constexpr size_t oU = oConv + 2 * kConvB;
    static constexpr size_t oZ = oU + 2 * kU;
    static constexpr size_t zrow = sizeof(C) * BW * (HC ? 2 : 1) + (HB ? sizeof(T) * BW : 0);
    // + 128: the dynamic segment is re-aligned to 128 bytes in the kernel (TMA destinations)
    static size_t smem(int planes) { return 128 + oZ + (size_t)planes * zrow; }
    static constexpr uint32_t kTxBytes = (uint32_t)(sizeof(MC) * RY * RX);
};

template <class T, class MC, int P, bool HB, bool HC, int NTY, int R, int KA, int KC>
__device__ __noinline__ double2 rb_run(const ApplyParams<T> &prm, const CUtensorMap *xmap, int x0, int y0, int z0,
                                       int z1, uint32_t &par, bool &dead) {
    using Sh = RbShape<T, MC, P, HB, HC, NTY, R>;
    using C = typename Sh::C;
    constexpr int BW = Sh::BW, TY = Sh::TY, RY = Sh::RY, RX = Sh::RX;
    constexpr int UT = 1, US = HB ? 2 : 1;
    extern __shared__ __align__(128) unsigned char rb_dyn[];
    unsigned char *rb_raw = rb_dyn + ((128u - (rb_smem(rb_dyn) & 127u)) & 127u);
    __shared__ T sYm[Sh::kYReg ? 1 : BW][TY];
    __shared__ T sYs[(HC && !Sh::kYReg) ? BW : 1][TY];
    __shared__ C sYt[HB ? BW : 1][TY];

    uint64_t *mbar = reinterpret_cast<uint64_t *>(rb_raw);
    MC *land = reinterpret_cast<MC *>(rb_raw + Sh::oLand);
    C *conv = reinterpret_cast<C *>(rb_raw + Sh::oConv);
    C *sU = reinterpret_cast<C *>(rb_raw + Sh::oU);
    C *sZA = reinterpret_cast<C *>(rb_raw + Sh::oZ);
    C *sZC = sZA + (size_t)prm.zchunk_planes * BW;
    T *sZM = reinterpret_cast<T *>(sZC + (HC ? (size_t)prm.zchunk_planes * BW : 0));
    auto landp = [&](int b) { return reinterpret_cast<MC *>(reinterpret_cast<unsigned char *>(land) + b * Sh::kLand); };
    auto convp = [&](int b) { return reinterpret_cast<C *>(reinterpret_cast<unsigned char *>(conv) + b * Sh::kConvB); };
    auto up = [&](int b, int s, int q) {   // x-stage results: [buf][stream][row][column]
        return reinterpret_cast<C *>(reinterpret_cast<unsigned char *>(sU) + b * Sh::kU) + ((size_t)s * RY + q) * kRbTX;
    };

    const int txw = blockDim.x, tx = threadIdx.x, ty = threadIdx.y, tid = ty * txw + tx, NT = txw * NTY;
    const int n0 = prm.n0, n1 = prm.n1, n2 = prm.n2;
    const MC *__restrict__ X = static_cast<const MC *>(prm.x);
    MC *__restrict__ Y = static_cast<MC *>(prm.y);
    const int gx = x0 + tx;
    const int zs = z0 - P;
    const int nplanes = (z1 - z0) + 2 * P;
    const int RXw = txw + 2 * P;

    // band rows: x (this thread's column) and y (its R rows) in registers
    T xm[BW], xs[HC ? BW : 1];
    C xt[HB ? BW : 1];
#pragma unroll
    for (int j = 0; j < BW; ++j) {
        const bool in = gx < n0;
        xm[j] = in ? prm.b0[((size_t)kM * n0 + gx) * BW + j] : T(0);
        if constexpr (HC) xs[j] = in ? prm.b0[((size_t)kS * n0 + gx) * BW + j] : T(0);
        if constexpr (HB) xt[j] = in ? comb_at<T, C>(prm.xT, prm.b0, n0, BW, gx, j) : czero<C>();
    }
    T ymr[Sh::kYReg ? R : 1][Sh::kYReg ? BW : 1], ysr[(Sh::kYReg && HC) ? R : 1][(Sh::kYReg && HC) ? BW : 1];
    if constexpr (Sh::kYReg) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int yy = y0 + ty * R + r;
            const bool in = yy < n1;
#pragma unroll
            for (int j = 0; j < BW; ++j) {
                ymr[r][j] = in ? prm.b1[((size_t)kM * n1 + yy) * BW + j] : T(0);
                if constexpr (HC) ysr[r][j] = in ? prm.b1[((size_t)kS * n1 + yy) * BW + j] : T(0);
            }
        }
    } else {
        for (int i = tid; i < BW * TY; i += NT) {
            const int j = i / TY, r = i % TY, yy = y0 + r;
            const bool in = yy < n1;
            sYm[j][r] = in ? prm.b1[((size_t)kM * n1 + yy) * BW + j] : T(0);
            if constexpr (HC) sYs[j][r] = in ? prm.b1[((size_t)kS * n1 + yy) * BW + j] : T(0);
        }
    }
    if constexpr (HB) {
        for (int i = tid; i < BW * TY; i += NT) {
            const int j = i / TY, r = i % TY, yy = y0 + r;
            sYt[j][r] = yy < n1 ? comb_at<T, C>(prm.yT, prm.b1, n1, BW, yy, j) : czero<C>();
        }
    }
    for (int i = tid; i < nplanes * BW; i += NT) {
        const int pl = i / BW, o = i % BW, zin = zs + pl;
        const bool in = zin >= 0 && zin < n2;
        sZA[i] = in ? comb_at<T, C>(prm.zA, prm.b2, n2, BW, zin, o) : czero<C>();
        if constexpr (HC) sZC[i] = in ? comb_at<T, C>(prm.zC, prm.b2, n2, BW, zin, o) : czero<C>();
        if constexpr (HB) sZM[i] = in ? prm.b2[((size_t)kM * n2 + zin) * BW + o] : T(0);
    }
    // the band rows and the previous run's readers of the staging buffers:
    // everything above is visible, nothing of the last run is still read
    __syncthreads();

    // staging of input plane it (zin = zs + it, inside the grid) into land[it % 3]
    const int lo = max(0, -zs), hi = min(nplanes, n2 - zs);
    const size_t plane = (size_t)n1 * n0;
    auto issue = [&](int it) {
        if (it >= hi) {
            if constexpr (!Sh::kTma) asm volatile("cp.async.commit_group;\n" ::);
            return;
        }
        const int b = it % 3;
        if constexpr (Sh::kTma) {
            if (tid == 0 && !dead) {
                const uint32_t bar = rb_smem(&mbar[b]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(Sh::kTxBytes)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                    "%4}], [%5];" ::"r"(rb_smem(landp(b))),
                    "l"(reinterpret_cast<uint64_t>(xmap)), "r"(2 * (x0 - P)), "r"(y0 - P), "r"(zs + it), "r"(bar)
                    : "memory");
            }
        } else {
            // rows ty, ty + NTY, ...; columns tx and tx + txw (2p <= 10 < txw)
            MC *dst = landp(b);
            const MC *src = X + (size_t)(zs + it) * plane;
            for (int r = ty; r < RY; r += NTY) {
                const int yy = y0 - P + r;
                const bool yin = yy >= 0 && yy < n1;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int c = tx + h * txw;
                    if (c >= RXw) break;
                    const int xx = x0 - P + c;
                    const bool in = yin && xx >= 0 && xx < n0;
                    const MC *s = in ? src + (size_t)yy * n0 + xx : X;
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(rb_smem(dst + r * RX + c)),
                                 "l"(s), "r"(in ? 8 : 0)
                                 : "memory");
                }
            }
            asm volatile("cp.async.commit_group;\n" ::);
        }
    };
    // plane it has arrived (for this thread's view); converted if needed
    auto arrive = [&](int it) {
        if (it >= hi) return;
        const int b = it % 3;
        if constexpr (Sh::kTma) {
            if (!dead) {
                if (!rb_mbar_wait(rb_smem(&mbar[b]), (par >> b) & 1u, prm.err)) dead = true;
            }
            par ^= 1u << b;
        } else {
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        }
        if constexpr (Sh::kConv) {
            const MC *s = landp(b);
            C *d = convp(it & 1);
            for (int r = ty; r < RY; r += NTY) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int c = tx + h * txw;
                    if (c >= RXw) break;
                    d[r * RX + c] = rb_load<C, MC>(s[r * RX + c]);
                }
            }
        }
    };
    auto tile = [&](int it) -> const C * {
        if constexpr (Sh::kConv) return convp(it & 1);
        else return reinterpret_cast<const C *>(landp(it % 3));
    };
    // x stage of plane it: tile(it) -> sU[it & 1]
    // (the thread's rows ty, ty + NTY, ... are unrolled together, so their
    // independent accumulation chains interleave)
    constexpr int XR = (RY + NTY - 1) / NTY;
    auto xstage = [&](int it) {
        const C *in = tile(it);
        const int buf = it & 1;
        C uM[XR], uT[XR], uS[XR];
#pragma unroll
        for (int k = 0; k < XR; ++k) { uM[k] = czero<C>(); uT[k] = czero<C>(); uS[k] = czero<C>(); }
#pragma unroll
        for (int j = 0; j < BW; ++j) {
#pragma unroll
            for (int k = 0; k < XR; ++k) {
                const int q = ty + k * NTY;
                if (k == XR - 1 && q >= RY) break;
                const C v = in[q * RX + tx + j];
                rfma(uM[k], xm[j], v);
                if constexpr (HB) cfma(uT[k], xt[j], v);
                if constexpr (HC) rfma(uS[k], xs[j], v);
            }
        }
#pragma unroll
        for (int k = 0; k < XR; ++k) {
            const int q = ty + k * NTY;
            if (k == XR - 1 && q >= RY) break;
            up(buf, 0, q)[tx] = cnorm(uM[k]);
            if constexpr (HB) up(buf, UT, q)[tx] = cnorm(uT[k]);
            if constexpr (HC) up(buf, US, q)[tx] = cnorm(uS[k]);
        }
    };
    // y and z stages of plane it; output plane zs + it - P + o of row r
    // accumulates in acc[r][(ring + o) % BW]
    C acc[R][BW];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int s = 0; s < BW; ++s) acc[r][s] = czero<C>();
    auto yzstage = [&](int it, int ring) {
        const int buf = it & 1;
        C wA[R], wB[R], wC[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { wA[r] = czero<C>(); wB[r] = czero<C>(); wC[r] = czero<C>(); }
#pragma unroll
        for (int qq = 0; qq < R + 2 * P; ++qq) {
            const int q = ty * R + qq;
            const C um = up(buf, 0, q)[tx];
            C us = czero<C>(), ut = czero<C>();
            if constexpr (HC) us = up(buf, US, q)[tx];
            if constexpr (HB) ut = up(buf, UT, q)[tx];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int j = qq - r;
                if (j < 0 || j >= BW) continue;
                const int row = ty * R + r;
                T ym;
                if constexpr (Sh::kYReg) ym = ymr[r][j];
                else ym = sYm[j][row];
                rfma(wA[r], ym, um);
                if constexpr (HB) {
                    rfma(wB[r], ym, ut);
                    cfma(wB[r], sYt[j][row], um);
                }
                if constexpr (HC) {
                    T ysv;
                    if constexpr (Sh::kYReg) ysv = ysr[r][j];
                    else ysv = sYs[j][row];
                    rfma(wC[r], ym, us);
                    rfma(wC[r], ysv, um);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            wA[r] = cnorm(wA[r]);
            if constexpr (HB) wB[r] = cnorm(wB[r]);
            if constexpr (HC) wC[r] = cnorm(wC[r]);
        }
        const C *zA = sZA + (size_t)it * BW;
#pragma unroll
        for (int o = 0; o < BW; ++o) {
            const C za = zA[o];
            C zc = czero<C>();
            T zm = T(0);
            if constexpr (HC) zc = sZC[(size_t)it * BW + o];
            if constexpr (HB) zm = sZM[(size_t)it * BW + o];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                C &a = acc[r][(ring + o) % BW];
                if constexpr (KA == 1) rfma(a, za.x, wA[r]);
                else if constexpr (KA == 2) ifma(a, za.y, wA[r]);
                else cfma(a, za, wA[r]);
                if constexpr (HB) rfma(a, zm, wB[r]);
                if constexpr (HC) {
                    if constexpr (KC == 1) rfma(a, zc.x, wC[r]);
                    else if constexpr (KC == 2) ifma(a, zc.y, wC[r]);
                    else cfma(a, zc, wC[r]);
                }
            }
        }
    };
    auto step = [&](int it, int ring) {
        arrive(it + 1);
        __syncthreads();
        issue(it + 3);
        if (it + 1 < hi) xstage(it + 1);
        yzstage(it, ring);
    };
    // prologue: planes lo, lo+1, lo+2 requested, plane lo staged and contracted along x
    if (lo < hi) {
        issue(lo);
        issue(lo + 1);
        arrive(lo);
        __syncthreads();
        issue(lo + 2);
        xstage(lo);
    }

    double2 racc = make_double2(0.0, 0.0);
    float2 facc = make_float2(0.f, 0.f);
    auto side_load = [&](int it, MC (&sv)[R]) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            sv[r] = MC{};
            const int gy = y0 + ty * R + r;
            if (it >= 2 * P && gx < n0 && gy < n1) {
                const size_t e = ((size_t)(zs + it - P) * n1 + gy) * n0 + gx;
                if (prm.sub) sv[r] = static_cast<const MC *>(prm.sub)[e];
                else if (prm.red_mode == 2) sv[r] = static_cast<const MC *>(prm.dotv)[e];
            }
        }
    };
    auto finish = [&](int it, int slot, const MC (&sv)[R]) {
        if (it < 2 * P) {   // a halo output plane of the run: not stored, its slot is reused
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r][slot] = czero<C>();
            return;
        }
        const int m = zs + it - P;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int gy = y0 + ty * R + r;
            if (gx < n0 && gy < n1) {
                const size_t e = ((size_t)m * n1 + gy) * n0 + gx;
                MC v;
                if (prm.sub) {
                    if constexpr (std::is_same<T, float>::value && IsF64Mem<MC>::v) {
                        // FP32 arithmetic on FP64 vectors: b - A x formed in FP64 (exact
                        // operands, one rounding), so the stored residual keeps b's bits
                        const double2 o = rb_store<MC, C>(acc[r][slot]);
                        v = make_double2(sv[r].x - o.x, sv[r].y - o.y);
                    } else {
                        v = rb_store<MC, C>(rb_sub<C, MC>(sv[r], acc[r][slot]));
                    }
                } else {
                    v = rb_store<MC, C>(acc[r][slot]);
                }
                Y[e] = v;
                if (prm.red_mode) {
                    if constexpr (std::is_same<T, float>::value) {
                        if (!prm.sub) {
                            // FP32 arithmetic: the run's partial sum in FP32 (its own error is
                            // below the apply's), off GB300's FP64 pipe
                            const float2 a = acc[r][slot];
                            if (prm.red_mode == 1) {
                                facc.x = fmaf(a.x, a.x, fmaf(a.y, a.y, facc.x));
                            } else {
                                const float2 d = rb_load<float2, MC>(sv[r]);
                                facc.x = fmaf(d.x, a.x, fmaf(d.y, a.y, facc.x));
                                facc.y = fmaf(d.x, a.y, fmaf(-d.y, a.x, facc.y));
                            }
                            acc[r][slot] = czero<C>();
                            continue;
                        }
                    }
                    if (prm.red_mode == 1) {
                        racc.x = fma((double)v.x, (double)v.x, fma((double)v.y, (double)v.y, racc.x));
                    } else {
                        const MC d = prm.sub ? static_cast<const MC *>(prm.dotv)[e] : sv[r];
                        racc.x = fma((double)d.x, (double)v.x, fma((double)d.y, (double)v.y, racc.x));
                        racc.y = fma((double)d.x, (double)v.y, fma(-(double)d.y, (double)v.x, racc.y));
                    }
                }
            }
            acc[r][slot] = czero<C>();
        }
    };

    if constexpr (kShiftRing<T>) {
        // double-float: one copy of the step, the ring shifts down by one slot per plane
#pragma unroll 1
        for (int it = 0; it < nplanes; ++it) {
            MC sv[R];
            side_load(it, sv);
            if (it >= lo && it < hi) step(it, 0);
            finish(it, 0, sv);
#pragma unroll
            for (int r = 0; r < R; ++r) {
#pragma unroll
                for (int s = 0; s + 1 < BW; ++s) acc[r][s] = acc[r][s + 1];
                acc[r][BW - 1] = czero<C>();
            }
        }
    } else {
        // FP32: the plane loop unrolled by the ring length, fixed slots
        for (int base = 0; base < nplanes; base += BW) {
#pragma unroll
            for (int ph = 0; ph < BW; ++ph) {
                const int it = base + ph;
                if (it >= nplanes) break;
                const int ring = (ph - P + 2 * BW) % BW;
                MC sv[R];
                side_load(it, sv);
                if (it >= lo && it < hi) step(it, ring);
                finish(it, ring, sv);
            }
        }
    }
    if constexpr (!Sh::kTma) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    racc.x += (double)facc.x;
    racc.y += (double)facc.y;
    return racc;
}

// Persistent CTAs over the (tile, z) order, z fastest: CTA b owns planes
// [b L, (b + 1) L) (L = prm.zchunk), in one or more runs of one tile each.
template <class T, class MC, int P, bool HB, bool HC, int NTY, int R, int KA, int KC>
__global__ void __launch_bounds__(kRbTX *NTY, RbMinBlocks<T>::v)
    k_apply3d_rb(const __grid_constant__ ApplyParams<T> prm, const __grid_constant__ CUtensorMap xmap) {
    using Sh = RbShape<T, MC, P, HB, HC, NTY, R>;
    extern __shared__ __align__(128) unsigned char rb_dyn[];
    unsigned char *rb_raw = rb_dyn + ((128u - (rb_smem(rb_dyn) & 127u)) & 127u);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(rb_raw);
    const int txw = blockDim.x;
    const int tid = threadIdx.y * txw + threadIdx.x;
    if constexpr (Sh::kTma) {
        if (tid == 0) {
            for (int b = 0; b < 3; ++b)
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(rb_smem(&mbar[b])), "r"(1) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        // the first run's barriers (before its staging) order the init before any use
    }
    const int n0 = prm.n0, n1 = prm.n1, n2 = prm.n2;
    const int tilesX = (n0 + txw - 1) / txw;
    const long long total = (long long)tilesX * ((n1 + Sh::TY - 1) / Sh::TY) * n2;
    long long pos = (long long)blockIdx.x * prm.zchunk;
    const long long end = min(total, pos + prm.zchunk);
    double2 racc = make_double2(0.0, 0.0);
    uint32_t par = 0;
    bool dead = false;
    for (; pos < end;) {
        const int t = (int)(pos / n2);
        const int z0 = (int)(pos - (long long)t * n2);
        const int z1 = (int)min((long long)n2, z0 + (end - pos));
        pos += z1 - z0;
        __syncthreads();   // the last run's readers of the shared buffers are done
        const double2 r = rb_run<T, MC, P, HB, HC, NTY, R, KA, KC>(prm, &xmap, (t % tilesX) * txw,
                                                                   (t / tilesX) * Sh::TY, z0, z1, par, dead);
        racc.x += r.x;
        racc.y += r.y;
    }
    if (prm.red_mode) {   // CTA sum -> red[blockIdx.x] (fixed order: deterministic)
        __shared__ double2 wsum[32];
        for (int off = 16; off > 0; off >>= 1) {
            racc.x += __shfl_down_sync(0xffffffffu, racc.x, off);
            racc.y += __shfl_down_sync(0xffffffffu, racc.y, off);
        }
        const int nw = (txw * NTY + 31) / 32;
        if ((tid & 31) == 0) wsum[tid >> 5] = racc;
        __syncthreads();
        if (tid == 0) {
            double2 s = make_double2(0.0, 0.0);
            for (int w = 0; w < nw; ++w) { s.x += wsum[w].x; s.y += wsum[w].y; }
            prm.red[blockIdx.x] = s;
        }
    }
}

// ---------------------------------------------------------------- launcher
// TMA map of an FP64 vector: FP64 values, dims (2 n0, n1, n2), box
// (2 (32 + 2p), TY + 2p, 1), zero fill outside the grid (apply.cu)
void rb_make_map(CUtensorMap *map, const void *x, int n0, int n1, int n2, int boxx, int boxy);

template <class T, class MC, int P, bool HB, bool HC, int KA = 0, int KC = 0>
inline void run3d_rb(const ApplyParams<T> &prm0, cudaStream_t st) {
    constexpr int NTY = std::is_same<T, float>::value ? 8 : 16;
    constexpr int R = std::is_same<T, float>::value ? 2 : 1;
    using Sh = RbShape<T, MC, P, HB, HC, NTY, R>;
    auto kern = k_apply3d_rb<T, MC, P, HB, HC, NTY, R, KA, KC>;
    constexpr size_t kMaxDyn = 220 * 1024;
    static const int nsm = [&] {   // once per instantiation (thread-safe static initialisation)
        TDZ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDyn));
        return sm_count();
    }();
    const int n2 = prm0.n2;
    TDZ_CHECK(Sh::smem(n2 + 2 * P) <= kMaxDyn, TDZ_ERR_UNSUPPORTED, "outer axis too long for the 3D apply");
    thread_local int occ_n2 = -1, occ_slots = 0;
    thread_local const void *occ_k = nullptr;
    if (occ_n2 != n2 || occ_k != reinterpret_cast<const void *>(kern)) {
        int per_sm = 0;
        TDZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRbTX * NTY, Sh::smem(n2 + 2 * P)));
        occ_slots = std::max(1, per_sm) * nsm;
        occ_n2 = n2;
        occ_k = reinterpret_cast<const void *>(kern);
    }
    const int slots = occ_slots;
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    if constexpr (Sh::kTma) {
        TDZ_CHECK(reinterpret_cast<uintptr_t>(prm0.x) % 16 == 0, TDZ_ERR_ARG, "FP64 vectors must be 16-byte aligned");
        rb_make_map(&map, prm0.x, prm0.n0, prm0.n1, n2, 2 * Sh::RX, Sh::RY);
    }
    auto tiles_for = [&](int txw) { return ((prm0.n0 + txw - 1) / txw) * ((prm0.n1 + Sh::TY - 1) / Sh::TY); };
    auto seg_for = [&](int txw, long long g) {
        const long long total = (long long)tiles_for(txw) * n2;
        return (int)std::min<long long>(total, std::max<long long>(4 * P, (total + g - 1) / g));
    };
    auto launch = [&](int txw, int seg, bool candidate = false) {
        ApplyParams<T> prm = prm0;
        const long long total = (long long)tiles_for(txw) * n2;
        if (candidate) prm.red_mode = 0;
        if (prm.red_mode) seg = (int)std::max<long long>(seg, (total + kApplyRedCap - 1) / kApplyRedCap);
        prm.zchunk = seg;
        prm.zchunk_planes = std::min(seg, n2) + 2 * P;
        const unsigned grid = (unsigned)((total + seg - 1) / seg);
        const size_t smem = Sh::smem(prm.zchunk_planes);
        TDZ_CHECK(smem <= kMaxDyn, TDZ_ERR_UNSUPPORTED, "outer axis too long for the 3D apply");
        kern<<<grid, dim3(txw, NTY), smem, st>>>(prm, map);
    };
    int txw = kRbTX;
    int zchunk = seg_for(txw, (long long)slots * 2);
    const TuneKey key{reinterpret_cast<const void *>(kern), prm0.n0, prm0.n1, prm0.n2};
    if (forced_shape(&txw, &zchunk)) {
        txw = std::max(16, std::min(kRbTX, txw / 4 * 4));
        zchunk = std::max(4 * P, zchunk);
    } else if (autotune_enabled() && !tune_lookup(key, &txw, &zchunk)) {
        std::vector<std::pair<int, int>> cand;
        for (int t = kRbTX; t >= 16; t -= 4) {
            if ((prm0.n0 + t - 1) / t * t > (prm0.n0 + kRbTX - 1) / kRbTX * kRbTX) continue;
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
                std::fprintf(stderr, "tdz autotune apply3d_rb<%s,%s,p%d,B%d,C%d,%d%d> %dx%dx%d: tile %dx%d run %d: %.1f us\n",
                             sizeof(T) == 4 ? "f32" : "df", IsF64Mem<MC>::v ? "m64" : "m32", P, (int)HB, (int)HC, KA,
                             KC, prm0.n0, prm0.n1, n2, c.first, Sh::TY, c.second, 500.f * ms);
            if (ms < best) { best = ms; txw = c.first; zchunk = c.second; }
        }
        TDZ_CUDA(cudaEventDestroy(e0));
        TDZ_CUDA(cudaEventDestroy(e1));
        tune_store(key, txw, zchunk);
    }
    launch(txw, zchunk);
}

// ---------------------------------------------------------------- dispatch
// 3D: the register-blocked kernel for FP32 and double-float arithmetic (with
// compile-time outer-combination kinds for the CN stage, KC = 2, and the
// mass, KA = 1), the plane-ring kernel of apply_kernels.cuh for native FP64;
// 2D: the row-tile kernel.
template <class T, class MC, int P>
inline void dispatch_rb(bool hb, bool hc, const ApplyParams<T> &prm, cudaStream_t st) {
    if (!hb && hc && prm.zc_kind == 2) { run3d_rb<T, MC, P, false, true, 0, 2>(prm, st); return; }   // CN stage
    if (!hb && !hc && prm.za_kind == 1) { run3d_rb<T, MC, P, false, false, 1, 0>(prm, st); return; }  // mass
    if (hb && hc) run3d_rb<T, MC, P, true, true>(prm, st);
    else if (hb) run3d_rb<T, MC, P, true, false>(prm, st);
    else if (hc) run3d_rb<T, MC, P, false, true>(prm, st);
    else run3d_rb<T, MC, P, false, false>(prm, st);
}

template <class T, int P>
inline void dispatch_streams(int dim, bool hb, bool hc, const ApplyParams<T> &prm, cudaStream_t st,
                             bool m64 = false) {
    if (dim == 3) {
        if constexpr (std::is_same<T, double>::value) {
            if (hb && hc) run3d<T, P, true, true>(prm, st);
            else if (hb) run3d<T, P, true, false>(prm, st);
            else if (hc) run3d<T, P, false, true>(prm, st);
            else run3d<T, P, false, false>(prm, st);
        } else if constexpr (std::is_same<T, float>::value) {
            if (m64) dispatch_rb<float, double2, P>(hb, hc, prm, st);
            else dispatch_rb<float, float2, P>(hb, hc, prm, st);
        } else {
            dispatch_rb<dff, double2, P>(hb, hc, prm, st);
        }
    } else {
        if (hb && hc) run2d<T, P, true, true>(prm, st);
        else if (hb) run2d<T, P, true, false>(prm, st);
        else if (hc) run2d<T, P, false, true>(prm, st);
        else run2d<T, P, false, false>(prm, st);
    }
}

}  // namespace tdz
