// Complex helpers on float2 / double2 (device). Internal.
#pragma once
#include <cuda_runtime.h>

namespace tdz {

// Double-float: a value hi + lo carried as two FP32 numbers (about 48
// significant bits; Dekker 1971, as in the double-double arithmetic of Hida,
// Li and Bailey 2001 with single-precision halves). The product a.hi b.hi is
// split exactly with an fma residual, the sum uses Knuth's two-sum error term.
// Accumulations skip the per-term renormalisation: lo collects the product
// and rounding errors of a whole banded sum (a few dozen terms, so it stays
// far below hi's last bit times the term count) and renorm() folds it into
// hi once per stage result. Every step is an explicitly rounded intrinsic, so
// the compiler cannot contract or reorder it. Relative error near 1e-14 on
// the FP32 pipes, which on this GPU run at 64x the FP64 rate.
struct dff {
    float hi, lo;
    dff() = default;
    __host__ __device__ constexpr dff(float v) : hi(v), lo(0.f) {}
    __host__ __device__ constexpr dff(float h, float l) : hi(h), lo(l) {}
};
struct cdff {
    dff x, y;
};
__device__ __forceinline__ dff operator-(dff a) { return dff(-a.hi, -a.lo); }
// a * b + c in the arithmetic type of the operands
__device__ __forceinline__ float tfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double tfma(double a, double b, double c) { return ::fma(a, b, c); }
// double-float, unnormalised result (12 FP32 instructions)
__device__ __forceinline__ dff tfma(dff a, dff b, dff c) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float s = __fadd_rn(c.hi, p);
    const float bv = __fsub_rn(s, c.hi);
    const float err = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
    return dff(s, __fadd_rn(__fadd_rn(c.lo, e), err));
}
// fold lo into hi (fast two-sum; |lo| <= |hi| for an accumulated value)
__device__ __forceinline__ dff renorm(dff a) {
    const float h = __fadd_rn(a.hi, a.lo);
    return dff(h, __fsub_rn(a.lo, __fsub_rn(h, a.hi)));
}
__host__ __device__ inline dff dff_from(double v) {
    const float h = (float)v;
    return dff(h, (float)(v - (double)h));
}

// FP64 -> double-float split with integer operations only (GB300's FP64 pipe,
// which also executes FP64 <-> FP32 conversions, issues 2 instructions per
// clock per SM). hi = v truncated to 24 significant bits, lo = the next 24
// bits (truncated), so hi + lo carries 48 bits. |v| < 2^-100 (and zero,
// subnormals) maps to 0; Inf/NaN and |v| >= 2^128 map to a non-finite hi.
__device__ __forceinline__ dff dff_split(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const unsigned int h32 = (unsigned int)(u >> 32), l32 = (unsigned int)u;
    const unsigned int sign = h32 & 0x80000000u;
    const int e = (int)((h32 >> 20) & 0x7FFu) - 1023;
    if (e < -100) return dff(__uint_as_float(sign), 0.f);
    if (e > 127) return dff(__uint_as_float(sign | (e == 1024 && ((h32 & 0xFFFFFu) | l32) ? 0x7FC00000u : 0x7F800000u)), 0.f);
    const unsigned int m23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
    const float hi = __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | m23);
    const unsigned int m29 = l32 & 0x1FFFFFFFu;
    if (m29 == 0u) return dff(hi, 0.f);
    const int lz = __clz((int)m29);                 // >= 3
    const int el = e - 52 + 31 - lz;                // exponent of the leading remainder bit
    if (el < -126) return dff(hi, 0.f);
    const unsigned int frac = (m29 << (lz + 1)) >> 9;
    return dff(hi, __uint_as_float(sign | ((unsigned int)(el + 127) << 23) | frac));
}
// exact FP32 -> FP64 widening with integer operations (normal values; zero and
// subnormals give signed zero, Inf/NaN stay non-finite)
__device__ __forceinline__ double f2d_exact(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int ex = (b >> 23) & 0xFFu;
    unsigned long long d = (unsigned long long)(b & 0x80000000u) << 32;
    if (ex == 0xFFu) d |= 0x7FF0000000000000ull | ((unsigned long long)(b & 0x7FFFFFu) << 29);
    else if (ex != 0u) d |= ((unsigned long long)(ex - 127 + 1023) << 52) | ((unsigned long long)(b & 0x7FFFFFu) << 29);
    return __longlong_as_double((long long)d);
}
// hi + lo rounded to FP64: one FP64 add
__device__ __forceinline__ double dff_to_double(dff a) { return f2d_exact(a.hi) + f2d_exact(a.lo); }

template <class T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };
template <> struct CT<dff> { using type = cdff; };

// complex type in memory for each arithmetic type
template <class T> struct MemC { using type = typename CT<T>::type; };
template <> struct MemC<dff> { using type = double2; };
template <class C, class M> __device__ __forceinline__ C load_c(const M &m) { return m; }
template <> __device__ __forceinline__ cdff load_c<cdff, double2>(const double2 &m) {
    cdff c;
    c.x = dff_split(m.x);
    c.y = dff_split(m.y);
    return c;
}
template <class M, class C> __device__ __forceinline__ M store_c(const C &c) { return c; }
template <> __device__ __forceinline__ double2 store_c<double2, cdff>(const cdff &c) {
    return make_double2(dff_to_double(c.x), dff_to_double(c.y));
}

template <class C> __device__ __forceinline__ C czero() { C c; c.x = 0; c.y = 0; return c; }
// renormalise a stage result (identity for native types)
template <class C> __device__ __forceinline__ C cnorm(const C &c) { return c; }
template <> __device__ __forceinline__ cdff cnorm<cdff>(const cdff &c) {
    cdff r;
    r.x = renorm(c.x);
    r.y = renorm(c.y);
    return r;
}
template <class T, class C> __device__ __forceinline__ void rfma(C &acc, T a, C v) {
    acc.x = tfma(a, v.x, acc.x);
    acc.y = tfma(a, v.y, acc.y);
}
template <class C> __device__ __forceinline__ void cfma(C &acc, C a, C v) {
    acc.x = tfma(a.x, v.x, acc.x);
    acc.x = tfma(-a.y, v.y, acc.x);
    acc.y = tfma(a.x, v.y, acc.y);
    acc.y = tfma(a.y, v.x, acc.y);
}
// acc += i b v (b real: the imaginary part of a purely imaginary coefficient)
template <class T, class C> __device__ __forceinline__ void ifma(C &acc, T b, C v) {
    acc.x = tfma(-b, v.y, acc.x);
    acc.y = tfma(b, v.x, acc.y);
}
// acc += a v with a of a known kind: 0 complex, 1 real, 2 imaginary
template <class C> __device__ __forceinline__ void kfma(C &acc, C a, C v, int kind) {
    if (kind == 1) rfma(acc, a.x, v);
    else if (kind == 2) ifma(acc, a.y, v);
    else cfma(acc, a, v);
}
// acc += conj(a) v
template <class C> __device__ __forceinline__ void cfma_conj(C &acc, C a, C v) {
    acc.x = tfma(a.x, v.x, acc.x);
    acc.x = tfma(a.y, v.y, acc.x);
    acc.y = tfma(a.x, v.y, acc.y);
    acc.y = tfma(-a.y, v.x, acc.y);
}

}  // namespace tdz
