// Complex helpers on float2 / double2 (device). Internal.
#pragma once
#include <cuda_runtime.h>

namespace tdz {

template <class T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };

template <class C> __device__ __forceinline__ C czero() { C c; c.x = 0; c.y = 0; return c; }
template <class T, class C> __device__ __forceinline__ void rfma(C &acc, T a, C v) {
    acc.x = fma(a, v.x, acc.x);
    acc.y = fma(a, v.y, acc.y);
}
template <class C> __device__ __forceinline__ void cfma(C &acc, C a, C v) {
    acc.x = fma(a.x, v.x, acc.x);
    acc.x = fma(-a.y, v.y, acc.x);
    acc.y = fma(a.x, v.y, acc.y);
    acc.y = fma(a.y, v.x, acc.y);
}
// acc += conj(a) v
template <class C> __device__ __forceinline__ void cfma_conj(C &acc, C a, C v) {
    acc.x = fma(a.x, v.x, acc.x);
    acc.x = fma(a.y, v.y, acc.x);
    acc.y = fma(a.x, v.y, acc.y);
    acc.y = fma(-a.y, v.x, acc.y);
}

}  // namespace tdz
