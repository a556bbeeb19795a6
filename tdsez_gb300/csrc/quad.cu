// Non-separable soft-core potential term by per-element quadrature (quad.h).
// One CTA per element: gather the (p+1)^d coefficients, interpolate to the
// Q^d Gauss points axis by axis (sum factorisation, shared memory ping-pong),
// multiply by w V with V from the closed form, project back axis by axis and
// add coef * result to y with atomics (neighbouring elements share
// coefficients). Work per element 2 d Q (p+1)^d (d-dimensional sum
// factorisation): the per-element tensor-contraction flops of this term.
#include "quad.h"

#include <cmath>

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
    for (int d = 0; d < dim; ++d) {
        const Axis1D &a = s.ax[d];
        TDZ_CHECK(a.nq == nq && a.p == p, TDZ_ERR_INTERNAL, "axis tables disagree");
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
