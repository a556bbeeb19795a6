// Device vector operations on interleaved complex arrays (FP32 / FP64), with
// deterministic FP64 reductions. Internal to the tdz library.
#pragma once

#include "common.h"

namespace tdz {
namespace blas {

constexpr int kMaxDot = 16;   // vectors per fused multi-dot / multi-axpy pass

// y = x
void copy(const void *x, void *y, size_t n, int prec, cudaStream_t st);
// x = 0
void zero(void *x, size_t n, int prec, cudaStream_t st);
// x *= a
void scale(void *x, cd a, size_t n, int prec, cudaStream_t st);
// y = a x + b y
void axpby(void *y, cd a, const void *x, cd b, size_t n, int prec, cudaStream_t st);
// y = a x + b y + c z
void axpbypcz(void *y, cd a, const void *x, cd b, const void *z, cd c, size_t n, int prec, cudaStream_t st);
// y (precision py) = x (precision px)
void cast(const void *x, int px, void *y, int py, size_t n, cudaStream_t st);
// x <- Re(x) (FP64: imaginary parts set to zero)
void keep_real(void *x, size_t n, cudaStream_t st);
// y64 += a * x32 (FP32 correction added to an FP64 vector)
void add_cast(double2 *y, cd a, const float2 *x, size_t n, cudaStream_t st);

// Reduction workspace: per-block partial sums and device results.
struct Reducer {
    DevBuf partial;   // [kMaxDot + 1][blocks] double2
    DevBuf result;    // [kMaxDot + 1] double2
    DevBuf hostbuf;   // pinned host mirror of result
    double2 *host = nullptr;
    int blocks = 0;
    void init();
    ~Reducer();
};

// out[i] = <V_i, w> = sum conj(V_i) w for i < k (any k; chunks of kMaxDot),
// precision prec; results copied to the host (synchronises the stream).
void mdot(Reducer &r, const void *const *V, int k, const void *w, size_t n, int prec, cd *out, cudaStream_t st);
// out (device double2) = <x, y> with scratch partials r.partial (no host sync)
void dot_device(Reducer &r, const void *x, const void *y, size_t n, int prec, double2 *out, cudaStream_t st);
// out[i] = <V_i, w> for i < k <= kMaxDot into device memory, per-block
// partials in the given scratch (blocks * k double2), no host sync
void mdot_partials(const void *const *V, int k, const void *w, size_t n, int prec, double2 *partial, int blocks,
                   double2 *out, cudaStream_t st);
constexpr int kRedBlocksPublic = 2 * 152;   // blocks of the reductions (partials per dot product)
// w += sum_i a_i V_i
void maxpy(void *w, int k, const void *const *V, const cd *a, size_t n, int prec, cudaStream_t st);
// FP64 psi = 2 x - psi + c z (Crank-Nicolson update with the last Krylov correction)
void cn_combine(void *psi, const void *x, const void *z, cd c, size_t n, cudaStream_t st);
// ||x||_2 (synchronises)
double nrm2(Reducer &r, const void *x, size_t n, int prec, cudaStream_t st);
// FP64 Arnoldi vector, fused Gram-Schmidt pass (k <= 16): w += sum_i a_i V_i,
// then dots[i] = <V_i, w> and / or *norm = ||w|| from the same pass
void gs_update(Reducer &r, void *w, int k, const void *const *V, const cd *a, size_t n, cd *dots, double *norm,
               cudaStream_t st);

}  // namespace blas

// tdz_vec_mdot with the partial sums in the library's static device array
// (noalloc.cu): k <= 8, no device allocation.
void mdot_noalloc(const void *const *V, int k, const void *w, size_t n, int prec, double2 *out, cudaStream_t st);

}  // namespace tdz
