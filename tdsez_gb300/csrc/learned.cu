// Learned coarse correction of the multigrid V-cycle (mg.h, LearnedCoarse).
//
// The coarsest level of the V-cycle is solved by a Chebyshev polynomial
// (the reference factorises it with MUMPS, src/multigrid.cpp:315-324, which
// has no GPU counterpart here). The network corrects that solve:
//   x = x0 + c rms(r) N(r / rms(r)),  r = b_c - A_c x0,  c = mean ||e|| / ||r||,
// N a 3D CNN (cnn.cu: 3x3x3 convolutions, BF16 weights, FP32 accumulation)
// on the coarsest grid with the real and imaginary parts as channels. The
// training pairs (r / rms(r), e / (c rms(r))), e = A_c^-1 r, come from the
// solver itself: random coarse right-hand sides, the production Chebyshev
// solve, and a 10x longer Chebyshev solve for e. Everything stays on the
// device in the V-cycle (rms(r) is a device scalar), so the corrected cycle
// needs no host synchronisation.
#include <cmath>
#include <random>

#include "cplx.cuh"
#include "mg.h"

namespace tdz {

namespace {

// s = sqrt(sum |r|^2) (one block)
__global__ void k_norm_one(const float2 *r, int n, float *s) {
    __shared__ float red[256];
    float a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += r[i].x * r[i].x + r[i].y * r[i].y;
    red[threadIdx.x] = a;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *s = sqrtf(red[0]);
}

// planar [2][n] = r / rms(r) (unit-RMS network input; 0 when r = 0)
__global__ void k_pack(const float2 *r, int n, const float *s, float *out) {
    const float inv = *s > 0.f ? sqrtf(2.f * n) / *s : 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[i] = r[i].x * inv;
        out[n + i] = r[i].y * inv;
    }
}

// x += rms(r) c (out[0] + i out[1])
__global__ void k_unpack_add(float2 *x, int n, const float *s, float c, const float *out) {
    const float sc = *s * c / sqrtf(2.f * n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i].x += sc * out[i];
        x[i].y += sc * out[n + i];
    }
}

// training pair: in = r / rms(r), target = e / (rms(r) c)
__global__ void k_pack_pair(const float2 *r, const float2 *e, int n, float in_scale, float tgt_scale, float *in,
                            float *tgt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        in[i] = r[i].x * in_scale;
        in[n + i] = r[i].y * in_scale;
        tgt[i] = e[i].x * tgt_scale;
        tgt[n + i] = e[i].y * tgt_scale;
    }
}

inline int blocks_for(int n) { return std::max(1, std::min((n + 255) / 256, 1024)); }

void random_rhs(DevBuf &b, size_t n, std::mt19937_64 &rng, cudaStream_t st) {
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> h(2 * n);
    for (float &v : h) v = nd(rng);
    TDZ_CUDA(cudaMemcpyAsync(b.ptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
}

double norm_host(const DevBuf &v, size_t n, cudaStream_t st) {
    std::vector<float> h(2 * n);
    TDZ_CUDA(cudaMemcpyAsync(h.data(), v.ptr, h.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (float x : h) s += (double)x * x;
    return std::sqrt(s);
}

}  // namespace

void Multigrid::learned_setup() {
    lrn.on = prec == TDZ_FP32;
    if (!lrn.on) return;
    MGLevel &m = lv.back();
    const int D = m.space.dim == 3 ? m.n[2] : 1;
    const int H = m.space.dim >= 2 ? m.n[1] : 1;
    const int W = m.n[0];
    lrn.net.init(2, lrn.width, 2, lrn.layers, D, H, W, lrn.batch, 20261203ull);
    lrn.in.alloc(2 * m.ndof * sizeof(float));
    lrn.out.alloc(2 * m.ndof * sizeof(float));
    lrn.scale.alloc(sizeof(float));
}

void Multigrid::coarse_correct(MGLevel &m, cudaStream_t st) {
    const int n = (int)m.ndof;
    // r = b - A x0
    m.opp->apply(TDZ_STAGE, TDZ_FP32, m.x.ptr, m.t1.ptr, st);
    blas::axpbypcz(m.r.ptr, 1.0, m.b.ptr, 0.0, m.t1.ptr, -1.0, m.ndof, TDZ_FP32, st);
    k_norm_one<<<1, 256, 0, st>>>(m.r.as<float2>(), n, lrn.scale.as<float>());
    k_pack<<<blocks_for(n), 256, 0, st>>>(m.r.as<float2>(), n, lrn.scale.as<float>(), lrn.in.as<float>());
    lrn.net.forward(lrn.in.as<float>(), lrn.out.as<float>(), 1, st, false);
    k_unpack_add<<<blocks_for(n), 256, 0, st>>>(m.x.as<float2>(), n, lrn.scale.as<float>(), lrn.cscale,
                                                lrn.out.as<float>());
    TDZ_CUDA(cudaGetLastError());
    count_launch(3);
}

void Multigrid::record_coarse(int capacity) {
    TDZ_CHECK(lrn.on, TDZ_ERR_STATE, "the learned coarse correction needs mg_learned and FP32 levels");
    TDZ_CHECK(capacity >= 0, TDZ_ERR_ARG, "negative capacity");
    if (capacity == 0) { lrn.rec_cap = lrn.rec_n; return; }
    lrn.rec.alloc((size_t)capacity * lv.back().ndof * sizeof(float2));
    lrn.rec_cap = capacity;
    lrn.rec_n = 0;
}

float Multigrid::train_recorded(int epochs, float lr, uint64_t seed, cudaStream_t st) {
    TDZ_CHECK(lrn.on, TDZ_ERR_STATE, "the learned coarse correction needs mg_learned and FP32 levels");
    TDZ_CHECK(lrn.rec_n >= lrn.batch, TDZ_ERR_STATE,
              "fewer recorded coarse right-hand sides than one training batch (record_coarse, then run steps)");
    const int pairs = lrn.rec_n / lrn.batch * lrn.batch;
    lrn.use_recorded = true;
    const float l = train_coarse(pairs, epochs, lr, seed, st);
    lrn.use_recorded = false;
    return l;
}

float Multigrid::train_coarse(int pairs, int epochs, float lr, uint64_t seed, cudaStream_t st) {
    TDZ_CHECK(lrn.on, TDZ_ERR_STATE, "the learned coarse correction needs mg_learned and FP32 levels");
    TDZ_CHECK(pairs >= lrn.batch && epochs >= 1, TDZ_ERR_ARG, "need at least one batch of pairs and one epoch");
    for (size_t l = 1; l < lv.size(); ++l) lv[l].opp->sigma = fine->sigma;
    MGLevel &m = lv.back();
    const int n = (int)m.ndof;
    const size_t per = 2 * (size_t)n;
    if (lrn.npairs < pairs) {
        lrn.pin.alloc((size_t)pairs * per * sizeof(float));
        lrn.ptgt.alloc((size_t)pairs * per * sizeof(float));
    }
    lrn.npairs = pairs;
    std::mt19937_64 rng(seed);
    DevBuf x0(m.ndof * sizeof(float2)), r(m.ndof * sizeof(float2));
    const double root = std::sqrt(2.0 * n);
    double ratio_sum = 0.0;
    for (int k = 0; k < pairs; ++k) {
        if (lrn.use_recorded)   // a coarse right-hand side of the run's own V-cycles
            blas::copy(lrn.rec.as<float2>() + (size_t)k * m.ndof, m.b.ptr, m.ndof, TDZ_FP32, st);
        else
            random_rhs(m.b, m.ndof, rng, st);
        chebyshev(m, TDZ_FP32, m.mu_lo, m.mu_hi, m.w_max, opt.coarse_its, true, st);   // production solve
        blas::copy(m.x.ptr, x0.ptr, m.ndof, TDZ_FP32, st);
        m.opp->apply(TDZ_STAGE, TDZ_FP32, x0.ptr, m.t1.ptr, st);
        blas::axpbypcz(r.ptr, 1.0, m.b.ptr, 0.0, m.t1.ptr, -1.0, m.ndof, TDZ_FP32, st);   // r = b - A x0
        blas::copy(r.ptr, m.b.ptr, m.ndof, TDZ_FP32, st);
        chebyshev(m, TDZ_FP32, m.mu_lo, m.mu_hi, m.w_max, 10 * opt.coarse_its, true, st);   // e = A^-1 r
        const double s = norm_host(r, m.ndof, st), se = norm_host(m.x, m.ndof, st);
        // global target scale c = mean ||e|| / ||r|| over the first pairs, so targets are O(1) too
        if (k < 32) {
            ratio_sum += s > 0.0 ? se / s : 0.0;
            lrn.cscale = (float)std::max(ratio_sum / (k + 1), 1e-30);
        }
        const float in_scale = s > 0.0 ? (float)(root / s) : 0.f;
        k_pack_pair<<<blocks_for(n), 256, 0, st>>>(r.as<float2>(), m.x.as<float2>(), n, in_scale,
                                                  in_scale / lrn.cscale, lrn.pin.as<float>() + (size_t)k * per,
                                                  lrn.ptgt.as<float>() + (size_t)k * per);
        TDZ_CUDA(cudaGetLastError());
    }
    lrn.net.read_loss(st);   // reset the accumulator
    const int nb = pairs / lrn.batch;
    float last = 0.f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int b = 0; b < nb; ++b)
            lrn.net.train_step(lrn.pin.as<float>() + (size_t)b * lrn.batch * per,
                               lrn.ptgt.as<float>() + (size_t)b * lrn.batch * per, lrn.batch, lr, st);
        last = lrn.net.read_loss(st) / nb;
    }
    lrn.trained = true;
    return last;
}

std::pair<double, double> Multigrid::coarse_gain(int trials, uint64_t seed, cudaStream_t st) {
    TDZ_CHECK(lrn.on && lrn.trained, TDZ_ERR_STATE, "the learned coarse correction is not trained");
    for (size_t l = 1; l < lv.size(); ++l) lv[l].opp->sigma = fine->sigma;
    MGLevel &m = lv.back();
    std::mt19937_64 rng(seed);
    DevBuf b(m.ndof * sizeof(float2)), e(m.ndof * sizeof(float2)), c(m.ndof * sizeof(float2));
    double plain = 0.0, learned = 0.0;
    for (int k = 0; k < trials; ++k) {
        random_rhs(b, m.ndof, rng, st);
        blas::copy(b.ptr, m.b.ptr, m.ndof, TDZ_FP32, st);
        chebyshev(m, TDZ_FP32, m.mu_lo, m.mu_hi, m.w_max, 10 * opt.coarse_its, true, st);
        blas::copy(m.x.ptr, e.ptr, m.ndof, TDZ_FP32, st);               // reference solution
        const double en = norm_host(e, m.ndof, st);
        blas::copy(b.ptr, m.b.ptr, m.ndof, TDZ_FP32, st);
        chebyshev(m, TDZ_FP32, m.mu_lo, m.mu_hi, m.w_max, opt.coarse_its, true, st);
        blas::axpbypcz(c.ptr, 1.0, e.ptr, 0.0, m.x.ptr, -1.0, m.ndof, TDZ_FP32, st);
        plain += norm_host(c, m.ndof, st) / en;
        coarse_correct(m, st);
        blas::axpbypcz(c.ptr, 1.0, e.ptr, 0.0, m.x.ptr, -1.0, m.ndof, TDZ_FP32, st);
        learned += norm_host(c, m.ndof, st) / en;
    }
    return {plain / trials, learned / trials};
}

}  // namespace tdz
