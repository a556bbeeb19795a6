// Learned coarse correction network: 3x3x3 convolutions (zero padding) with
// ReLU between layers, BF16 weights and FP32 accumulation, trained on the GPU
// by hand-written backward kernels and Adam. Layout: [batch][channel][D][H][W].
#include "cnn.h"

#include <cuda_bf16.h>

#include <cmath>
#include <random>

namespace tdz {

namespace {

constexpr int TB = 8;          // spatial tile edge (TB^3 threads)
constexpr int CC = 4;          // input channels per shared-memory chunk
constexpr int MAXC = 32;       // max output channels per launch

// out[b][co][p] = bias[co] + sum_ci sum_k W[co][ci][k] in[b][ci][p + k - 1]
__global__ void __launch_bounds__(TB *TB *TB) k_conv_fwd(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ Wt,
                                                          const float *__restrict__ bias, float *__restrict__ out,
                                                          int Ci, int Co, int D, int H, int W, int relu) {
    __shared__ float tile[CC][TB + 2][TB + 2][TB + 2];
    __shared__ float wsm[MAXC][CC][27];
    const int tx = threadIdx.x % TB, ty = (threadIdx.x / TB) % TB, tz = threadIdx.x / (TB * TB);
    const int tilesX = (W + TB - 1) / TB, tilesY = (H + TB - 1) / TB;
    const int bx = blockIdx.x % tilesX, by = (blockIdx.x / tilesX) % tilesY, bz = blockIdx.x / (tilesX * tilesY);
    const int x0 = bx * TB, y0 = by * TB, z0 = bz * TB;
    const int b = blockIdx.y;
    const size_t N = (size_t)D * H * W;
    float acc[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) acc[c] = 0.f;
    for (int c0 = 0; c0 < Ci; c0 += CC) {
        __syncthreads();
        const int nc = min(CC, Ci - c0);
        for (int i = threadIdx.x; i < CC * (TB + 2) * (TB + 2) * (TB + 2); i += blockDim.x) {
            const int c = i / ((TB + 2) * (TB + 2) * (TB + 2));
            const int r = i % ((TB + 2) * (TB + 2) * (TB + 2));
            const int lz = r / ((TB + 2) * (TB + 2)), ly = (r / (TB + 2)) % (TB + 2), lx = r % (TB + 2);
            const int z = z0 + lz - 1, y = y0 + ly - 1, x = x0 + lx - 1;
            float v = 0.f;
            if (c < nc && z >= 0 && z < D && y >= 0 && y < H && x >= 0 && x < W)
                v = in[((size_t)b * Ci + c0 + c) * N + ((size_t)z * H + y) * W + x];
            tile[c][lz][ly][lx] = v;
        }
        for (int i = threadIdx.x; i < MAXC * CC * 27; i += blockDim.x) {
            const int co = i / (CC * 27), c = (i / 27) % CC, k = i % 27;
            wsm[co][c][k] = (co < Co && c < nc) ? __bfloat162float(Wt[((size_t)co * Ci + c0 + c) * 27 + k]) : 0.f;
        }
        __syncthreads();
        for (int c = 0; c < nc; ++c)
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const float v = tile[c][tz + k / 9][ty + (k / 3) % 3][tx + k % 3];
#pragma unroll
                for (int co = 0; co < MAXC; ++co) acc[co] = fmaf(wsm[co][c][k], v, acc[co]);
            }
    }
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    if (x < W && y < H && z < D) {
        const size_t p = ((size_t)z * H + y) * W + x;
        for (int co = 0; co < Co; ++co) {
            float v = acc[co] + (bias ? bias[co] : 0.f);
            if (relu) v = fmaxf(v, 0.f);
            out[((size_t)b * Co + co) * N + p] = v;
        }
    }
}

// g *= (pre > 0)
__global__ void k_relu_bwd(float *g, const float *pre, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (pre[i] <= 0.f) g[i] = 0.f;
}

// gW[co][ci][k] += sum_p gout[b][co][p] in[b][ci][p + k - 1]; gb[co] += sum_p gout[b][co][p]
__global__ void __launch_bounds__(TB *TB *TB) k_conv_wgrad(const float *__restrict__ in, const float *__restrict__ gout,
                                                            float *__restrict__ gW, float *__restrict__ gb, int Ci,
                                                            int Co, int D, int H, int W) {
    __shared__ float tile[CC][TB + 2][TB + 2][TB + 2];
    __shared__ float gt[MAXC][TB * TB * TB];
    const int tilesX = (W + TB - 1) / TB, tilesY = (H + TB - 1) / TB;
    const int bx = blockIdx.x % tilesX, by = (blockIdx.x / tilesX) % tilesY, bz = blockIdx.x / (tilesX * tilesY);
    const int x0 = bx * TB, y0 = by * TB, z0 = bz * TB;
    const int b = blockIdx.y;
    const int c0 = blockIdx.z * CC;
    const int nc = min(CC, Ci - c0);
    const size_t N = (size_t)D * H * W;
    for (int i = threadIdx.x; i < MAXC * TB * TB * TB; i += blockDim.x) {
        const int co = i / (TB * TB * TB), r = i % (TB * TB * TB);
        const int lz = r / (TB * TB), ly = (r / TB) % TB, lx = r % TB;
        const int z = z0 + lz, y = y0 + ly, x = x0 + lx;
        float v = 0.f;
        if (co < Co && z < D && y < H && x < W) v = gout[((size_t)b * Co + co) * N + ((size_t)z * H + y) * W + x];
        gt[co][r] = v;
    }
    for (int i = threadIdx.x; i < CC * (TB + 2) * (TB + 2) * (TB + 2); i += blockDim.x) {
        const int c = i / ((TB + 2) * (TB + 2) * (TB + 2));
        const int r = i % ((TB + 2) * (TB + 2) * (TB + 2));
        const int lz = r / ((TB + 2) * (TB + 2)), ly = (r / (TB + 2)) % (TB + 2), lx = r % (TB + 2);
        const int z = z0 + lz - 1, y = y0 + ly - 1, x = x0 + lx - 1;
        float v = 0.f;
        if (c < nc && z >= 0 && z < D && y >= 0 && y < H && x >= 0 && x < W)
            v = in[((size_t)b * Ci + c0 + c) * N + ((size_t)z * H + y) * W + x];
        tile[c][lz][ly][lx] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < Co * nc * 27; e += blockDim.x) {
        const int co = e / (nc * 27), c = (e / 27) % nc, k = e % 27;
        const int dz = k / 9, dy = (k / 3) % 3, dx = k % 3;
        float s = 0.f;
        for (int r = 0; r < TB * TB * TB; ++r) {
            const int lz = r / (TB * TB), ly = (r / TB) % TB, lx = r % TB;
            s = fmaf(gt[co][r], tile[c][lz + dz][ly + dy][lx + dx], s);
        }
        atomicAdd(&gW[((size_t)co * Ci + c0 + c) * 27 + k], s);
    }
    if (blockIdx.z == 0)
        for (int co = threadIdx.x; co < Co; co += blockDim.x) {
            float s = 0.f;
            for (int r = 0; r < TB * TB * TB; ++r) s += gt[co][r];
            atomicAdd(&gb[co], s);
        }
}

// Adam on FP32 master weights; refresh the BF16 copy and the flipped /
// transposed BF16 copy used by the data-gradient convolution
__global__ void k_adam(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void k_to_bf16(const float *w, __nv_bfloat16 *wb, __nv_bfloat16 *wf, int Co, int Ci) {
    const int n = Co * Ci * 27;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int co = i / (Ci * 27), ci = (i / 27) % Ci, k = i % 27;
        const __nv_bfloat16 v = __float2bfloat16(w[i]);
        wb[i] = v;
        wf[((size_t)ci * Co + co) * 27 + (26 - k)] = v;   // [ci][co][flipped k]
    }
}

// relative MSE: loss += sum_b ||y_b - t_b||^2 / ||t_b||^2 / B ; g = 2 (y - t) / (B ||t_b||^2)
__global__ void k_loss(const float *y, const float *t, float *g, size_t per, int B, float *loss) {
    const int b = blockIdx.x;
    __shared__ float s1[256], s2[256];
    float a = 0.f, c = 0.f;
    for (size_t i = threadIdx.x; i < per; i += blockDim.x) {
        const float d = y[b * per + i] - t[b * per + i];
        a += d * d;
        c += t[b * per + i] * t[b * per + i];
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = c;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { s1[threadIdx.x] += s1[threadIdx.x + s]; s2[threadIdx.x] += s2[threadIdx.x + s]; }
        __syncthreads();
    }
    const float tn = fmaxf(s2[0], 1e-30f);
    if (threadIdx.x == 0) atomicAdd(loss, s1[0] / tn / B);
    for (size_t i = threadIdx.x; i < per; i += blockDim.x) g[b * per + i] = 2.f * (y[b * per + i] - t[b * per + i]) / (B * tn);
}

inline int nb(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

}  // namespace

void CNN::init(int cin_, int width_, int cout_, int layers_, int D_, int H_, int W_, int batch_, uint64_t seed) {
    cin = cin_; width = width_; cout = cout_; layers = layers_;
    D = D_; H = H_; W = W_; batch = batch_;
    TDZ_CHECK(width <= MAXC && cout <= MAXC && cin <= 64, TDZ_ERR_UNSUPPORTED, "network too wide");
    ci.assign(layers, width);
    co.assign(layers, width);
    ci[0] = cin;
    co[layers - 1] = cout;
    std::mt19937_64 rng(seed);
    w32.resize(layers); wbf.resize(layers); wflip.resize(layers); b.resize(layers);
    gw.resize(layers); gb.resize(layers); mw.resize(layers); vw.resize(layers); mb.resize(layers); vb.resize(layers);
    for (int l = 0; l < layers; ++l) {
        const size_t nw = (size_t)co[l] * ci[l] * 27;
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (ci[l] * 27.0)) * (l + 1 == layers ? 0.1 : 1.0));
        std::vector<float> wh(nw), bh(co[l], 0.f);
        for (auto &v : wh) v = (float)nd(rng);
        upload(w32[l], wh);
        upload(b[l], bh);
        wbf[l].alloc(nw * sizeof(__nv_bfloat16));
        wflip[l].alloc(nw * sizeof(__nv_bfloat16));
        for (DevBuf *d : {&gw[l], &mw[l], &vw[l]}) { d->alloc(nw * sizeof(float)); TDZ_CUDA(cudaMemset(d->ptr, 0, nw * 4)); }
        for (DevBuf *d : {&gb[l], &mb[l], &vb[l]}) { d->alloc(co[l] * sizeof(float)); TDZ_CUDA(cudaMemset(d->ptr, 0, co[l] * 4)); }
        k_to_bf16<<<nb(nw), 256>>>(w32[l].as<float>(), wbf[l].as<__nv_bfloat16>(), wflip[l].as<__nv_bfloat16>(), co[l], ci[l]);
        TDZ_CUDA(cudaGetLastError());
    }
    const size_t N = (size_t)D * H * W;
    act.resize(layers + 1);
    pre.resize(layers);
    for (int l = 0; l <= layers; ++l) act[l].alloc((size_t)batch * (l == 0 ? cin : co[l - 1]) * N * sizeof(float));
    for (int l = 0; l < layers; ++l) pre[l].alloc((size_t)batch * co[l] * N * sizeof(float));
    for (auto &g : gbuf) g.alloc((size_t)batch * std::max(width, std::max(cin, cout)) * N * sizeof(float));
    loss.alloc(sizeof(float));
    TDZ_CUDA(cudaMemset(loss.ptr, 0, sizeof(float)));
    TDZ_CUDA(cudaDeviceSynchronize());
}

static void conv(const float *in, const void *w, const float *bias, float *out, int B, int Ci, int Co, int D, int H,
                 int W, bool relu, cudaStream_t st) {
    const int tiles = ((W + TB - 1) / TB) * ((H + TB - 1) / TB) * ((D + TB - 1) / TB);
    k_conv_fwd<<<dim3(tiles, B), TB * TB * TB, 0, st>>>(in, static_cast<const __nv_bfloat16 *>(w), bias, out, Ci, Co,
                                                        D, H, W, relu ? 1 : 0);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void CNN::forward(const float *in, float *out, int B, cudaStream_t st, bool keep) {
    TDZ_CHECK(B <= batch, TDZ_ERR_ARG, "batch larger than the network's buffers");
    const size_t N = (size_t)D * H * W;
    const float *h = in;
    for (int l = 0; l < layers; ++l) {
        const bool last = l + 1 == layers;
        float *dst = last ? out : act[l + 1].as<float>();
        if (keep && !last) {
            // keep the pre-activation for the backward pass
            conv(h, wbf[l].ptr, b[l].as<float>(), pre[l].as<float>(), B, ci[l], co[l], D, H, W, false, st);
            TDZ_CUDA(cudaMemcpyAsync(dst, pre[l].ptr, (size_t)B * co[l] * N * 4, cudaMemcpyDeviceToDevice, st));
            k_relu_bwd<<<nb((size_t)B * co[l] * N), 256, 0, st>>>(dst, pre[l].as<float>(), (size_t)B * co[l] * N);
            count_launch();
        } else {
            conv(h, wbf[l].ptr, b[l].as<float>(), dst, B, ci[l], co[l], D, H, W, !last, st);
        }
        h = dst;
    }
}

void CNN::train_step(const float *in, const float *target, int B, float lr, cudaStream_t st) {
    const size_t N = (size_t)D * H * W;
    TDZ_CUDA(cudaMemcpyAsync(act[0].ptr, in, (size_t)B * cin * N * 4, cudaMemcpyDeviceToDevice, st));
    forward(act[0].as<float>(), act[layers].as<float>(), B, st, true);
    float *g = gbuf[0].as<float>();
    k_loss<<<B, 256, 0, st>>>(act[layers].as<float>(), target, g, (size_t)cout * N, B, loss.as<float>());
    count_launch();
    int cur = 0;
    for (int l = layers - 1; l >= 0; --l) {
        TDZ_CUDA(cudaMemsetAsync(gw[l].ptr, 0, (size_t)co[l] * ci[l] * 27 * 4, st));
        TDZ_CUDA(cudaMemsetAsync(gb[l].ptr, 0, (size_t)co[l] * 4, st));
        const int tiles = ((W + TB - 1) / TB) * ((H + TB - 1) / TB) * ((D + TB - 1) / TB);
        k_conv_wgrad<<<dim3(tiles, B, (ci[l] + CC - 1) / CC), TB * TB * TB, 0, st>>>(
            act[l].as<float>(), gbuf[cur].as<float>(), gw[l].as<float>(), gb[l].as<float>(), ci[l], co[l], D, H, W);
        TDZ_CUDA(cudaGetLastError());
        count_launch();
        if (l > 0) {
            // data gradient: convolution with flipped, transposed weights, then the ReLU mask
            float *gn = gbuf[cur ^ 1].as<float>();
            conv(gbuf[cur].as<float>(), wflip[l].ptr, nullptr, gn, B, co[l], ci[l], D, H, W, false, st);
            k_relu_bwd<<<nb((size_t)B * ci[l] * N), 256, 0, st>>>(gn, pre[l - 1].as<float>(), (size_t)B * ci[l] * N);
            count_launch();
            cur ^= 1;
        }
    }
    ++step_count;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, (float)step_count), c2 = 1.f - std::pow(b2, (float)step_count);
    for (int l = 0; l < layers; ++l) {
        const size_t nw = (size_t)co[l] * ci[l] * 27;
        k_adam<<<nb(nw), 256, 0, st>>>(w32[l].as<float>(), gw[l].as<float>(), mw[l].as<float>(), vw[l].as<float>(), nw,
                                      lr, b1, b2, eps, c1, c2);
        k_adam<<<1, 256, 0, st>>>(b[l].as<float>(), gb[l].as<float>(), mb[l].as<float>(), vb[l].as<float>(), co[l], lr,
                                  b1, b2, eps, c1, c2);
        k_to_bf16<<<nb(nw), 256, 0, st>>>(w32[l].as<float>(), wbf[l].as<__nv_bfloat16>(), wflip[l].as<__nv_bfloat16>(),
                                          co[l], ci[l]);
        TDZ_CUDA(cudaGetLastError());
        count_launch(3);
    }
}

float CNN::read_loss(cudaStream_t st) {
    float h = 0.f;
    TDZ_CUDA(cudaMemcpyAsync(&h, loss.ptr, 4, cudaMemcpyDeviceToHost, st));
    TDZ_CUDA(cudaStreamSynchronize(st));
    TDZ_CUDA(cudaMemsetAsync(loss.ptr, 0, 4, st));
    return h;
}

void CNN::get_params(std::vector<float> &out) const {
    out.clear();
    for (int l = 0; l < layers; ++l) {
        const size_t nw = (size_t)co[l] * ci[l] * 27;
        std::vector<float> w(nw), bb(co[l]);
        TDZ_CUDA(cudaMemcpy(w.data(), w32[l].ptr, nw * 4, cudaMemcpyDeviceToHost));
        TDZ_CUDA(cudaMemcpy(bb.data(), b[l].ptr, co[l] * 4, cudaMemcpyDeviceToHost));
        out.insert(out.end(), w.begin(), w.end());
        out.insert(out.end(), bb.begin(), bb.end());
    }
}

void CNN::set_params(const std::vector<float> &in) {
    size_t o = 0;
    for (int l = 0; l < layers; ++l) {
        const size_t nw = (size_t)co[l] * ci[l] * 27;
        TDZ_CHECK(o + nw + co[l] <= in.size(), TDZ_ERR_ARG, "parameter vector too short");
        TDZ_CUDA(cudaMemcpy(w32[l].ptr, in.data() + o, nw * 4, cudaMemcpyHostToDevice));
        TDZ_CUDA(cudaMemcpy(b[l].ptr, in.data() + o + nw, co[l] * 4, cudaMemcpyHostToDevice));
        o += nw + co[l];
        k_to_bf16<<<nb(nw), 256>>>(w32[l].as<float>(), wbf[l].as<__nv_bfloat16>(), wflip[l].as<__nv_bfloat16>(), co[l], ci[l]);
        TDZ_CUDA(cudaGetLastError());
    }
    TDZ_CUDA(cudaDeviceSynchronize());
}

void CNN::get_grads(std::vector<float> &out) const {
    out.clear();
    for (int l = 0; l < layers; ++l) {
        const size_t nw = (size_t)co[l] * ci[l] * 27;
        std::vector<float> w(nw), bb(co[l]);
        TDZ_CUDA(cudaMemcpy(w.data(), gw[l].ptr, nw * 4, cudaMemcpyDeviceToHost));
        TDZ_CUDA(cudaMemcpy(bb.data(), gb[l].ptr, co[l] * 4, cudaMemcpyDeviceToHost));
        out.insert(out.end(), w.begin(), w.end());
        out.insert(out.end(), bb.begin(), bb.end());
    }
}

}  // namespace tdz
