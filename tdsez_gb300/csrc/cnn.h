// Learned coarse correction: a small 3D convolutional network on a multigrid
// level (hand-written forward / backward / Adam kernels). Internal.
#pragma once

#include <vector>

#include "common.h"

namespace tdz {

struct CNN {
    int cin = 4, width = 32, cout = 2, layers = 4;
    int D = 0, H = 0, W = 0, batch = 0;        // grid and training batch
    std::vector<int> ci, co;                   // channels per layer
    std::vector<DevBuf> w32, wbf, wflip, b;    // FP32 master weights, BF16 copy, flipped/transposed BF16, bias
    std::vector<DevBuf> gw, gb, mw, vw, mb, vb;
    std::vector<DevBuf> act, pre;              // activations (batch) per layer
    DevBuf gbuf[2];                            // gradient ping-pong
    DevBuf loss;                               // device loss accumulator
    long long step_count = 0;

    void init(int cin_, int width_, int cout_, int layers_, int D_, int H_, int W_, int batch_, uint64_t seed);
    // out[B][cout][DHW] for in[B][cin][DHW] (FP32)
    void forward(const float *in, float *out, int B, cudaStream_t st, bool keep);
    // one training step on (in, target); returns nothing (loss accumulated on device)
    void train_step(const float *in, const float *target, int B, float lr, cudaStream_t st);
    float read_loss(cudaStream_t st);
    void get_params(std::vector<float> &out) const;   // w, b per layer (FP32 master)
    void set_params(const std::vector<float> &in);
    void get_grads(std::vector<float> &out) const;
};

}  // namespace tdz
