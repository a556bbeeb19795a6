// Batched complex-by-real transforms on the 5th-generation tensor cores
// (tcgen05, TF32 with a hi/lo split of both operands, FP32 accuracy). Internal.
//
//   out[p][n][c][r] = sum_k in[p][r][c][k] B[k][n]      (p < planes, r < R, c = re/im)
//
// "Row-planar complex" layout: complex row r of plane p is stored as a row of
// real parts followed by a row of imaginary parts, in[((p R + r) 2 + c) ldi + k].
// The result is stored transposed per plane, out[((p N + n) 2 + c) ldo + r], so
// a chain of transforms contracts a different axis each time while every
// contraction runs over the contiguous index (K-major operands for the MMA).
// These are the eigenvector transforms of the fast-diagonalisation
// preconditioner along x and y.
#pragma once

#include <cuda.h>

#include <vector>

#include "common.h"

namespace tdz {

// B split into TF32 hi + lo parts, K-major ([n][k]), zero-padded to Kp
// (multiple of 16) and Np (multiple of 16, at most 256), stored [2][Np][Kp].
struct TransformMat {
    int K = 0, N = 0, Kp = 0, Np = 0;
    DevBuf hilo;
    CUtensorMap map{};
    // B is K x N, row-major, FP64
    void build(const std::vector<double> &B, int K, int N);
};

// true when the tensor-core transform handles an N x N matrix of this size
bool transform_supported(int N);

// Device error word of the transform kernels (0 = no error): a bounded wait
// that ran out sets it; read and cleared by take_transform_error().
int take_transform_error();

void transform(const TransformMat &T, const float *in, int planes, int R, int ldi, float *out, int ldo,
               cudaStream_t st);

}  // namespace tdz
