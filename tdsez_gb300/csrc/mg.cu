// Tensor prolongation / restriction: contraction of one axis of a 3D array
// with a fixed-width row-sparse 1D matrix (Boehm rows or their transpose),
// one thread per output coefficient, consecutive threads on consecutive x.
#include "cplx.cuh"
#include "mg.h"

namespace tdz {

namespace {

template <class T>
__global__ void k_axis_contract(const int *__restrict__ col, const T *__restrict__ val, int width, int axis,
                                const typename CT<T>::type *__restrict__ in, typename CT<T>::type *__restrict__ out,
                                int o0, int o1, int o2, int i0, int i1, bool accumulate) {
    using C = typename CT<T>::type;
    const size_t total = (size_t)o0 * o1 * o2;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % o0);
        const size_t r = e / o0;
        const int b = (int)(r % o1);
        const int c = (int)(r / o1);
        const int row = axis == 0 ? a : (axis == 1 ? b : c);
        C acc = czero<C>();
        for (int t = 0; t < width; ++t) {
            const int j = col[(size_t)row * width + t];
            if (j < 0) break;
            const T v = val[(size_t)row * width + t];
            size_t src;
            if (axis == 0) src = ((size_t)c * i1 + b) * i0 + j;
            else if (axis == 1) src = ((size_t)c * i1 + j) * i0 + a;
            else src = ((size_t)j * i1 + b) * i0 + a;
            rfma(acc, v, in[src]);
        }
        if (accumulate) {
            C old = out[e];
            acc.x += old.x;
            acc.y += old.y;
        }
        out[e] = acc;
    }
}

}  // namespace

void axis_contract(const RowSparse &A, int axis, const void *in, void *out, int n0, int n1, int n2, bool accumulate,
                   int prec, cudaStream_t st) {
    // input shape (n2, n1, n0); output replaces the axis length by A.rows
    int o[3] = {n0, n1, n2};
    TDZ_CHECK(o[axis] == A.cols, TDZ_ERR_INTERNAL, "axis length does not match the 1D matrix");
    o[axis] = A.rows;
    const size_t total = (size_t)o[0] * o[1] * o[2];
    const int threads = 256;
    const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)16 * sm_count());
    if (prec == TDZ_FP64)
        k_axis_contract<double><<<blocks, threads, 0, st>>>(A.dcol.as<int>(), A.dval64.as<double>(), A.width, axis,
                                                            static_cast<const double2 *>(in), static_cast<double2 *>(out),
                                                            o[0], o[1], o[2], n0, n1, accumulate);
    else
        k_axis_contract<float><<<blocks, threads, 0, st>>>(A.dcol.as<int>(), A.dval32.as<float>(), A.width, axis,
                                                           static_cast<const float2 *>(in), static_cast<float2 *>(out),
                                                           o[0], o[1], o[2], n0, n1, accumulate);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tdz
