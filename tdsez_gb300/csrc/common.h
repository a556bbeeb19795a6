// Shared definitions of the tdz library (internal; the public C ABI is
// include/tdz.h).
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tdz.h"

namespace tdz {

using cd = std::complex<double>;

// Error carried from the C++ layer to the C ABI as a status code plus a
// message (no exception crosses the ABI).
struct Error : std::runtime_error {
    tdz_status code;
    Error(tdz_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

// Kernels launched by the library (all entry points), for launch accounting.
void count_launch(long long n = 1);
long long launch_count();

// Multiprocessors of the current device (looked up once per device; grids
// of the persistent and grid-stride kernels are sized in multiples of it).
int sm_count();

#define TDZ_CHECK(cond, code, msg)                                                          \
    do {                                                                                    \
        if (!(cond)) throw ::tdz::Error((code), std::string(msg) + " (" __FILE__ ":" +      \
                                                    std::to_string(__LINE__) + ")");        \
    } while (0)

#define TDZ_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            throw ::tdz::Error(TDZ_ERR_CUDA, std::string(#call) + ": " +                    \
                                                 cudaGetErrorString(e_) + " (" __FILE__ ":" + \
                                                 std::to_string(__LINE__) + ")");           \
    } while (0)

// Owning device buffer (allocated at set-up, never on the stepping path).
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    explicit DevBuf(size_t b) { alloc(b); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), bytes(o.bytes) { o.ptr = nullptr; o.bytes = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); ptr = o.ptr; bytes = o.bytes; o.ptr = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t b) {
        release();
        if (b == 0) return;
        TDZ_CUDA(cudaMalloc(&ptr, b));
        bytes = b;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

template <class T> inline void upload(DevBuf &b, const std::vector<T> &v) {
    b.alloc(v.size() * sizeof(T));
    if (!v.empty()) TDZ_CUDA(cudaMemcpy(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

}  // namespace tdz
