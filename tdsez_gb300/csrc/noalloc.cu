// Allocation-free fused multi-dot for callers that cannot allocate device
// memory: code that runs inside a host application that owns every device
// allocation (a PETSc VECCUDA build with a fixed memory pool, a plugin that
// must not grow the process's device footprint after start-up), or code that
// must avoid cudaMalloc's implicit device synchronisation in the middle of a
// time step. Same kernels as tdz_vec_mdot; the per-block partial sums live in
// the file-scope device array below instead of library-allocated scratch.
#include <map>
#include <mutex>

#include "blas.h"

namespace tdz {
namespace {

// Scratch: per-block partial sums of up to kNoAllocDots dot products
// (kNoAllocDots * kRedBlocksPublic complex doubles = 8 * 304 * 16 B = 38 KB).
// It is part of the library image: every GPU that loads the library holds it
// until the process exits.
constexpr int kNoAllocDots = 8;
__device__ __align__(256) double2 g_noalloc_partials[kNoAllocDots * blas::kRedBlocksPublic];

std::mutex g_mu;
std::map<int, double2 *> g_addr;   // device address of the array, per device

// Device address of the scratch on the current device. In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and cached.
double2 *scratch_address() {
    int dev = 0;
    TDZ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_addr.find(dev);
    if (it != g_addr.end()) return it->second;
    void *p = nullptr;
    TDZ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_addr[dev] = static_cast<double2 *>(p);
    return static_cast<double2 *>(p);
}

}  // namespace

void mdot_noalloc(const void *const *V, int k, const void *w, size_t n, int prec, double2 *out, cudaStream_t st) {
    TDZ_CHECK(k >= 1 && k <= kNoAllocDots, TDZ_ERR_ARG,
              "tdz_vec_mdot_noalloc: k = " + std::to_string(k) + " exceeds the " + std::to_string(kNoAllocDots) +
                  " dot products its static scratch holds (use tdz_vec_mdot)");
    double2 *partials = scratch_address();
    // every block writes its partial before the final sum reads it: nothing
    // of the previous call's contents is read
    blas::mdot_partials(V, k, w, n, prec, partials, blas::kRedBlocksPublic, out, st);
}

}  // namespace tdz
