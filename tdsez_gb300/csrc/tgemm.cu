// tcgen05 transform kernel (see tgemm.h).
//
// Persistent CTAs (one per SM, 160 threads) walk 256 x Np output tiles (two
// 128-row sub-tiles), 64 complex rows per sub-tile with real and imaginary
// part rows interleaved; the accumulators live in tensor memory (TMEM,
// columns 0 and 256). K runs in chunks of 16 (one 64-byte swizzled row per
// operand row) through an NS-stage ring (as many stages as fit, 5 for
// Np = 176) that warp 4 fills with TMA (cp.async.bulk.tensor, 64-byte
// swizzle) up to NS chunks ahead, across tile boundaries:
//   stage = A (256 x 16 FP32, split by warps 0-3 in place into TF32 hi, with
//           the lo part in one of two extra buffers; both rounded to nearest)
//         + B hi, B lo (Np x 16 each, split on the host).
// Short chunks and a deep ring keep several chunks of loads in flight behind
// the MMAs (with two 32-wide stages the loads of a chunk could only start
// when the MMAs two chunks back had finished, which left the tensor pipe idle
// most of the time).
// Per 8-wide K step thread 0 issues four MMAs,
//   D += A_hi B_hi + A_hi B_lo + A_lo B_hi + A_lo B_lo,
// the full product of the hi/lo splits (each part rounded to TF32), so the
// result has FP32 accuracy at TF32 tensor-core rates. At the end
// of a tile warps 0-3 read TMEM with tcgen05.ld (warp w owns lanes
// 32w..32w+31, lane = tile row) and store the tile transposed per plane.
// Every wait on an mbarrier is bounded (clock64): on time-out the kernel sets
// the error word, the consumers leave together, and TMEM is still freed.
#include "tgemm.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <set>

namespace tdz {

namespace {

constexpr int TM = 128;        // tile rows (GEMM rows)
constexpr int KC = 16;         // K per stage (64 bytes of FP32: one 64-byte swizzled row)
constexpr int A_BYTES = TM * KC * 4;   // 8 KB
constexpr long long kWaitCycles = 4000000000LL;   // about 2 s at 2 GHz

__device__ int g_tgemm_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) {
            atomicExch(&g_tgemm_error, 1);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// shared-memory matrix descriptor: K-major operand in the canonical 64-byte
// swizzled layout (8-row groups 512 bytes apart), start address addr
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);          // start address >> 4      bits  0-13
    d |= (uint64_t)1 << 16;                          // leading offset (unused) bits 16-29
    d |= (uint64_t)((8 * KC * 4) >> 4) << 32;        // stride offset 512 B     bits 32-45
    d |= (uint64_t)1 << 46;                          // descriptor version      bits 46-47
    d |= (uint64_t)4 << 61;                          // 64-byte swizzle         bits 61-63
    return d;
}

// instruction descriptor: kind::tf32, FP32 accumulator, K-major A and B, M = 128
__host__ __device__ constexpr uint32_t instr_desc(int n) {
    return (1u << 4)                         // D format F32
           | (2u << 7)                       // A format TF32
           | (2u << 10)                      // B format TF32
           | ((uint32_t)(n >> 3) << 17)      // N >> 3
           | ((uint32_t)(TM >> 4) << 24);    // M >> 4
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// nearest TF32 value (10 explicit mantissa bits; halfway cases away from zero)
__device__ __forceinline__ float tf32_round(float v) {
    return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
}

struct TGParams {
    float *out;
    int rows;      // GEMM rows = 2 planes R
    int R, N, ldo, nchunks, tiles;
};

// barrier.sync + AND-reduction over `count` threads on named barrier `id`
__device__ __forceinline__ bool bar_and(int id, int count, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(count)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// MS = 128-row sub-tiles per tile (1 or 2): with 2, each B chunk loaded by TMA
// serves 256 rows (two accumulators in TMEM at columns 0 and 256)
// Stages: as many as fit (up to 6), so that a stage's loads have several
// chunks of MMA time to land.
template <int NP, int MS> struct TGShape {
    static constexpr int B_BYTES = NP * KC * 4;
    static constexpr int A_T = MS * A_BYTES;
    static constexpr int STAGE = A_T + 2 * B_BYTES;          // A (FP32 -> TF32 hi in place), B hi, B lo
    static constexpr size_t smem_for(int ns) { return 1024 + (size_t)ns * STAGE + 2 * A_T + 2 * ns * 8 + 16; }
    static constexpr int NS = smem_for(6) <= 232448   ? 6
                              : smem_for(5) <= 232448 ? 5
                              : smem_for(4) <= 232448 ? 4
                              : smem_for(3) <= 232448 ? 3
                                                      : 2;
    static constexpr size_t SMEM = smem_for(NS);
    static constexpr bool fits = SMEM <= 232448;
};

// Persistent, warp-specialised: warps 0-3 split A, issue the MMAs (thread 0)
// and run the epilogue; warp 4 (one lane) is the TMA producer, running up to
// NS chunks ahead across tile boundaries, so loads overlap the epilogue.
template <int NP, int MS>
__global__ void __launch_bounds__(160, 1)
    k_transform(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap, const TGParams prm) {
    using S = TGShape<NP, MS>;
    constexpr int NS = S::NS, STAGE = S::STAGE, B_BYTES = S::B_BYTES, A_T = S::A_T, TMT = TM * MS;
    constexpr uint32_t TMEM_COLS = MS == 2 ? 512 : NP <= 32 ? 32 : NP <= 64 ? 64 : NP <= 128 ? 128 : 256;
    static_assert(NP % 16 == 0 && NP >= 16 && NP <= 256, "N tile");
    static_assert(S::fits, "shared memory");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *alo_base = base + NS * STAGE;
    uint64_t *bars = reinterpret_cast<uint64_t *>(alo_base + 2 * A_T);   // full[NS], done[NS]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NS);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nch = prm.nchunks;
    const int my_tiles = prm.tiles > (int)blockIdx.x ? (prm.tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int G = my_tiles * nch;
    auto a_st = [&](int s) { return base + s * STAGE; };
    auto bh_st = [&](int s) { return base + s * STAGE + A_T; };
    auto bl_st = [&](int s) { return base + s * STAGE + A_T + B_BYTES; };
    auto a_lo = [&](int g) { return alo_base + (g & 1) * A_T; };
    const uint32_t full0 = smem_u32(&bars[0]), done0 = smem_u32(&bars[NS]);

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(done0 + 8 * s, 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 4) {
        // ---- producer
        if (lane == 0) {
            constexpr uint32_t TX = A_T + 2 * B_BYTES;
            for (int g = 0; g < G; ++g) {
                const int s = g % NS;
                if (g >= NS && !mbar_wait(done0 + 8 * s, ((g - NS) / NS) & 1)) break;
                const int tile = (int)blockIdx.x + (g / nch) * (int)gridDim.x, c = g % nch;
                mbar_expect_tx(full0 + 8 * s, TX);
                tma_load_2d(smem_u32(a_st(s)), &amap, c * KC, tile * TMT, full0 + 8 * s);
                tma_load_2d(smem_u32(bh_st(s)), &bmap, c * KC, 0, full0 + 8 * s);
                tma_load_2d(smem_u32(bl_st(s)), &bmap, c * KC, NP, full0 + 8 * s);
            }
        }
    } else {
        // ---- consumers: 128 threads, named barrier 1
        const uint32_t idesc = instr_desc(NP);
        for (int g = 0; g < G; ++g) {
            const int s = g % NS, c = g % nch;
            bool ok = mbar_wait(full0 + 8 * s, (g / NS) & 1);
            if (ok && g >= 2) ok = mbar_wait(done0 + 8 * ((g - 2) % NS), ((g - 2) / NS) & 1);   // A_lo[g & 1] free
            if (!bar_and(1, 128, ok)) break;
            // split A into TF32 hi (in place) and lo, both rounded to nearest
            float4 *ah = reinterpret_cast<float4 *>(a_st(s));
            float4 *al = reinterpret_cast<float4 *>(a_lo(g));
#pragma unroll
            for (int q = 0; q < A_T / 16 / 128; ++q) {
                const int e = tid + q * 128;
                const float4 v = ah[e];
                const float4 h = make_float4(tf32_round(v.x), tf32_round(v.y), tf32_round(v.z), tf32_round(v.w));
                ah[e] = h;
                al[e] = make_float4(tf32_round(v.x - h.x), tf32_round(v.y - h.y), tf32_round(v.z - h.z),
                                    tf32_round(v.w - h.w));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bar_sync(1, 128);
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t ah_a = smem_u32(a_st(s)), al_a = smem_u32(a_lo(g));
                const uint32_t bh_a = smem_u32(bh_st(s)), bl_a = smem_u32(bl_st(s));
#pragma unroll
                for (int j = 0; j < KC / 8; ++j) {
                    const uint32_t off = j * 32;   // 8 TF32 = 32 bytes along the 64-byte swizzled row
                    const uint64_t dbh = smem_desc(bh_a + off), dbl = smem_desc(bl_a + off);
#pragma unroll
                    for (int t = 0; t < MS; ++t) {   // sub-tile t: A rows 128 t.., accumulator columns 256 t..
                        const uint64_t dah = smem_desc(ah_a + t * A_BYTES + off), dal = smem_desc(al_a + t * A_BYTES + off);
                        const uint32_t d = tmem + (uint32_t)(t * 256);
                        mma_tf32(d, dah, dbh, idesc, (c > 0 || j > 0) ? 1u : 0u);
                        mma_tf32(d, dah, dbl, idesc, 1u);
                        mma_tf32(d, dal, dbh, idesc, 1u);
                        mma_tf32(d, dal, dbl, idesc, 1u);
                    }
                }
                mma_commit(done0 + 8 * s);
            }
            if (c == nch - 1) {
                // tile complete: TMEM -> registers -> global (transposed per plane)
                const bool okd = mbar_wait(done0 + 8 * s, (g / NS) & 1);
                if (!bar_and(1, 128, okd)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int tile = (int)blockIdx.x + (g / nch) * (int)gridDim.x;
                const size_t nstride = (size_t)2 * prm.ldo;
#pragma unroll 1
                for (int t = 0; t < MS; ++t) {
                    const int row = tile * TMT + t * TM + warp * 32 + lane;
                    const bool row_ok = row < prm.rows;
                    const int cr = row >> 1, part = row & 1;
                    const int p = row_ok ? cr / prm.R : 0, r = row_ok ? cr % prm.R : 0;
                    float *orow = prm.out + ((size_t)p * prm.N * 2 + part) * prm.ldo + r;
#pragma unroll 1
                    for (int c0 = 0; c0 < NP; c0 += 16) {
                        uint32_t v[16];
                        const uint32_t taddr = tmem + (uint32_t)(t * 256) + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                            "%12, %13, %14, %15}, [%16];"
                            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                              "=r"(v[14]), "=r"(v[15])
                            : "r"(taddr));
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        if (row_ok) {
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int n = c0 + j;
                                if (n < prm.N) orow[(size_t)n * nstride] = __uint_as_float(v[j]);
                            }
                        }
                    }
                }
                // the next tile's first MMA overwrites the accumulator
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                bar_sync(1, 128);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// Warp-specialised variant with double-buffered accumulators (320 threads,
// one CTA per SM, 128-row tiles):
//   warps 0-3  split each A chunk into TF32 hi (in place) and lo (a buffer of
//              the same stage), then arrive on the stage's `split` barrier;
//   warp 9     (one thread) issues the stage's MMAs into accumulator
//              tile & 1 (TMEM columns 0 or 256) and commits them to the
//              stage's `done` barrier, and at the end of a tile to `accf`;
//   warps 4-7  drain accumulator tile & 1 (warp w reads TMEM lanes
//              32 (w % 4)..) into the transposed output, then arrive on
//              `acce`, so the MMAs of the next tile run meanwhile;
//   warp 8     (one thread) keeps the stage ring full with TMA.
// The lo part lives in its stage, so the split of a chunk never waits for
// MMAs (the producer recycles a stage only after its MMAs completed).
template <int NP> struct WSShape {
    static constexpr int B_BYTES = NP * KC * 4;
    static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;   // A (hi in place), A lo, B hi, B lo
    static constexpr size_t smem_for(int ns) { return 1024 + (size_t)ns * STAGE + (3 * ns + 4) * 8 + 16; }
    static constexpr int NS = smem_for(6) <= 232448   ? 6
                              : smem_for(5) <= 232448 ? 5
                              : smem_for(4) <= 232448 ? 4
                              : smem_for(3) <= 232448 ? 3
                                                      : 2;
    static constexpr size_t SMEM = smem_for(NS);
    static constexpr bool fits = SMEM <= 232448;
};

template <int NP>
__global__ void __launch_bounds__(320, 1)
    k_transform_ws(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                   const TGParams prm) {
    using S = WSShape<NP>;
    constexpr int NS = S::NS, STAGE = S::STAGE, B_BYTES = S::B_BYTES;
    constexpr uint32_t TMEM_COLS = 512;   // two accumulators, columns 0 and 256
    static_assert(NP % 16 == 0 && NP >= 16 && NP <= 256, "N tile");
    static_assert(S::fits, "shared memory");
    static_assert(STAGE % 1024 == 0 && A_BYTES % 1024 == 0 && B_BYTES % 512 == 0, "swizzle alignment");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + NS * STAGE);   // full, split, done [NS]; accf, acce [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 3 * NS + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nch = prm.nchunks;
    const int my_tiles = prm.tiles > (int)blockIdx.x ? (prm.tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int G = my_tiles * nch;
    auto a_st = [&](int s) { return base + s * STAGE; };
    auto alo_st = [&](int s) { return base + s * STAGE + A_BYTES; };
    auto bh_st = [&](int s) { return base + s * STAGE + 2 * A_BYTES; };
    auto bl_st = [&](int s) { return base + s * STAGE + 2 * A_BYTES + B_BYTES; };
    const uint32_t full0 = smem_u32(&bars[0]), split0 = smem_u32(&bars[NS]), done0 = smem_u32(&bars[2 * NS]);
    const uint32_t accf0 = smem_u32(&bars[3 * NS]), acce0 = smem_u32(&bars[3 * NS + 2]);

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(split0 + 8 * s, 128);
            mbar_init(done0 + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(accf0 + 8 * b, 1);
            mbar_init(acce0 + 8 * b, 128);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 8) {
        // ---- producer
        if (lane == 0) {
            constexpr uint32_t TX = A_BYTES + 2 * B_BYTES;
            for (int g = 0; g < G; ++g) {
                const int s = g % NS;
                if (g >= NS && !mbar_wait(done0 + 8 * s, ((g - NS) / NS) & 1)) break;
                const int tile = (int)blockIdx.x + (g / nch) * (int)gridDim.x, c = g % nch;
                mbar_expect_tx(full0 + 8 * s, TX);
                tma_load_2d(smem_u32(a_st(s)), &amap, c * KC, tile * TM, full0 + 8 * s);
                tma_load_2d(smem_u32(bh_st(s)), &bmap, c * KC, 0, full0 + 8 * s);
                tma_load_2d(smem_u32(bl_st(s)), &bmap, c * KC, NP, full0 + 8 * s);
            }
        }
    } else if (warp == 9) {
        // ---- MMA issue
        if (lane == 0) {
            const uint32_t idesc = instr_desc(NP);
            for (int g = 0; g < G; ++g) {
                const int s = g % NS, c = g % nch, t = g / nch, b = t & 1;
                if (c == 0 && t >= 2 && !mbar_wait(acce0 + 8 * b, ((t - 2) >> 1) & 1)) break;
                if (!mbar_wait(split0 + 8 * s, (g / NS) & 1)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t ah_a = smem_u32(a_st(s)), al_a = smem_u32(alo_st(s));
                const uint32_t bh_a = smem_u32(bh_st(s)), bl_a = smem_u32(bl_st(s));
                const uint32_t d = tmem + (uint32_t)(b * 256);
#pragma unroll
                for (int j = 0; j < KC / 8; ++j) {
                    const uint32_t off = j * 32;   // 8 TF32 = 32 bytes along the 64-byte swizzled row
                    const uint64_t dah = smem_desc(ah_a + off), dal = smem_desc(al_a + off);
                    const uint64_t dbh = smem_desc(bh_a + off), dbl = smem_desc(bl_a + off);
                    // the full product of the splits: without lo.lo (2^-22 of each
                    // product) the FDM guess of the CN step is a few times less
                    // accurate, and the certified FP32 Arnoldi cycle fails its bound
                    // on some steps (measured: 4.30 against 3.69 ms per step)
                    mma_tf32(d, dah, dbh, idesc, (c > 0 || j > 0) ? 1u : 0u);
                    mma_tf32(d, dah, dbl, idesc, 1u);
                    mma_tf32(d, dal, dbh, idesc, 1u);
                    mma_tf32(d, dal, dbl, idesc, 1u);
                }
                mma_commit(done0 + 8 * s);
                if (c == nch - 1) mma_commit(accf0 + 8 * b);
            }
        }
    } else if (warp < 4) {
        // ---- A split: TF32 hi in place, lo into the stage's lo buffer, both rounded to nearest
        for (int g = 0; g < G; ++g) {
            const int s = g % NS;
            if (!mbar_wait(full0 + 8 * s, (g / NS) & 1)) break;
            float4 *ah = reinterpret_cast<float4 *>(a_st(s));
            float4 *al = reinterpret_cast<float4 *>(alo_st(s));
#pragma unroll
            for (int q = 0; q < A_BYTES / 16 / 128; ++q) {
                const int e = tid + q * 128;
                const float4 v = ah[e];
                const float4 h = make_float4(tf32_round(v.x), tf32_round(v.y), tf32_round(v.z), tf32_round(v.w));
                ah[e] = h;
                al[e] = make_float4(tf32_round(v.x - h.x), tf32_round(v.y - h.y), tf32_round(v.z - h.z),
                                    tf32_round(v.w - h.w));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(split0 + 8 * s);
        }
    } else {
        // ---- epilogue: TMEM -> registers -> global (transposed per plane)
        const int q = warp & 3;
        const size_t nstride = (size_t)2 * prm.ldo;
        for (int t = 0; t < my_tiles; ++t) {
            const int b = t & 1;
            if (!mbar_wait(accf0 + 8 * b, (t >> 1) & 1)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int tile = (int)blockIdx.x + t * (int)gridDim.x;
            const int row = tile * TM + q * 32 + lane;
            const bool row_ok = row < prm.rows;
            const int cr = row >> 1, part = row & 1;
            const int p = row_ok ? cr / prm.R : 0, r = row_ok ? cr % prm.R : 0;
            float *orow = prm.out + ((size_t)p * prm.N * 2 + part) * prm.ldo + r;
            const uint32_t tbase = tmem + (uint32_t)(b * 256) + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
            for (int c0 = 0; c0 < NP; c0 += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                    "%12, %13, %14, %15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                      "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                      "=r"(v[14]), "=r"(v[15])
                    : "r"(tbase + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (row_ok) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int n = c0 + j;
                        if (n < prm.N) orow[(size_t)n * nstride] = __uint_as_float(v[j]);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(acce0 + 8 * b);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    TDZ_CHECK(fn != nullptr, TDZ_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

// 2D FP32 tensor map: inner extent `inner` (elements), `outer` rows of pitch
// `pitch` elements, box KC x box_rows, 64-byte swizzle, zero fill outside
void make_map(CUtensorMap *map, const void *ptr, uint64_t inner, uint64_t outer, uint64_t pitch, uint32_t box_rows) {
    TDZ_CHECK((reinterpret_cast<uintptr_t>(ptr) & 15) == 0, TDZ_ERR_ARG, "transform operand not 16-byte aligned");
    TDZ_CHECK((pitch * 4) % 16 == 0, TDZ_ERR_ARG, "transform row pitch not a multiple of 16 bytes");
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {pitch * 4};
    const cuuint32_t box[2] = {(cuuint32_t)KC, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims, strides,
                                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TDZ_CHECK(r == CUDA_SUCCESS, TDZ_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

float tf32_round_host(double v) {
    float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    std::memcpy(&f, &u, 4);
    return f;
}

// 256-row tiles where two sub-tiles' stages fit in shared memory (Np <= 192), else 128
template <int NP> constexpr int sub_tiles() { return TGShape<NP, 2>::fits ? 2 : 1; }

// the warp-specialised kernel unless TDZ_TRANSFORM=split asks for the
// single-accumulator-pair one
bool use_ws() {
    static const bool ws = [] {
        const char *e = std::getenv("TDZ_TRANSFORM");
        return !(e && std::string(e) == "split");
    }();
    return ws;
}

template <int NP>
void launch(const TransformMat &T, const float *in, int ldi, TGParams prm, cudaStream_t st) {
    const bool ws = use_ws();
    constexpr int MS = sub_tiles<NP>();
    const size_t smem = ws ? WSShape<NP>::SMEM : TGShape<NP, MS>::SMEM;
    // opt-in to the tile's shared memory once per device (guarded: the batch
    // API steps runs from several host threads)
    {
        static std::mutex mu;
        static std::set<int> done;
        int dev = 0;
        TDZ_CUDA(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> lk(mu);
        if (!done.count(dev)) {
            TDZ_CUDA(cudaFuncSetAttribute(k_transform<NP, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TGShape<NP, MS>::SMEM));
            TDZ_CUDA(cudaFuncSetAttribute(k_transform_ws<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)WSShape<NP>::SMEM));
            done.insert(dev);
        }
    }
    CUtensorMap amap;
    const int rows_per_tile = ws ? TM : TM * MS;
    make_map(&amap, in, (uint64_t)T.K, (uint64_t)prm.rows, (uint64_t)ldi, (uint32_t)rows_per_tile);
    prm.tiles = (prm.rows + rows_per_tile - 1) / rows_per_tile;
    const int grid = std::min(prm.tiles, sm_count());
    if (ws) k_transform_ws<NP><<<grid, 320, smem, st>>>(amap, T.map, prm);
    else k_transform<NP, MS><<<grid, 160, smem, st>>>(amap, T.map, prm);
}

}  // namespace

bool transform_supported(int N) { return N >= 1 && N <= 256; }

void TransformMat::build(const std::vector<double> &B, int K_, int N_) {
    K = K_;
    N = N_;
    TDZ_CHECK(transform_supported(N), TDZ_ERR_UNSUPPORTED, "tensor-core transform supports N <= 256");
    TDZ_CHECK((int)B.size() == K * N, TDZ_ERR_ARG, "transform matrix size");
    Kp = (K + KC - 1) / KC * KC;
    Np = (N + 15) / 16 * 16;
    std::vector<float> h((size_t)2 * Np * Kp, 0.f);
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < K; ++k) {
            const double v = B[(size_t)k * N + n];
            const float hi = tf32_round_host(v);
            h[(size_t)n * Kp + k] = hi;
            h[(size_t)(Np + n) * Kp + k] = tf32_round_host(v - (double)hi);
        }
    upload(hilo, h);
    make_map(&map, hilo.ptr, Kp, 2 * (uint64_t)Np, Kp, (uint32_t)Np);
}

int take_transform_error() {
    int h = 0;
    TDZ_CUDA(cudaMemcpyFromSymbol(&h, g_tgemm_error, sizeof(int)));
    if (h) {
        const int z = 0;
        TDZ_CUDA(cudaMemcpyToSymbol(g_tgemm_error, &z, sizeof(int)));
    }
    return h;
}

void transform(const TransformMat &T, const float *in, int planes, int R, int ldi, float *out, int ldo,
               cudaStream_t st) {
    TDZ_CHECK(ldi >= T.K && ldo >= R, TDZ_ERR_ARG, "transform pitches too small");
    const long long rows = 2LL * planes * R;
    TDZ_CHECK(rows < (1LL << 31), TDZ_ERR_ARG, "transform too large");
    TGParams prm{};
    prm.out = out;
    prm.rows = (int)rows;
    prm.R = R;
    prm.N = T.N;
    prm.ldo = ldo;
    prm.nchunks = T.Kp / KC;
    switch (T.Np) {
    case 16: launch<16>(T, in, ldi, prm, st); break;
    case 32: launch<32>(T, in, ldi, prm, st); break;
    case 48: launch<48>(T, in, ldi, prm, st); break;
    case 64: launch<64>(T, in, ldi, prm, st); break;
    case 80: launch<80>(T, in, ldi, prm, st); break;
    case 96: launch<96>(T, in, ldi, prm, st); break;
    case 112: launch<112>(T, in, ldi, prm, st); break;
    case 128: launch<128>(T, in, ldi, prm, st); break;
    case 144: launch<144>(T, in, ldi, prm, st); break;
    case 160: launch<160>(T, in, ldi, prm, st); break;
    case 176: launch<176>(T, in, ldi, prm, st); break;
    case 192: launch<192>(T, in, ldi, prm, st); break;
    case 208: launch<208>(T, in, ldi, prm, st); break;
    case 224: launch<224>(T, in, ldi, prm, st); break;
    case 240: launch<240>(T, in, ldi, prm, st); break;
    case 256: launch<256>(T, in, ldi, prm, st); break;
    default: throw Error(TDZ_ERR_INTERNAL, "bad transform tile width");
    }
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tdz
