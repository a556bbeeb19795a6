// Dispatch of the fused apply: stage scalars folded into the kernel
// parameters, degree-specific instantiations in apply_p<P>.cu.
#include "apply3d_rb.cuh"

#include <atomic>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <type_traits>

namespace tdz {

namespace {
std::atomic<int> g_autotune{1};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tune;
}  // namespace

bool autotune_enabled() { return g_autotune.load() != 0; }
namespace {
// forced launch shape of the 3D apply, packed (tile_x << 32 | run); 0 = none.
// Initialised from TDZ_APPLY3D_SHAPE="tile_x,run", changed by tdz_set_apply3d_shape.
long long shape_from_env() {
    const char *v = std::getenv("TDZ_APPLY3D_SHAPE");
    int a = 0, b = 0;
    if (!v || std::sscanf(v, "%d,%d", &a, &b) != 2 || a <= 0 || b <= 0) return 0;
    return ((long long)a << 32) | (unsigned)b;
}
std::atomic<long long> g_shape{shape_from_env()};
}  // namespace

bool forced_shape(int *txw, int *run) {
    const long long v = g_shape.load();
    if (!v) return false;
    *txw = (int)(v >> 32);
    *run = (int)(v & 0xffffffffLL);
    return true;
}
void set_forced_shape(int txw, int run) {
    g_shape.store(txw > 0 && run > 0 ? (((long long)txw << 32) | (unsigned)run) : 0);
}
bool tune_verbose() {
    static const bool v = std::getenv("TDZ_AUTOTUNE_VERBOSE") != nullptr;
    return v;
}
void set_autotune(int on) { g_autotune.store(on ? 1 : 0); }

// error word of the 3D apply kernels' bounded waits, one per device,
// allocated with the first apply on the device
int *apply_error_word() {
    static std::mutex mu;
    static std::map<int, int *> words;
    int dev = 0;
    TDZ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = words.find(dev);
    if (it != words.end()) return it->second;
    int *p = nullptr;
    TDZ_CUDA(cudaMalloc(&p, sizeof(int)));
    TDZ_CUDA(cudaMemset(p, 0, sizeof(int)));
    words[dev] = p;
    return p;
}

int take_apply_error() {
    int *p = apply_error_word();
    int v = 0;
    TDZ_CUDA(cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) TDZ_CUDA(cudaMemset(p, 0, sizeof(int)));
    return v;
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 rb_encode_fn() {
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
}  // namespace

void rb_make_map(CUtensorMap *map, const void *x, int n0, int n1, int n2, int boxx, int boxy) {
    const cuuint64_t dims[3] = {(cuuint64_t)2 * n0, (cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[2] = {(cuuint64_t)16 * n0, (cuuint64_t)16 * n0 * n1};   // bytes, multiples of 16
    const cuuint32_t box[3] = {(cuuint32_t)boxx, (cuuint32_t)boxy, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = rb_encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(x), dims, strides,
                                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TDZ_CHECK(r == CUDA_SUCCESS, TDZ_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}
bool tune_lookup(const TuneKey &k, int *txw, int *zchunk) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(k);
    if (it == g_tune.end()) return false;
    *txw = it->second.first;
    *zchunk = it->second.second;
    return true;
}
void tune_store(const TuneKey &k, int txw, int zchunk) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[k] = {txw, zchunk};
}

namespace {

template <class T> T to_t(double v) { return (T)v; }
template <> dff to_t<dff>(double v) { return dff_from(v); }

template <class T>
CombP<T> eval_comb(const Comb &c, const std::array<cd, 5> &sg) {
    CombP<T> out{};
    out.n = c.n;
    for (int i = 0; i < c.n; ++i) {
        const cd v = c.factor[i] * sg[c.scalar[i]];
        out.base[i] = c.base[i];
        out.re[i] = to_t<T>(v.real());
        out.im[i] = to_t<T>(v.imag());
    }
    return out;
}

// 1: every coefficient of the combination is real, 2: every one is imaginary, else 0
inline int comb_kind(const Comb &c, const std::array<cd, 5> &sg) {
    bool re = true, im = true;
    for (int i = 0; i < c.n; ++i) {
        const cd v = c.factor[i] * sg[c.scalar[i]];
        if (v.imag() != 0.0) re = false;
        if (v.real() != 0.0) im = false;
    }
    return re ? 1 : im ? 2 : 0;
}

template <class T> const DevBuf &bands_of(const Operator &op, int d) {
    if (std::is_same<T, double>::value) return op.dev64[d];
    if (std::is_same<T, dff>::value) return op.devdf[d];
    return op.dev32[d];
}

template <class T>
ApplyParams<T> make_params(const Operator &op, const Plan &pl, const void *x, void *y) {
    ApplyParams<T> prm{};
    const Space &s = *op.sp;
    prm.x = x;
    prm.y = y;
    prm.n0 = s.ax[0].n;
    prm.n1 = s.dim > 1 ? s.ax[1].n : 1;
    prm.n2 = s.dim > 2 ? s.ax[2].n : 1;
    prm.b0 = static_cast<const T *>(bands_of<T>(op, 0).ptr);
    prm.b1 = s.dim > 1 ? static_cast<const T *>(bands_of<T>(op, 1).ptr) : nullptr;
    prm.b2 = s.dim > 2 ? static_cast<const T *>(bands_of<T>(op, 2).ptr) : nullptr;
    const std::array<cd, 5> sg = op.sigma_for(pl.which);
    prm.xT = eval_comb<T>(pl.xT, sg);
    prm.yT = eval_comb<T>(pl.yT, sg);
    prm.zA = eval_comb<T>(pl.zA, sg);
    prm.zC = eval_comb<T>(pl.zC, sg);
    prm.za_kind = comb_kind(pl.zA, sg);
    prm.zc_kind = comb_kind(pl.zC, sg);
    prm.p = s.ax[0].p;
    prm.walls = 0;
    if (pl.walls) {
        prm.walls = 1;
        for (int w = 0; w < 2; ++w) {
            cd d = 0;
            if (pl.wall_m >= 0) d += sg[pl.wall_m] * op.m_wall[w];
            if (pl.wall_h >= 0) d += sg[pl.wall_h] * op.h_wall[w];
            prm.wall_re[w] = to_t<T>(d.real());
            prm.wall_im[w] = to_t<T>(d.imag());
        }
    }
    return prm;
}

template <class T>
void launch_1d(const ApplyParams<T> &prm, cudaStream_t st) {
    const int threads = 128;
    k_apply1d<T><<<(prm.n0 + threads - 1) / threads, threads, 0, st>>>(prm);
}

}  // namespace

// sum of the fused-reduction partials, one block, fixed order
__global__ void k_apply_red_finish(const double2 *part, int n, double2 *out) {
    __shared__ double2 s[256];
    double2 t = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        t.x += part[i].x;
        t.y += part[i].y;
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s[threadIdx.x].x += s[threadIdx.x + h].x;
            s[threadIdx.x].y += s[threadIdx.x + h].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

void apply_red_finish(const double2 *part, double2 *out, cudaStream_t st) {
    k_apply_red_finish<<<1, 256, 0, st>>>(part, kApplyRedCap, out);
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

void launch_apply(const Operator &op, const Plan &pl, int prec, const void *x, void *y, cudaStream_t st,
                  const ApplyExtra &ex) {
    const int dim = op.sp->dim;
    TDZ_CHECK(!ex.red_mode || dim == 3, TDZ_ERR_INTERNAL, "fused reductions are 3D only");
    auto params = [&](auto tag) {
        auto prm = make_params<decltype(tag)>(op, pl, x, y);
        prm.sub = ex.sub;
        prm.red = ex.red;
        prm.dotv = ex.dotv;
        prm.red_mode = ex.red_mode;
        prm.err = apply_error_word();
        return prm;
    };
    if (dim == 1) {
        // 1D operators are tiny: the double-float request runs in native FP64
        if (prec != TDZ_FP32) launch_1d(params(double{}), st);
        else launch_1d(params(float{}), st);
    } else {
        TDZ_CHECK(prec != kPrecF32M64 || dim == 3, TDZ_ERR_INTERNAL, "FP32 arithmetic on FP64 vectors is 3D only");
        ApplyParams<float> pf{};
        ApplyParams<double> pd{};
        ApplyParams<dff> pdf{};
        if (prec == TDZ_FP64) pd = params(double{});
        else if (prec == TDZ_FP64_DF) pdf = params(dff{});
        else pf = params(float{});
        switch (op.P) {
        case 2: apply_p2(dim, pl.hasB, pl.hasC, pf, pd, pdf, prec, st); break;
        case 3: apply_p3(dim, pl.hasB, pl.hasC, pf, pd, pdf, prec, st); break;
        case 4: apply_p4(dim, pl.hasB, pl.hasC, pf, pd, pdf, prec, st); break;
        case 5: apply_p5(dim, pl.hasB, pl.hasC, pf, pd, pdf, prec, st); break;
        default: throw Error(TDZ_ERR_UNSUPPORTED, "2D/3D apply supports degrees 2..5");
        }
    }
    TDZ_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tdz
