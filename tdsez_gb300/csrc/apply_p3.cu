// Instantiations of the fused 2D/3D apply kernels for degree 3.
#include "apply3d_rb.cuh"

namespace tdz {

void apply_p3(int dim, bool hb, bool hc, const ApplyParams<float> &pf, const ApplyParams<double> &pd,
              const ApplyParams<dff> &pdf, int prec, cudaStream_t st) {
    if (prec == TDZ_FP64) dispatch_streams<double, 3>(dim, hb, hc, pd, st);
    else if (prec == TDZ_FP64_DF) dispatch_streams<dff, 3>(dim, hb, hc, pdf, st);
    else dispatch_streams<float, 3>(dim, hb, hc, pf, st, prec == kPrecF32M64);
}

}  // namespace tdz
