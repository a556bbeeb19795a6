// Instantiations of the fused 2D/3D apply kernels for degree 5.
#include "apply3d_rb.cuh"

namespace tdz {

void apply_p5(int dim, bool hb, bool hc, const ApplyParams<float> &pf, const ApplyParams<double> &pd,
              const ApplyParams<dff> &pdf, int prec, cudaStream_t st) {
    if (prec == TDZ_FP64) dispatch_streams<double, 5>(dim, hb, hc, pd, st);
    else if (prec == TDZ_FP64_DF) dispatch_streams<dff, 5>(dim, hb, hc, pdf, st);
    else dispatch_streams<float, 5>(dim, hb, hc, pf, st, prec == kPrecF32M64);
}

}  // namespace tdz
