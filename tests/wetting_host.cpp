// Host build of the per-node wetting step (mf-lbm_gb300/csrc/wetting.cuh) in FP64 and FP32
// for the CPU tests (compiled with -ffp-contract=off).
#include <cmath>

#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif

namespace hostchk {
using std::sqrt;
#include "../mf-lbm_gb300/csrc/wetting.cuh"
}  // namespace hostchk

extern "C" {
// n (in/out, 3), nw (3); min_one_m = 0: the reference's expression
void wh_f64(double *n, const double *nw, double cos_t, double sin_t, double min_one_m) {
    double v[3] = {n[0], n[1], n[2]};
    hostchk::wetting_normal<double>(v, nw[0], nw[1], nw[2], cos_t, sin_t, min_one_m);
    n[0] = v[0]; n[1] = v[1]; n[2] = v[2];
}
void wh_f32(float *n, const float *nw, float cos_t, float sin_t, float min_one_m) {
    float v[3] = {n[0], n[1], n[2]};
    hostchk::wetting_normal<float>(v, nw[0], nw[1], nw[2], cos_t, sin_t, min_one_m);
    n[0] = v[0]; n[1] = v[1]; n[2] = v[2];
}
}
