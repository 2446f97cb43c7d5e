// Host build of the double-word arithmetic (mf-lbm_gb300/csrc/ffloat.cuh) for the CPU
// tests: the CUDA rounding intrinsics are mapped onto IEEE binary32/binary64 operations
// of the host (SSE / NEON arithmetic, no contraction: compiled with -ffp-contract=off),
// and the bit-casts onto memcpy.  Exposes each operation through a C entry point.
#include "cuda_host_shim.h"

#include "../mf-lbm_gb300/csrc/ffloat.cuh"

using mflbm::ff;

extern "C" {
void ffh_from_f64(const double *d, float *hi, float *lo, int n) {
    for (int i = 0; i < n; ++i) {
        const ff x = mflbm::ff_from_f64(d[i]);
        hi[i] = x.hi;
        lo[i] = x.lo;
    }
}
// the select-free split: per value its (hi, lo) and whether its span passed
void ffh_from_f64_in_range(const double *d, float *hi, float *lo, int *inside, int n) {
    for (int i = 0; i < n; ++i) {
        unsigned span = 0u;
        const ff x = mflbm::ff_from_f64_in_range(d[i], span);
        hi[i] = x.hi;
        lo[i] = x.lo;
        inside[i] = span <= mflbm::kFfInRangeSpan;
    }
}
void ffh_to_f64(const float *hi, const float *lo, double *d, int n) {
    for (int i = 0; i < n; ++i) d[i] = mflbm::f64_of_ff(ff{hi[i], lo[i]});
}
void ffh_f32_to_f64(const float *x, double *d, int n) {
    for (int i = 0; i < n; ++i) d[i] = mflbm::f64_of_f32(x[i]);
}
// op 0: x + y, 1: x - y, 2: x * y, 3: x * y.hi (FP32 factor), 4: x * 0.5, 5: x / y
void ffh_op(int op, const float *xh, const float *xl, const float *yh, const float *yl, float *zh, float *zl, int n) {
    for (int i = 0; i < n; ++i) {
        const ff x{xh[i], xl[i]}, y{yh[i], yl[i]};
        ff z;
        switch (op) {
            case 0: z = x + y; break;
            case 1: z = x - y; break;
            case 2: z = x * y; break;
            case 3: z = mflbm::ff_mulf(x, y.hi); break;
            case 5: z = x / y; break;
            case 6: z = mflbm::ff_sqrt(x); break;
            case 4: z = mflbm::ff_pow2(x, 0.5f); break;
            default: z = x; break;
        }
        zh[i] = z.hi;
        zl[i] = z.lo;
    }
}
void ffh_const(double d, float *hi, float *lo) {
    const ff x = mflbm::ff_const(d);
    *hi = x.hi;
    *lo = x.lo;
}
}
