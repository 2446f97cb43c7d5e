// Host build of the double-word arithmetic (mf-lbm_gb300/csrc/ffloat.cuh) for the CPU
// tests: the CUDA rounding intrinsics are mapped onto IEEE binary32/binary64 operations
// of the host (SSE / NEON arithmetic, no contraction: compiled with -ffp-contract=off),
// and the bit-casts onto memcpy.  Exposes each operation through a C entry point.
#include <cmath>
#include <cstdint>
#include <cstring>

#define __host__
#define __device__
#define __forceinline__ inline
#define FFLOAT_HOST_INTRINSICS 1

static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fsqrt_rn(float a) { return std::sqrt(a); }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline float __double2float_rn(double d) { return (float)d; }
static inline long long __double_as_longlong(double d) {
    long long r;
    std::memcpy(&r, &d, 8);
    return r;
}
static inline float __uint_as_float(unsigned u) {
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
static inline unsigned __float_as_uint(float f) {
    unsigned r;
    std::memcpy(&r, &f, 4);
    return r;
}
static inline unsigned __funnelshift_l(unsigned lo, unsigned hi, unsigned shift) {
    const unsigned long long v = ((unsigned long long)hi << 32) | lo;
    return (unsigned)((v << (shift & 31)) >> 32);
}
static inline double __hiloint2double(int hi, int lo) {
    const unsigned long long v = ((unsigned long long)(unsigned)hi << 32) | (unsigned)lo;
    double r;
    std::memcpy(&r, &v, 8);
    return r;
}

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
