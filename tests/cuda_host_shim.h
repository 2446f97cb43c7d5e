// cuda_host_shim.h -- the CUDA rounding and bit-cast intrinsics used by ffloat.cuh, as IEEE
// binary32/binary64 operations of the host (compile with -ffp-contract=off: no contraction)
// and memcpy bit-casts, for host builds of the double-word arithmetic in the CPU tests.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif
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

