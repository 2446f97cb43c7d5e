// ffloat.cuh -- double-word ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers, |lo| of the order of
// ulp(hi): about 48 significant bits.  GB300 issues 64 FP32 operations per FP64 operation,
// and an add or a multiply in this form costs 6-8 FP32 operations, so a collision that
// keeps FP64 storage but computes in this form runs on the FP32 pipe several times faster
// than on the FP64 pipe.  The building blocks are the error-free transformations of the
// literature:
//   TwoSum   (Knuth, TAOCP vol. 2, sec. 4.2.2)  s + e = a + b exactly, 6 operations
//   Fast2Sum (Dekker 1971)                       the same when |a| >= |b|, 3 operations
//   TwoProd  (with a fused multiply-add)         p + e = a * b exactly, 2 operations
// combined as in Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44(2), 2017: the sum is their
// sloppy sum without the final renormalisation (absolute error about 2^-47 (|x| + |y|),
// the bound that matters for populations that are differenced later), the products are
// the FMA-based ones with the lo*lo term dropped, also left unnormalised.  Every operation is a
// _rn intrinsic, so no contraction (--fmad) or re-association can break a transformation,
// and the default and strict builds give identical results.
#pragma once
#include <cstdint>
#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif

namespace mflbm {

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit constexpr ff(float h) : hi(h), lo(0.0f) {}
    // the FP64 value rounded to hi, the remainder rounded to lo (constant-folded for
    // literals; on the host for run parameters)
    __host__ __device__ explicit constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__host__ __device__ constexpr ff ff_const(double d) { return ff(d); }

// the arithmetic needs the CUDA rounding intrinsics (device code, or a host build that
// supplies them)
#if defined(__CUDACC__) || defined(FFLOAT_HOST_INTRINSICS)

__device__ __forceinline__ ff ff_fast2sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// x + y: TwoSum of the high parts, the low parts and the rounding error summed in FP32;
// the result is left unnormalised (the next operation tolerates |lo| of a few ulp(hi)).
__device__ __forceinline__ ff operator+(ff x, ff y) {
    const ff s = ff_two_sum(x.hi, y.hi);
    return ff{s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo))};
}
__device__ __forceinline__ ff operator-(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + (-y); }

// x * y: TwoProd of the high parts with the cross terms folded into its error FMA; the
// pair (ch, cl) is returned as it stands (|cl| is about ulp(ch), which every consumer
// accepts, so the renormalising Fast2Sum would only cost three operations)
__device__ __forceinline__ ff operator*(ff x, ff y) {
    const float ch = __fmul_rn(x.hi, y.hi);
    float cl = __fmaf_rn(x.hi, y.hi, -ch);
    cl = __fmaf_rn(x.hi, y.lo, cl);
    cl = __fmaf_rn(x.lo, y.hi, cl);
    return ff{ch, cl};
}

// x * k for an FP32 number k (same form)
__device__ __forceinline__ ff ff_mulf(ff x, float k) {
    const float ch = __fmul_rn(x.hi, k);
    float cl = __fmaf_rn(x.hi, k, -ch);
    cl = __fmaf_rn(x.lo, k, cl);
    return ff{ch, cl};
}

// x * 2^n: exact
__device__ __forceinline__ ff ff_pow2(ff x, float p2) { return ff{__fmul_rn(x.hi, p2), __fmul_rn(x.lo, p2)}; }

// x / y: the long-division form of the double-word quotient (Joldes, Muller and Popescu
// 2017, DWDivDW1): q1 = x.hi / y.hi, the remainder r = x - q1 y in double-word arithmetic
// (exact TwoProd of q1 y.hi), q2 = r.hi / y.hi; relative error about 2^-45.  The FP32
// divisions are IEEE round-to-nearest (__fdiv_rn).
__device__ __forceinline__ ff operator/(ff x, ff y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const float p = __fmul_rn(q1, y.hi);
    const float pe = __fmaf_rn(q1, y.hi, -p);          // q1 * y.hi = p + pe exactly
    const ff d = ff_two_sum(x.hi, -p);
    // remainder x - q1 y = (x.hi - p) - pe + x.lo - q1 y.lo
    const float r = __fadd_rn(d.hi, __fadd_rn(__fadd_rn(d.lo, -pe), __fmaf_rn(-q1, y.lo, x.lo)));
    const float q2 = __fdiv_rn(r, y.hi);
    return ff_fast2sum(q1, q2);
}

// sqrt(x) for x >= 0: s = sqrt(x.hi) (IEEE round to nearest), then one correction with
// the exact residual x - s^2 (TwoProd of s, s): s + (x - s^2) / (2 s) (Karp and Markstein,
// 1997); relative error about 2^-46.  x = 0 gives 0.
__device__ __forceinline__ ff ff_sqrt(ff x) {
    const float s = __fsqrt_rn(x.hi);
    if (s == 0.0f) return ff{0.0f, 0.0f};
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);                 // s^2 = p + pe exactly
    const float r = __fadd_rn(__fadd_rn(__fsub_rn(x.hi, p), -pe), x.lo);
    return ff_fast2sum(s, __fdiv_rn(r, __fadd_rn(s, s)));
}

// x < y, decided on the double-word value
__device__ __forceinline__ bool ff_less(ff x, ff y) {
    const ff d = x - y;
    return d.hi < 0.0f || (d.hi == 0.0f && d.lo < 0.0f);
}

// FP64 -> double word on the integer pipe only (selects, no FP64 instruction: GB300
// executes FP64 conversions on its narrow FP64 pipe, and a predicated fallback would still
// issue them).  hi is the FP64 significand truncated to 24 bits (the exponent rebased from
// 1023 to 127), lo the next 23 bits rounded to nearest, built exactly as
// (2^E + m ulp) - 2^E: |d - (hi + lo)| <= 2^-47 |d| for |d| in [2^-103, 2^128).
// Below 2^-103 lo is 0 (below 2^-126 hi too: the value flushes to a signed zero); at and
// above 2^128 hi is an infinity, NaN stays NaN.
__device__ __forceinline__ ff ff_from_f64(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned sgn = hw & 0x80000000u;
    const unsigned a = hw & 0x7fffffffu;
    const unsigned ed = a >> 20;
    unsigned hb = __funnelshift_l(lw, a - (896u << 20), 3);
    const bool nan = a > 0x7ff00000u || (a == 0x7ff00000u && lw != 0u);
    hb = ed < 897u ? 0u : (ed > 1150u ? (nan ? 0x7fc00000u : 0x7f800000u) : hb);
    const unsigned m = ((lw >> 6) & 0x7fffffu) + ((lw >> 5) & 1u);
    const unsigned eb = (ed - 919u) << 23;
    float lo = __fsub_rn(__uint_as_float(eb + m), __uint_as_float(eb));
    lo = (ed - 920u > 230u) ? 0.0f : lo;
    return ff{__uint_as_float(hb | sgn), __uint_as_float(__float_as_uint(lo) | sgn)};
}

// ff_from_f64 without its range selects, for |d| in [2^-103, 2^128) (biased FP64
// exponents 920..1150), where it returns the same hi and lo.  `span` collects
// max(biased exponent - 920) over the values split: a span above kFfInRangeSpan means one
// of them lay outside the range and its result is meaningless (split it again with
// ff_from_f64).  Populations of a running simulation always lie inside, so a collision
// sweep splits its 19 loads this way and takes the general split only on that rare span.
constexpr unsigned kFfInRangeSpan = 230u;
__device__ __forceinline__ ff ff_from_f64_in_range(double d, unsigned &span) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned sgn = hw & 0x80000000u;
    const unsigned a = hw & 0x7fffffffu;
    const unsigned ed = a >> 20;
    span = span > ed - 920u ? span : ed - 920u;
    const unsigned hb = __funnelshift_l(lw, a - (896u << 20), 3);
    const unsigned m = ((lw >> 6) & 0x7fffffu) + ((lw >> 5) & 1u);
    const unsigned eb = (ed - 919u) << 23;
    const float lo = __fsub_rn(__uint_as_float(eb + m), __uint_as_float(eb));
    return ff{__uint_as_float(hb | sgn), __uint_as_float(__float_as_uint(lo) | sgn)};
}

// FP32 -> FP64 exactly on the integer pipe (selects only): normal numbers exactly, zero and
// FP32 subnormals (below 2^-126) as a signed zero, infinities and NaN kept
__device__ __forceinline__ double f64_of_f32(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned a = u & 0x7fffffffu;
    unsigned h = (a >> 3) + (896u << 20);
    h = a < 0x00800000u ? 0u : (a >= 0x7f800000u ? (0x7ff00000u | (a >> 3)) : h);
    const unsigned l = a < 0x00800000u ? 0u : (u << 29);
    return __hiloint2double((int)(h | (u & 0x80000000u)), (int)l);
}

// double word -> FP64: both parts exact, one FP64 add rounds the sum to nearest
__device__ __forceinline__ double f64_of_ff(ff x) { return __dadd_rn(f64_of_f32(x.hi), f64_of_f32(x.lo)); }
#endif

}  // namespace mflbm
