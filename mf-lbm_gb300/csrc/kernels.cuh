// kernels.cuh -- sm_103a kernels of the per-step lattice update.
//
// This header is compiled twice, once per floating-point flavour, inside namespace
// mflbm::MFLBM_NS:
//   kernels_fast.cu    (MFLBM_NS = fast)   default nvcc contraction of a*b+c into FMA
//   kernels_strict.cu  (MFLBM_NS = strict) --fmad=false: every operation rounds on its
//                      own, in the reference's written order, so results are
//                      bit-identical to an IEEE FP64 restatement of the Fortran.
// The host layer picks the flavour per context (mflbm_params.strict_fp).
#pragma once
#include <type_traits>
#include "bulk.cuh"
#include "common.cuh"
#include "kernels_api.h"

namespace mflbm {
namespace MFLBM_NS {

// ---------------------------------------------------------------------------------
// constants (multiphase_3D/0.src/Module.F90:116-131, 225-227)
// ---------------------------------------------------------------------------------
constexpr double mrt_coef1 = 1.0 / 19.0;
constexpr double mrt_coef2 = 1.0 / 2394.0;
constexpr double mrt_coef3 = 1.0 / 252.0;
constexpr double mrt_coef4 = 1.0 / 72.0;
constexpr double mrt_e2_coef1 = 0.0;
constexpr double mrt_e2_coef2 = -475.0 / 63.0;
constexpr double mrt_omega_xx = 0.0;
constexpr double w_equ_0 = 1.0 / 3.0;
constexpr double w_equ_1 = 1.0 / 18.0;
constexpr double w_equ_2 = 1.0 / 36.0;
constexpr double ISO4_1 = 1.0 / 6.0;
constexpr double ISO4_2 = 1.0 / 12.0;

__host__ __device__ constexpr double WEQ(int q) { return q == 0 ? w_equ_0 : (q <= 6 ? w_equ_1 : w_equ_2); }
// Rest state of the reference MRT (its equilibrium energy-square moment is 0, so the
// rest distribution is 4/21, 13/126, 1/63 rather than the BGK weights).  FP16 storage
// keeps deviations from this state so that a fluid at rest stores zeros.
__host__ __device__ constexpr double WREST(int q) { return q == 0 ? 4.0 / 21.0 : (q <= 6 ? 13.0 / 126.0 : 1.0 / 63.0); }

// direction tables for run-time q (boundary-node lists): offsets and weight class
// (0 rest, 1 axis, 2 diagonal); indexed 0..18
static __constant__ signed char c_ex[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static __constant__ signed char c_ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static __constant__ signed char c_ez[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static __constant__ signed char c_opp[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
__device__ __forceinline__ int OPP_RT(int q) { return c_opp[q]; }

// neighbour offset of direction q in the padded PDF layout
__device__ __forceinline__ int64_t qoff(const Layout &L, int q) {
    return (int64_t)EX(q) + (int64_t)EY(q) * L.pitch + (int64_t)EZ(q) * L.pz;
}

// ---------------------------------------------------------------------------------
// PDF storage types.
//   double  FP64 value (the plain drop-in)
//   float   FP32 value (multiphase mixed form: a vanishing species makes deviations
//           from a rest state no smaller than the values)
//   dfloat  FP32 deviation d = f_q - w_q * ref from the MRT rest state (singlephase
//           mixed form)
//   __half  FP16 scaled deviation (f_q - w_q * ref) * scale (singlephase)
// ld/st work on values (boundary conditions); ldd/std on deviations, which is how the
// singlephase sweep of the deviation forms runs its collision: the rest state W is a
// fixed point of the reference's MRT collision C, which is affine in f apart from
// terms in the momentum j (W carries none) and the force, so C(W + d) - W is the same
// code applied to d with density sum(d).  Arithmetic on d keeps FP32's 24 bits for the
// ~1e-6 signal of a creeping flow instead of spending them on the ~0.1 of f.
// ld64/st64 convert to and from FP64 without passing through an FP32 value.
// ---------------------------------------------------------------------------------
struct dfloat { float x; };

template <class S> struct Store;
template <> struct Store<double> {
    using R = double;
    using RS = R;   // arithmetic type of the collision sweep
    static constexpr bool kDev = false;
    __device__ __forceinline__ static R ld(const double *p, int64_t o, R, R) { return p[o]; }
    __device__ __forceinline__ static void st(double *p, int64_t o, R v, R, R) { p[o] = v; }
    __device__ __forceinline__ static R ldd(const double *p, int64_t o, R) { return p[o]; }
    __device__ __forceinline__ static void std_(double *p, int64_t o, R v, R) { p[o] = v; }
    __device__ __forceinline__ static double ld64(const double *p, int64_t o, double, float) { return p[o]; }
    __device__ __forceinline__ static void st64(double *p, int64_t o, double v, double, float) { p[o] = v; }
};
template <> struct Store<float> {
    using R = float;
    using RS = R;   // arithmetic type of the collision sweep
    static constexpr bool kDev = false;
    __device__ __forceinline__ static R ld(const float *p, int64_t o, R, R) { return p[o]; }
    __device__ __forceinline__ static void st(float *p, int64_t o, R v, R, R) { p[o] = v; }
    __device__ __forceinline__ static R ldd(const float *p, int64_t o, R) { return p[o]; }
    __device__ __forceinline__ static void std_(float *p, int64_t o, R v, R) { p[o] = v; }
    __device__ __forceinline__ static double ld64(const float *p, int64_t o, double, float) { return (double)p[o]; }
    __device__ __forceinline__ static void st64(float *p, int64_t o, double v, double, float) { p[o] = (float)v; }
};
template <> struct Store<dfloat> {
    using R = float;
    using RS = R;   // arithmetic type of the collision sweep
    static constexpr bool kDev = true;
    __device__ __forceinline__ static R ld(const dfloat *p, int64_t o, R w_ref, R) { return w_ref + p[o].x; }
    __device__ __forceinline__ static void st(dfloat *p, int64_t o, R v, R w_ref, R) { p[o].x = v - w_ref; }
    __device__ __forceinline__ static R ldd(const dfloat *p, int64_t o, R) { return p[o].x; }
    __device__ __forceinline__ static void std_(dfloat *p, int64_t o, R d, R) { p[o].x = d; }
    __device__ __forceinline__ static double ld64(const dfloat *p, int64_t o, double w_ref, float) {
        return w_ref + (double)p[o].x;
    }
    __device__ __forceinline__ static void st64(dfloat *p, int64_t o, double v, double w_ref, float) {
        p[o].x = (float)(v - w_ref);
    }
};
template <> struct Store<__half> {
    using R = float;
    using RS = R;
    static constexpr bool kDev = true;
    // w_ref = w_q * ref density; sc = scale (store) / 1/scale (load)
    __device__ __forceinline__ static R ld(const __half *p, int64_t o, R w_ref, R inv_scale) {
        return w_ref + __half2float(p[o]) * inv_scale;
    }
    __device__ __forceinline__ static void st(__half *p, int64_t o, R v, R w_ref, R scale) {
        p[o] = __float2half_rn((v - w_ref) * scale);
    }
    __device__ __forceinline__ static R ldd(const __half *p, int64_t o, R inv_scale) { return __half2float(p[o]) * inv_scale; }
    __device__ __forceinline__ static void std_(__half *p, int64_t o, R d, R scale) { p[o] = __float2half_rn(d * scale); }
    __device__ __forceinline__ static double ld64(const __half *p, int64_t o, double w_ref, float inv_scale) {
        return w_ref + (double)__half2float(p[o]) * (double)inv_scale;
    }
    __device__ __forceinline__ static void st64(__half *p, int64_t o, double v, double w_ref, float scale) {
        p[o] = __float2half_rn((float)((v - w_ref) * (double)scale));
    }
};

// f64ff: FP64 storage whose collision sweep computes in double-word arithmetic on the
// FP32 pipe (ffloat.cuh); the sweep converts on load and store.  Every other kernel of
// this form runs on the storage as `double`.
struct f64ff { double v; };
template <> struct Store<f64ff> {
    using R = ff;
    using RS = ff;
    static constexpr bool kDev = false;
};

// ffs: double-word storage (two FP32 per population, hi + lo, about 48 significant bits;
// 8 bytes like FP64), collision in double-word arithmetic without any conversion in the
// sweep.  The boundary, monitor, initialisation and conversion kernels see FP64 values
// (one FP64 add to join a pair, integer operations to split one).
struct __align__(8) ffs { float hi, lo; };
template <> struct Store<ffs> {
    using R = double;
    using RS = ff;
    static constexpr bool kDev = false;
    __device__ __forceinline__ static R ld(const ffs *p, int64_t o, R, R) {
        const ffs v = p[o];
        return f64_of_ff(ff{v.hi, v.lo});
    }
    __device__ __forceinline__ static void st(ffs *p, int64_t o, R v, R, R) {
        const ff x = ff_from_f64(v);
        p[o] = ffs{x.hi, x.lo};
    }
    __device__ __forceinline__ static R ldd(const ffs *p, int64_t o, R) { return ld(p, o, R(0), R(0)); }
    __device__ __forceinline__ static void std_(ffs *p, int64_t o, R v, R) { st(p, o, v, R(0), R(0)); }
    __device__ __forceinline__ static double ld64(const ffs *p, int64_t o, double, float) { return ld(p, o, 0.0, 0.0); }
    __device__ __forceinline__ static void st64(ffs *p, int64_t o, double v, double, float) { st(p, o, v, 0.0, 0.0); }
};

// Resident 128-thread blocks per SM that the sweep kernels ask the register allocator
// for.  The double-word storage sweep issues about 1,500 instructions per node and waits
// on memory between them: its natural 96 registers leave 5 blocks per SM; a cap of 72
// registers gives 7 at about 70 bytes of spill, measured 7 % faster on GB300 (5 / 6 / 7
// blocks: 14.0 / 14.5 / 15.0 GLUPS on a 256^3 packing).  Since the even step runs through
// the TMA kernel, the cap acts on the odd step (and the dense sweep): 5 / 6 / 7 / 8 blocks
// gave 14,778 / 15,094 / 15,800 / 15,498 MLUPS.  The FP64-storage double-word sweep is
// issue-bound and gained nothing; the other forms keep the allocator's choice.
#ifndef MFLBM_FF_MIN_BLOCKS
#define MFLBM_FF_MIN_BLOCKS 7
#endif
template <class S> struct SweepOcc { static constexpr int kMinBlocks = 1; };
template <> struct SweepOcc<ffs> { static constexpr int kMinBlocks = MFLBM_FF_MIN_BLOCKS; };

// load/store of the collision sweep: deviations for the deviation forms, values else
template <class S>
__device__ __forceinline__ typename Store<S>::RS ld_sweep(const S *p, int64_t o, int q, typename Store<S>::RS inv) {
    using R = typename Store<S>::RS;
    if constexpr (std::is_same<S, f64ff>::value) return ff_from_f64(p[o].v);
    else if constexpr (std::is_same<S, ffs>::value) { const ffs v = p[o]; return ff{v.hi, v.lo}; }
    else if constexpr (Store<S>::kDev) return Store<S>::ldd(p, o, inv);
    else return Store<S>::ld(p, o, R(WREST(q)), inv);
}
template <class S>
__device__ __forceinline__ void st_sweep(S *p, int64_t o, int q, typename Store<S>::RS v, typename Store<S>::RS sc) {
    using R = typename Store<S>::RS;
    if constexpr (std::is_same<S, f64ff>::value) p[o].v = f64_of_ff(v);
    else if constexpr (std::is_same<S, ffs>::value) {
        const ff n = ff_fast2sum(v.hi, v.lo);   // stored normalised
        p[o] = ffs{n.hi, n.lo};
    }
    else if constexpr (Store<S>::kDev) Store<S>::std_(p, o, v, sc);
    else Store<S>::st(p, o, v, R(WREST(q)), sc);
}

// the 19 loads of one node's collision, slot of population q at addr(q).  FP64 storage
// split for the double-word collision (f64ff): the select-free split of the common range,
// and, if any population lies outside it, all 19 read again and split by the general
// form (nothing has been written yet, so the second read sees the same values).
template <class S, class Addr>
__device__ __forceinline__ void ld_node(typename Store<S>::RS (&ft)[19], const S *p, Addr addr,
                                        typename Store<S>::RS inv) {
    if constexpr (std::is_same<S, f64ff>::value) {
        unsigned span = 0u;
#pragma unroll
        for (int q = 0; q < 19; ++q) ft[q] = ff_from_f64_in_range(p[addr(q)].v, span);
        if (__builtin_expect(span > kFfInRangeSpan, 0)) {
            // a pointer the compiler cannot equate with p, so the first loads are not kept
            // live for this path
            const S *p2 = p;
            asm volatile("" : "+l"(p2) : "r"(span));
#pragma unroll
            for (int q = 0; q < 19; ++q) ft[q] = ff_from_f64(p2[addr(q)].v);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) ft[q] = ld_sweep<S>(p, addr(q), q, inv);
    }
}

// ---------------------------------------------------------------------------------
// MRT collision, the "MRT kernel, repeated part" of the reference
// (multiphase_3D/0.src/Kernel_multiphase.F90:158-267, singlephase Kernel.F90:60-169),
// in the written operation order.
// ---------------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void mrt_collide(R (&ft)[19], R den, R fx, R fy, R fz, R s_e, R s_e2, R s_q, R s_nu, R s_pi,
                                            R s_t) {
    const R ux = ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] + R(0.5) * fx;
    const R uy = ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] + R(0.5) * fy;
    const R uz = ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] + R(0.5) * fz;
    const R u2 = ux * ux + uy * uy + uz * uz;

    R sum1 = ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6];
    R sum2 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
    R sum3 = ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14];
    R sum4 = ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    R sum5 = ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18];
    R sum6 = R(2.0) * (ft[1] + ft[2]) - ft[3] - ft[4] - ft[5] - ft[6];
    R sum7 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] - R(2.0) * (ft[15] + ft[16] + ft[17] + ft[18]);
    R sum8 = ft[3] + ft[4] - ft[5] - ft[6];
    R sum9 = ft[7] + ft[8] + ft[9] + ft[10] - ft[11] - ft[12] - ft[13] - ft[14];

    R m_rho = den;
    R m_e = R(-30.0) * ft[0] - R(11.0) * sum1 + R(8.0) * sum2;
    R m_e2 = R(12.0) * ft[0] - R(4.0) * sum1 + sum2;
    R m_jx = ft[1] - ft[2] + sum3;
    R m_qx = R(-4.0) * (ft[1] - ft[2]) + sum3;
    R m_jy = ft[3] - ft[4] + sum4;
    R m_qy = R(-4.0) * (ft[3] - ft[4]) + sum4;
    R m_jz = ft[5] - ft[6] + sum5;
    R m_qz = R(-4.0) * (ft[5] - ft[6]) + sum5;
    R m_3pxx = sum6 + sum7;
    R m_3pixx = R(-2.0) * sum6 + sum7;
    R m_pww = sum8 + sum9;
    R m_piww = R(-2.0) * sum8 + sum9;
    R m_pxy = ft[7] - ft[8] - ft[9] + ft[10];
    R m_pyz = ft[15] - ft[16] - ft[17] + ft[18];
    R m_pzx = ft[11] - ft[12] - ft[13] + ft[14];
    R m_tx = ft[7] - ft[8] + ft[9] - ft[10] - ft[11] + ft[12] - ft[13] + ft[14];
    R m_ty = -ft[7] - ft[8] + ft[9] + ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    R m_tz = ft[11] + ft[12] - ft[13] - ft[14] - ft[15] - ft[16] + ft[17] + ft[18];

    const R c23 = R(-0.666666666666666667);
    const R c13 = R(0.333333333333333333);
    m_e = m_e - s_e * (m_e - (R(-11.0) * den + R(19.0) * u2)) + (R(38.0) - R(19.0) * s_e) * (fx * ux + fy * uy + fz * uz);
    m_e2 = m_e2 - s_e2 * (m_e2 - (R(mrt_e2_coef1) * den + R(mrt_e2_coef2) * u2)) +
           (R(-11.0) + R(5.5) * s_e2) * (fx * ux + fy * uy + fz * uz);
    m_jx = m_jx + fx;
    m_qx = m_qx - s_q * (m_qx - (c23 * ux)) + (c23 + c13 * s_q) * fx;
    m_jy = m_jy + fy;
    m_qy = m_qy - s_q * (m_qy - (c23 * uy)) + (c23 + c13 * s_q) * fy;
    m_jz = m_jz + fz;
    m_qz = m_qz - s_q * (m_qz - (c23 * uz)) + (c23 + c13 * s_q) * fz;

    m_3pxx = m_3pxx - s_nu * (m_3pxx - (R(3.0) * ux * ux - u2)) + (R(2.0) - s_nu) * (R(2.0) * fx * ux - fy * uy - fz * uz);
    m_3pixx = m_3pixx - s_pi * (m_3pixx - R(mrt_omega_xx) * (R(3.0) * ux * ux - u2)) +
              (R(1.0) - R(0.5) * s_pi) * (R(-2.0) * fx * ux + fy * uy + fz * uz);
    m_pww = m_pww - s_nu * (m_pww - (uy * uy - uz * uz)) + (R(2.0) - s_nu) * (fy * uy - fz * uz);
    m_piww = m_piww - s_pi * (m_piww - R(mrt_omega_xx) * (uy * uy - uz * uz)) + (R(1.0) - R(0.5) * s_pi) * (-fy * uy + fz * uz);
    m_pxy = m_pxy - s_nu * (m_pxy - (ux * uy)) + (R(1.0) - R(0.5) * s_nu) * (fx * uy + fy * ux);
    m_pyz = m_pyz - s_nu * (m_pyz - (uy * uz)) + (R(1.0) - R(0.5) * s_nu) * (fy * uz + fz * uy);
    m_pzx = m_pzx - s_nu * (m_pzx - (ux * uz)) + (R(1.0) - R(0.5) * s_nu) * (fx * uz + fz * ux);
    m_tx = m_tx - s_t * (m_tx);
    m_ty = m_ty - s_t * (m_ty);
    m_tz = m_tz - s_t * (m_tz);

    m_rho = R(mrt_coef1) * m_rho;
    m_e = R(mrt_coef2) * m_e;
    m_e2 = R(mrt_coef3) * m_e2;
    m_jx = R(0.1) * m_jx;
    m_qx = R(0.025) * m_qx;
    m_jy = R(0.1) * m_jy;
    m_qy = R(0.025) * m_qy;
    m_jz = R(0.1) * m_jz;
    m_qz = R(0.025) * m_qz;
    m_3pxx = R(2.0 * mrt_coef4) * m_3pxx;
    m_3pixx = R(mrt_coef4) * m_3pixx;
    m_pww = R(6.0 * mrt_coef4) * m_pww;
    m_piww = R(3.0 * mrt_coef4) * m_piww;
    m_pxy = R(0.25) * m_pxy;
    m_pyz = R(0.25) * m_pyz;
    m_pzx = R(0.25) * m_pzx;
    m_tx = R(0.125) * m_tx;
    m_ty = R(0.125) * m_ty;
    m_tz = R(0.125) * m_tz;
    sum1 = m_rho - R(11.0) * m_e - R(4.0) * m_e2;
    sum2 = R(2.0) * m_3pxx - R(4.0) * m_3pixx;
    sum3 = m_pww - R(2.0) * m_piww;
    sum4 = m_rho + R(8.0) * m_e + m_e2;
    sum5 = m_jx + m_qx;
    sum6 = m_jy + m_qy;
    sum7 = m_jz + m_qz;
    sum8 = m_3pxx + m_3pixx;
    sum9 = m_pww + m_piww;

    ft[0] = m_rho - R(30.0) * m_e + R(12.0) * m_e2;
    ft[1] = sum1 + m_jx - R(4.0) * m_qx + sum2;
    ft[2] = sum1 - m_jx + R(4.0) * m_qx + sum2;
    ft[3] = sum1 + m_jy - R(4.0) * m_qy - R(0.5) * sum2 + sum3;
    ft[4] = sum1 - m_jy + R(4.0) * m_qy - R(0.5) * sum2 + sum3;
    ft[5] = sum1 + m_jz - R(4.0) * m_qz - R(0.5) * sum2 - sum3;
    ft[6] = sum1 - m_jz + R(4.0) * m_qz - R(0.5) * sum2 - sum3;
    ft[7] = sum4 + sum5 + sum6 + sum8 + sum9 + m_pxy + m_tx - m_ty;
    ft[8] = sum4 - sum5 + sum6 + sum8 + sum9 - m_pxy - m_tx - m_ty;
    ft[9] = sum4 + sum5 - sum6 + sum8 + sum9 - m_pxy + m_tx + m_ty;
    ft[10] = sum4 - sum5 - sum6 + sum8 + sum9 + m_pxy - m_tx + m_ty;
    ft[11] = sum4 + sum5 + sum7 + sum8 - sum9 + m_pzx - m_tx + m_tz;
    ft[12] = sum4 - sum5 + sum7 + sum8 - sum9 - m_pzx + m_tx + m_tz;
    ft[13] = sum4 + sum5 - sum7 + sum8 - sum9 - m_pzx - m_tx - m_tz;
    ft[14] = sum4 - sum5 - sum7 + sum8 - sum9 + m_pzx + m_tx - m_tz;
    ft[15] = sum4 + sum6 + sum7 - sum8 * R(2.0) + m_pyz + m_ty - m_tz;
    ft[16] = sum4 - sum6 + sum7 - sum8 * R(2.0) - m_pyz - m_ty - m_tz;
    ft[17] = sum4 + sum6 - sum7 - sum8 * R(2.0) - m_pyz + m_ty + m_tz;
    ft[18] = sum4 - sum6 - sum7 - sum8 * R(2.0) + m_pyz - m_ty + m_tz;
}

#include "collide.cuh"

// ---------------------------------------------------------------------------------
// singlephase kernel_even / kernel_odd (singlephase_3D/0.src/Kernel.F90:5-400).
// One thread per interior node; solid nodes are skipped, so their slots carry the
// implicit full-way bounce-back of the AA pattern.
// odd : ft_q <- f_q(x - e_q) ... f_opp(q)(x + e_q) <- ft_q
// even: ft_q <- f_opp(q)(x)  ... f_q(x) <- ft_q
// ---------------------------------------------------------------------------------
template <class S, bool ODD, bool UNIT>
__global__ void __launch_bounds__(128, SweepOcc<S>::kMinBlocks) k_sp_step(S *__restrict__ f, const int32_t *__restrict__ cells, const int ncell,
                                                 const Layout L, const StepParams P,
                                                 const MrtFold<typename Store<S>::RS> cf, const float scale) {
    using St = Store<S>;
    using R = typename St::RS;
    // one thread per fluid node: the sorted fluid-cell list keeps every lane busy
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) return;
    const int64_t c = cells[t];
    const R inv_scale = R(1.0f / scale);
    R ft[19];
    ld_node<S>(ft, f, [&](int q) -> int64_t {
        return ODD ? (int64_t)q * L.qs + c - qoff(L, q) : (int64_t)OPP(q) * L.qs + c;
    }, inv_scale);
    if constexpr (std::is_same<R, ff>::value) {
        mrt_collide_ff<UNIT>(ft, cf);
    } else {
#ifdef MFLBM_STRICT
        const R den = ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] + ft[11] +
                      ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
        mrt_collide<R>(ft, den, R(0.0), R(0.0), R(P.force_z), R(P.s_e), R(P.s_e2), R(P.s_q), R(P.s_nu), R(P.s_pi),
                       R(P.s_t));
#else
        // force_z travels in the same coefficient set, already converted to R on the host
        mrt_collide_pairs<R, false, true, UNIT>(ft, R(0.0), R(0.0), R(0.0), cf.fz, cf);
#endif
    }
    const R sc = R(scale);
    if (ODD) {
        st_sweep<S>(f, c, 0, ft[0], sc);
#pragma unroll
        for (int q = 1; q < 19; ++q) st_sweep<S>(f, (int64_t)OPP(q) * L.qs + c + qoff(L, q), q, ft[q], sc);
    } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) st_sweep<S>(f, (int64_t)q * L.qs + c, q, ft[q], sc);
    }
}

// ---------------------------------------------------------------------------------
// multiphase kernel_even_color / kernel_odd_color
// (multiphase_3D/0.src/Kernel_multiphase.F90:6-725): total-PDF MRT collision with the
// CSF force, viscosity interpolation in 1/nu, R-K recolouring into f (fluid 1) and
// g (fluid 2), phi written for the gradient pass.
// ---------------------------------------------------------------------------------
// The fluid-list even steps walk the nodes from the last to the first, the odd steps from
// the first to the last: each sweep starts on the nodes the previous one touched last,
// whose slots are still in L2.  Only the order of independent node updates changes.
#ifndef MFLBM_EVEN_REVERSE
#define MFLBM_EVEN_REVERSE 1
#endif
// the list node of this thread: block order reversed on even steps
template <bool ODD>
__device__ __forceinline__ int list_node_index() {
    const int b = (!ODD && MFLBM_EVEN_REVERSE) ? (int)(gridDim.x - 1 - blockIdx.x) : (int)blockIdx.x;
    return b * (int)blockDim.x + (int)threadIdx.x;
}

// T = double: the FP64 drop-in; T = float: the mixed form (FP32 storage of f, g, phi
// and the gradient fields, FP32 arithmetic).
// The node of a multiphase collision thread and the slots of its populations: the dense
// planes (cells[t] is the padded-layout index; pull from c - e_q on odd steps) or the fluid
// list (cells[t] is the halo-1 index of fluid node t; nb[d-1][t] is the slot of t + e_d).
// Defines c, i, j, k and the slot functions src(q) (read) and dst(q) (write, q >= 1).
#define MP_NODE_ADDRESSING                                                                          \
    int64_t c;                                                                                      \
    int i, j, k;                                                                                    \
    int32_t nbr[18];                                                                                \
    if constexpr (LIST) {                                                                           \
        c = t;                                                                                      \
        const int64_t h = cells[t];                                                                 \
        k = (int)(h / L.h1xy);                                                                      \
        const int64_t r_ = h - (int64_t)k * L.h1xy;                                                 \
        j = (int)(r_ / L.h1x);                                                                      \
        i = (int)(r_ - (int64_t)j * L.h1x);                                                         \
        if constexpr (ODD) {                                                                        \
            _Pragma("unroll") for (int d = 0; d < 18; ++d) nbr[d] = nb[(int64_t)d * ncell + t];     \
        }                                                                                           \
    } else {                                                                                        \
        c = cells[t];                                                                               \
        k = (int)(c / L.pz);                                                                        \
        const int64_t r_ = c - (int64_t)k * L.pz;                                                   \
        j = (int)(r_ / L.pitch);                                                                    \
        i = (int)(r_ - (int64_t)j * L.pitch) - L.xo;                                                \
        (void)nbr;                                                                                  \
    }                                                                                               \
    auto src = [&](int q) -> int64_t {                                                              \
        if constexpr (LIST && ODD)                                                                  \
            return q == 0 ? c : (int64_t)q * stride + nbr[OPP(q) - 1];                             \
        else if constexpr (LIST)                                                                    \
            return (int64_t)OPP(q) * stride + c;                                                    \
        else                                                                                        \
            return ODD ? (int64_t)q * L.qs + c - qoff(L, q) : (int64_t)OPP(q) * L.qs + c;           \
    };                                                                                              \
    auto dst = [&](int q) -> int64_t {                                                              \
        if constexpr (LIST && ODD)                                                                  \
            return (int64_t)OPP(q) * stride + nbr[q - 1];                                           \
        else if constexpr (LIST)                                                                    \
            return (int64_t)q * stride + c;                                                         \
        else                                                                                        \
            return ODD ? (int64_t)OPP(q) * L.qs + c + qoff(L, q) : (int64_t)q * L.qs + c;           \
    };

// Resident blocks per SM (128 threads each) the compiler must allow for the multiphase
// collision, i.e. its register cap.  FP32: 6 (at most 80 registers; the fluid-list odd step,
// which preloads its 18 table entries, spills 36 bytes).  With the normals read as one
// record, the sweep 4/5/6 gave 0.648 / 0.678 / 0.701 of the roofline on the C3 packing
// (without them 1/4/5/6: 0.579 / 0.646 / 0.691 / 0.689).  FP64: 3 (FP64-pipe bound; 4 and
// above spill).  The FP32 even step, which computes the curvature from the normal records
// (fused) and has no neighbour table, takes its own cap: 5 blocks (96 registers) against
// 4 / 6 / 7 gave C3 256^2 x 320 FP32 8,841 against 8,739 / 8,722 / 8,704 MLUPS with the odd
// step at 6.  Tuning parameters: MFLBM_NVCC_FLAGS=-DMFLBM_MP_MIN_BLOCKS_F32=n (odd step),
// -DMFLBM_MP_MIN_BLOCKS_F32_EVEN=n.
#ifndef MFLBM_MP_MIN_BLOCKS_F32
#define MFLBM_MP_MIN_BLOCKS_F32 6
#endif
#ifndef MFLBM_MP_MIN_BLOCKS_F64
#define MFLBM_MP_MIN_BLOCKS_F64 3
#endif
#ifndef MFLBM_MP_MIN_BLOCKS_F32_EVEN
#define MFLBM_MP_MIN_BLOCKS_F32_EVEN 5
#endif
template <class T, bool ODD> struct MpOcc { static constexpr int kMinBlocks = MFLBM_MP_MIN_BLOCKS_F64; };
template <> struct MpOcc<float, true> { static constexpr int kMinBlocks = MFLBM_MP_MIN_BLOCKS_F32; };
template <> struct MpOcc<float, false> { static constexpr int kMinBlocks = MFLBM_MP_MIN_BLOCKS_F32_EVEN; };

// curvature of one cell from accessors of cn_x, cn_y, cn_z (defined with the gradient kernels)
template <class T, class FX, class FY, class FZ>
__device__ __forceinline__ T curvature_of(FX X, FY Y, FZ Z);

// FUSE: the node's curvature is computed here from the 19 normal records around it (the
// expression of the curvature kernels, so the same value) instead of read from curv, which
// the colour-gradient pass then leaves unwritten
template <class T, bool ODD, bool LIST = false, bool FUSE = false>
__global__ void __launch_bounds__(128, MpOcc<T, ODD>::kMinBlocks) k_mp_step(T *__restrict__ f, T *__restrict__ g, T *__restrict__ phi,
                                                 const Nrm<T> *__restrict__ cn,
                                                 const T *__restrict__ curv, const int32_t *__restrict__ cells,
                                                 const int ncell, const Layout L, const StepParams P, const double rk_weight2,
                                                 const int32_t *__restrict__ nb = nullptr, const int64_t stride = 0) {
    const int t = LIST ? list_node_index<ODD>() : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= ncell) return;
    MP_NODE_ADDRESSING
    const int64_t w2 = L.i2(i, j, k);
    T ft[19];
    T rho1 = T(0.0), rho2 = T(0.0);
    // pull (odd) or local swapped read (even); rho1/rho2 accumulate in the written order
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const T a = f[src(q)];
        ft[q] = a;
        rho1 = q == 0 ? a : rho1 + a;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const T b = g[src(q)];
        ft[q] = ft[q] + b;
        rho2 = q == 0 ? b : rho2 + b;
    }
#ifdef MFLBM_STRICT
    const T ph = (rho1 - rho2) / (rho1 + rho2);
#else
    const T inv_den = T(1.0) / (rho1 + rho2);   // one division serves phi and the recolouring
    const T ph = (rho1 - rho2) * inv_den;
#endif
    phi[L.i4(i, j, k)] = ph;
    const Nrm<T> nr = cn[w2];
    const T cx = nr.x, cy = nr.y, cz = nr.z;
    T kap;
    if constexpr (FUSE) {
        auto X = [&](int a, int b, int c) { return cn[w2 + a + L.h2x * b + L.h2xy * c].x; };
        auto Y = [&](int a, int b, int c) { return cn[w2 + a + L.h2x * b + L.h2xy * c].y; };
        auto Z = [&](int a, int b, int c) { return cn[w2 + a + L.h2x * b + L.h2xy * c].z; };
        kap = curvature_of<T>(X, Y, Z);
    } else {
        kap = curv[L.i1(i, j, k)];
    }
    T tmp = T(0.5) * T(P.gamma) * kap * nr.n;
    const T fx = tmp * cx;
    const T fy = tmp * cy;
    const T fz = tmp * cz + T(P.force_z);
    const T nui1 = T(P.la_nui1), nui2 = T(P.la_nui2);
#ifdef MFLBM_STRICT
    const T omega = T(1.0) / (T(6.0) / ((T(1.0) + ph) * nui1 + (T(1.0) - ph) * nui2) + T(0.5));
#else
    // 1/(6/X + 1/2) = X / (6 + X/2): one division
    const T visc = (T(1.0) + ph) * nui1 + (T(1.0) - ph) * nui2;
    const T omega = visc / (T(6.0) + T(0.5) * visc);
#endif
    const T den = rho1 + rho2;
#ifdef MFLBM_STRICT
    T s_e, s_e2, s_pi, s_q, s_t;
    if (P.mrt == 1) {
        s_e = omega; s_e2 = omega; s_pi = omega;
        s_q = T(8.0) * (T(2.0) - omega) / (T(8.0) - omega);
        s_t = s_q;
    } else if (P.mrt == 3) {
        s_e = omega; s_e2 = omega; s_pi = omega; s_q = omega; s_t = omega;
    } else if (P.mrt == 4) {
        s_e = omega; s_e2 = omega; s_pi = omega;
        s_q = (T(6.0) - T(3.0) * omega) / (T(3.0) - omega);
        s_t = omega;
    } else {
        s_e = T(1.19); s_e2 = T(1.4); s_pi = T(1.4); s_q = T(1.2); s_t = T(1.98);
    }
    mrt_collide<T>(ft, den, fx, fy, fz, s_e, s_e2, s_q, omega, s_pi, s_t);
#else
    // rates of Kernel_multiphase.F90:124-155; each branch folds its literal rates
    MrtFold<T> cf;
    if (P.mrt == 1) {
        const T sq = T(8.0) * (T(2.0) - omega) / (T(8.0) - omega);
        cf = fold_rates_dev<T>(omega, omega, sq, omega, omega, sq);
    } else if (P.mrt == 3) {
        cf = fold_rates_dev<T>(omega, omega, omega, omega, omega, omega);
    } else if (P.mrt == 4) {
        const T sq = (T(6.0) - T(3.0) * omega) / (T(3.0) - omega);
        cf = fold_rates_dev<T>(omega, omega, sq, omega, omega, omega);
    } else {
        cf = fold_rates_dev<T>(T(1.19), T(1.4), T(1.2), omega, T(1.4), T(1.98));
    }
    mrt_collide_pairs<T, true, false>(ft, den, fx, fy, fz, cf);
#endif
    // recolouring (Kernel_multiphase.F90:272-315)
#ifdef MFLBM_STRICT
    const T tmp1 = rho1 / den;
    tmp = rho1 * rho2 * T(P.beta) / den;
#else
    const T tmp1 = rho1 * inv_den;
    tmp = rho1 * rho2 * T(P.beta) * inv_den;
#endif
    f[c] = tmp1 * ft[0];
    g[c] = ft[0] * (T(1.0) - tmp1);
    const T rkw2 = T(rk_weight2);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const T ex = (T)EX(q), ey = (T)EY(q), ez = (T)EZ(q);
        T proj;
        // the reference writes each projection as a signed sum of the two non-zero
        // components in x, y, z order, e.g. (-cnx + cny)
        if (q <= 6)
            proj = EX(q) != 0 ? ex * cx : (EY(q) != 0 ? ey * cy : ez * cz);
        else if (EZ(q) == 0)
            proj = ex * cx + ey * cy;
        else if (EY(q) == 0)
            proj = ex * cx + ez * cz;
        else
            proj = ey * cy + ez * cz;
        const T wq = q <= 6 ? T(w_equ_1) : rkw2;
        const T a = tmp1 * ft[q] + wq * tmp * (proj);
        const T b = ft[q] - a;
        const int64_t o = dst(q);
        f[o] = a;
        g[o] = b;
    }
}

// The multiphase collision of the double-word form (MFLBM_FP64FF): FP64 storage of f, g,
// phi and the gradient fields, arithmetic in FP32 pairs (ffloat.cuh).  The operations are
// k_mp_step's default build, term for term: phi and the recolouring weights from one
// reciprocal of the density, the CSF force, the per-node viscosity and MRT rates folded by
// fold_rates_dev, the pair-form MRT collision with a general force, the recolouring.  Each
// FP64 value is split on load and joined on store (one FP64 add), so the FP64 pipe carries
// 39 adds per node instead of the whole collision.
// S: double (MFLBM_FP64FF, FP64 storage split on load and joined on store) or ffs
// (MFLBM_FF, the double-word pairs stored as they are, renormalised on store)
template <bool ODD, class S = double, bool LIST = false>
__global__ void __launch_bounds__(128, 4) k_mp_step_ff(S *__restrict__ f, S *__restrict__ g,
                                                    double *__restrict__ phi, const Nrm<double> *__restrict__ cn,
                                                    const double *__restrict__ curv,
                                                    const int32_t *__restrict__ cells, const int ncell, const Layout L,
                                                    const MpConstFF K, const int mrt,
                                                    const int32_t *__restrict__ nb = nullptr, const int64_t stride = 0) {
    auto ldp = [](const S &v) -> ff {
        if constexpr (std::is_same<S, ffs>::value) return ff{v.hi, v.lo};
        else return ff_from_f64(v);
    };
    auto stp = [](S &dst, ff v) {
        if constexpr (std::is_same<S, ffs>::value) {
            const ff n = ff_fast2sum(v.hi, v.lo);
            dst = ffs{n.hi, n.lo};
        } else {
            dst = f64_of_ff(v);
        }
    };
    const int t = LIST ? list_node_index<ODD>() : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= ncell) return;
    MP_NODE_ADDRESSING
    const int64_t w2 = L.i2(i, j, k);
    ff ft[19];
    ff rho1, rho2;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const ff a = ldp(f[src(q)]);
        ft[q] = a;
        rho1 = q == 0 ? a : rho1 + a;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const ff b = ldp(g[src(q)]);
        ft[q] = ft[q] + b;
        rho2 = q == 0 ? b : rho2 + b;
    }
    const ff den = rho1 + rho2;
    const ff inv_den = ff(1.0f) / den;
    const ff ph = (rho1 - rho2) * inv_den;
    phi[L.i4(i, j, k)] = f64_of_ff(ph);
    const Nrm<double> nr = cn[w2];
    const ff cx = ff_from_f64(nr.x), cy = ff_from_f64(nr.y), cz = ff_from_f64(nr.z);
    const ff tmpf = K.half_gamma * ff_from_f64(curv[L.i1(i, j, k)]) * ff_from_f64(nr.n);
    const ff fx = tmpf * cx, fy = tmpf * cy, fz = tmpf * cz + K.force_z;
    const ff visc = (ff(1.0f) + ph) * K.nui1 + (ff(1.0f) - ph) * K.nui2;
    const ff omega = visc / (ff(6.0f) + ff_pow2(visc, 0.5f));
    MrtFold<ff> cf;
    if (mrt == 1) {
        const ff sq = ff_mulf(ff(2.0f) - omega, 8.0f) / (ff(8.0f) - omega);
        cf = fold_rates_dev<ff>(omega, omega, sq, omega, omega, sq);
    } else if (mrt == 3) {
        cf = fold_rates_dev<ff>(omega, omega, omega, omega, omega, omega);
    } else if (mrt == 4) {
        const ff sq = (ff(6.0f) - ff_mulf(omega, 3.0f)) / (ff(3.0f) - omega);
        cf = fold_rates_dev<ff>(omega, omega, sq, omega, omega, omega);
    } else {
        cf = fold_rates_dev<ff>(ff(1.19), ff(1.4), ff(1.2), omega, ff(1.4), ff(1.98));
    }
    mrt_collide_pairs<ff, true, false>(ft, den, fx, fy, fz, cf);
    // recolouring (Kernel_multiphase.F90:272-315)
    const ff tmp1 = rho1 * inv_den;
    const ff tmp = rho1 * rho2 * K.beta * inv_den;
    stp(f[c], tmp1 * ft[0]);
    stp(g[c], ft[0] * (ff(1.0f) - tmp1));
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const ff sx = EX(q) > 0 ? cx : -cx, sy = EY(q) > 0 ? cy : -cy, sz = EZ(q) > 0 ? cz : -cz;
        ff proj;
        if (q <= 6)
            proj = EX(q) != 0 ? sx : (EY(q) != 0 ? sy : sz);
        else if (EZ(q) == 0)
            proj = sx + sy;
        else if (EY(q) == 0)
            proj = sx + sz;
        else
            proj = sy + sz;
        const ff wt = q <= 6 ? K.w1_tmp_scale * tmp : K.rkw2 * tmp;
        const ff a = tmp1 * ft[q] + wt * proj;
        const ff b = ft[q] - a;
        const int64_t o = dst(q);
        stp(f[o], a);
        stp(g[o], b);
    }
}

// ---------------------------------------------------------------------------------
// Periodic halo exchange (single-device form of Mpi.F90:101-598).  Faces copy the five
// PDFs that cross the face over the interior tangential range; the edge kernel then
// copies the one PDF per edge, and must run after the faces (it overrides four slots
// that two face copies also write in the push direction, Mpi.F90:417-431).
// ---------------------------------------------------------------------------------
static __device__ __constant__ int c_plus[3][5] = {{1, 7, 9, 11, 13}, {3, 7, 8, 15, 17}, {5, 11, 12, 15, 16}};
static __device__ __constant__ int c_minus[3][5] = {{2, 8, 10, 12, 14}, {4, 10, 9, 16, 18}, {6, 14, 13, 18, 17}};

// one thread per (face cell, species); dim 0=x, 1=y, 2=z
template <class S>
__global__ void k_wrap_faces(S *__restrict__ f, int nspecies, const Layout L, int dim, int pull) {
    const int64_t n1 = dim == 0 ? L.ny : L.nx;  // fastest tangential extent
    const int64_t n2 = dim == 2 ? L.ny : L.nz;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2 * nspecies) return;
    const int s = (int)(t / (n1 * n2));
    const int64_t r = t % (n1 * n2);
    const int a = (int)(r % n1) + 1, b = (int)(r / n1) + 1;
    S *A = f + (int64_t)s * 19 * L.qs;
    const int n = dim == 0 ? L.nx : (dim == 1 ? L.ny : L.nz);
    auto cell = [&](int layer) -> int64_t {
        if (dim == 0) return L.cell(layer, a, b);
        if (dim == 1) return L.cell(a, layer, b);
        return L.cell(a, b, layer);
    };
    if (pull) {
        // ghost 0 <- interior n for the + set; ghost n+1 <- interior 1 for the - set
        const int64_t g0 = cell(0), in_n = cell(n), g1 = cell(n + 1), in_1 = cell(1);
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const int qp = c_plus[dim][m], qm = c_minus[dim][m];
            A[(int64_t)qp * L.qs + g0] = A[(int64_t)qp * L.qs + in_n];
            A[(int64_t)qm * L.qs + g1] = A[(int64_t)qm * L.qs + in_1];
        }
    } else {
        // interior 1 <- ghost n+1 for the - set; interior n <- ghost 0 for the + set
        const int64_t g0 = cell(0), in_n = cell(n), g1 = cell(n + 1), in_1 = cell(1);
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const int qp = c_plus[dim][m], qm = c_minus[dim][m];
            A[(int64_t)qm * L.qs + in_1] = A[(int64_t)qm * L.qs + g1];
            A[(int64_t)qp * L.qs + in_n] = A[(int64_t)qp * L.qs + g0];
        }
    }
}

// edges: along x when y and z are periodic (the reference's case), along y (x,z) and
// along z (x,y) for the x-periodic extension.  One thread per edge cell and species.
template <class S>
__global__ void k_wrap_edges(S *__restrict__ f, int nspecies, const Layout L, int axis, int pull) {
    const int n = axis == 0 ? L.nx : (axis == 1 ? L.ny : L.nz);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * nspecies) return;
    const int s = (int)(t / n);
    const int a = (int)(t % n) + 1;
    S *A = f + (int64_t)s * 19 * L.qs;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    auto X = [&](int q, int i, int j, int k) -> S & { return A[(int64_t)q * L.qs + L.cell(i, j, k)]; };
    if (axis == 0) {  // y,z periodic; i = a
        const int i = a;
        if (pull) {
            X(18, i, ny + 1, nz + 1) = X(18, i, 1, 1);
            X(16, i, ny + 1, 0) = X(16, i, 1, nz);
            X(17, i, 0, nz + 1) = X(17, i, ny, 1);
            X(15, i, 0, 0) = X(15, i, ny, nz);
        } else {
            X(15, i, ny, nz) = X(15, i, 0, 0);
            X(17, i, ny, 1) = X(17, i, 0, nz + 1);
            X(16, i, 1, nz) = X(16, i, ny + 1, 0);
            X(18, i, 1, 1) = X(18, i, ny + 1, nz + 1);
        }
    } else if (axis == 1) {  // x,z periodic; j = a
        const int j = a;
        if (pull) {
            X(11, 0, j, 0) = X(11, nx, j, nz);
            X(12, nx + 1, j, 0) = X(12, 1, j, nz);
            X(13, 0, j, nz + 1) = X(13, nx, j, 1);
            X(14, nx + 1, j, nz + 1) = X(14, 1, j, 1);
        } else {
            X(11, nx, j, nz) = X(11, 0, j, 0);
            X(12, 1, j, nz) = X(12, nx + 1, j, 0);
            X(13, nx, j, 1) = X(13, 0, j, nz + 1);
            X(14, 1, j, 1) = X(14, nx + 1, j, nz + 1);
        }
    } else {  // x,y periodic; k = a
        const int k = a;
        if (pull) {
            X(7, 0, 0, k) = X(7, nx, ny, k);
            X(8, nx + 1, 0, k) = X(8, 1, ny, k);
            X(9, 0, ny + 1, k) = X(9, nx, 1, k);
            X(10, nx + 1, ny + 1, k) = X(10, 1, 1, k);
        } else {
            X(7, nx, ny, k) = X(7, 0, 0, k);
            X(8, 1, ny, k) = X(8, nx + 1, 0, k);
            X(9, nx, 1, k) = X(9, 0, ny + 1, k);
            X(10, 1, 1, k) = X(10, nx + 1, ny + 1, k);
        }
    }
}

// phi halo, 4 layers (MPI_phi_async_pack / MPI_phi_sync_update, Mpi.F90:608-867):
// z faces (i,j interior), y faces (i,k interior), x-edges; sources are all interior.
template <class T>
__global__ void k_wrap_phi(T *__restrict__ phi, const Layout L, int py, int pz) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const int64_t nzf = pz ? (int64_t)4 * nx * ny : 0;
    const int64_t nyf = py ? (int64_t)4 * nx * nz : 0;
    const int64_t ned = (py && pz) ? (int64_t)16 * nx : 0;
    if (t < nzf) {
        const int i = (int)(t % nx) + 1;
        const int j = (int)((t / nx) % ny) + 1;
        const int k = (int)(t / ((int64_t)nx * ny)) + 1;
        phi[L.i4(i, j, k - 4)] = phi[L.i4(i, j, nz + k - 4)];
        phi[L.i4(i, j, k + nz)] = phi[L.i4(i, j, k)];
        return;
    }
    int64_t u = t - nzf;
    if (u < nyf) {
        const int i = (int)(u % nx) + 1;
        const int j = (int)((u / nx) % 4) + 1;
        const int k = (int)(u / ((int64_t)nx * 4)) + 1;
        phi[L.i4(i, j - 4, k)] = phi[L.i4(i, ny + j - 4, k)];
        phi[L.i4(i, j + ny, k)] = phi[L.i4(i, j, k)];
        return;
    }
    u -= nyf;
    if (u < ned) {
        const int i = (int)(u % nx) + 1;
        const int j = (int)((u / nx) % 4) + 1;
        const int k = (int)(u / ((int64_t)nx * 4)) + 1;
        phi[L.i4(i, j - 4, k - 4)] = phi[L.i4(i, ny + j - 4, nz + k - 4)];
        phi[L.i4(i, j + ny, k - 4)] = phi[L.i4(i, j, nz + k - 4)];
        phi[L.i4(i, j + ny, k + nz)] = phi[L.i4(i, j, k)];
        phi[L.i4(i, j - 4, k + nz)] = phi[L.i4(i, ny + j - 4, k)];
    }
}

// ---------------------------------------------------------------------------------
// Inlet / outlet boundary conditions on the z planes; one thread per (i,j).
// The reference's masking x*(1-w) + y*w is kept literally.
// ---------------------------------------------------------------------------------
template <class R> __device__ __forceinline__ R sel(R x, R y, int w) { return x * (R)(1 - w) + y * (R)w; }

// velocity inlet (Boundary_multiphase_inlet.F90:6-102; singlephase Boundary.F90:5-73)
template <class S>
__global__ void k_inlet_velocity(S *__restrict__ f, S *__restrict__ g, typename Store<S>::R *__restrict__ phi,
                                 const int8_t *__restrict__ walls, const double *__restrict__ w_in, const Layout L, const PdfAt pa,
                                 const StepParams P, int before_odd, int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1;
    if (i > L.nx) return;
    const int wi = walls[L.i2(i, j, 1)];
    if (multiphase) {
        const double p0 = P.phi_inlet * (double)(1 - wi) + phi[L.i4(i, j, 0)] * (double)wi;
        phi[L.i4(i, j, 0)] = p0;
        phi[L.i4(i, j, -1)] = p0;
        phi[L.i4(i, j, -2)] = p0;
        phi[L.i4(i, j, -3)] = p0;
    }
    double tmp2 = w_in[L.ip(i, j)] * P.relaxation;
    double tmp1;
    if (multiphase) {
        tmp1 = tmp2 * P.sa_inject;
        tmp2 = tmp2 - tmp1;
    } else {
        tmp1 = tmp2;
    }
    const R inv = R(1.0f / scale), sc = R(scale);
    for (int s = 0; s < (multiphase ? 2 : 1); ++s) {
        S *A = s == 0 ? f : g;
        const R t = R(s == 0 ? tmp1 : tmp2);
        const float rf = ref;
        auto ld = [&](int q, int ii, int jj, int kk) { return St::ld(A, pa(L, q, ii, jj, kk), R(WREST(q) * rf), inv); };
        auto st = [&](int q, int ii, int jj, int kk, R v) { St::st(A, pa(L, q, ii, jj, kk), v, R(WREST(q) * rf), sc); };
        const R c1 = R(6.0 * w_equ_1), c2 = R(6.0 * w_equ_2);
        if (before_odd) {
            st(5, i, j, 0, sel<R>(ld(6, i, j, 1) + c1 * t, ld(5, i, j, 0), wi));
            st(11, i - 1, j, 0, sel<R>(ld(14, i, j, 1) + c2 * t, ld(11, i - 1, j, 0), wi));
            st(12, i + 1, j, 0, sel<R>(ld(13, i, j, 1) + c2 * t, ld(12, i + 1, j, 0), wi));
            st(15, i, j - 1, 0, sel<R>(ld(18, i, j, 1) + c2 * t, ld(15, i, j - 1, 0), wi));
            st(16, i, j + 1, 0, sel<R>(ld(17, i, j, 1) + c2 * t, ld(16, i, j + 1, 0), wi));
        } else {
            st(6, i, j, 1, sel<R>(ld(5, i, j, 0) + c1 * t, ld(6, i, j, 1), wi));
            st(13, i, j, 1, sel<R>(ld(12, i + 1, j, 0) + c2 * t, ld(13, i, j, 1), wi));
            st(14, i, j, 1, sel<R>(ld(11, i - 1, j, 0) + c2 * t, ld(14, i, j, 1), wi));
            st(17, i, j, 1, sel<R>(ld(16, i, j + 1, 0) + c2 * t, ld(17, i, j, 1), wi));
            st(18, i, j, 1, sel<R>(ld(15, i, j - 1, 0) + c2 * t, ld(18, i, j, 1), wi));
        }
    }
}

// Zou-He pressure inlet (Boundary_multiphase_inlet.F90:115-294; Boundary.F90:80-187)
template <class S>
__global__ void k_inlet_zouhe(S *__restrict__ f, S *__restrict__ g, typename Store<S>::R *__restrict__ phi,
                              const int8_t *__restrict__ walls, const Layout L, const PdfAt pa, const StepParams P, int before_odd,
                              int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1;
    if (i > L.nx) return;
    const int wi = walls[L.i2(i, j, 1)];
    double rhos[2];
    if (multiphase) {
        const double p0 = P.phi_inlet * (double)(1 - wi) + phi[L.i4(i, j, 0)] * (double)wi;
        phi[L.i4(i, j, 0)] = p0;
        phi[L.i4(i, j, -1)] = p0;
        phi[L.i4(i, j, -2)] = p0;
        phi[L.i4(i, j, -3)] = p0;
        double tmpRho2 = P.rho_in;
        const double tmpRho1 = P.rho_in * P.sa_inject;
        tmpRho2 = tmpRho2 - tmpRho1;
        rhos[0] = tmpRho1;
        rhos[1] = tmpRho2;
    } else {
        rhos[0] = P.rho_in;
        rhos[1] = 0.0;
    }
    const R inv = R(1.0f / scale), sc = R(scale);
    for (int s = 0; s < (multiphase ? 2 : 1); ++s) {
        S *A = s == 0 ? f : g;
        const float rf = ref;
        auto ld = [&](int q, int ii, int jj, int kk) { return St::ld(A, pa(L, q, ii, jj, kk), R(WREST(q) * rf), inv); };
        auto st = [&](int q, int ii, int jj, int kk, R v) { St::st(A, pa(L, q, ii, jj, kk), v, R(WREST(q) * rf), sc); };
        const R c3 = R(0.333333333333333333), c6 = R(0.166666666666666667);
        if (before_odd) {
            const R t = (R(rhos[s]) - (ld(0, i, j, 1) + ld(1, i - 1, j, 1) + ld(2, i + 1, j, 1) + ld(3, i, j - 1, 1) +
                                       ld(4, i, j + 1, 1) + ld(7, i - 1, j - 1, 1) + ld(8, i + 1, j - 1, 1) +
                                       ld(9, i - 1, j + 1, 1) + ld(10, i + 1, j + 1, 1) +
                                       R(2.0) * (ld(6, i, j, 2) + ld(14, i + 1, j, 2) + ld(13, i - 1, j, 2) +
                                                 ld(18, i, j + 1, 2) + ld(17, i, j - 1, 2)))) *
                        R(P.relaxation);
            const R tnx = R(0.5) * (ld(1, i - 1, j, 1) + ld(7, i - 1, j - 1, 1) + ld(9, i - 1, j + 1, 1) -
                                    (ld(2, i + 1, j, 1) + ld(8, i + 1, j - 1, 1) + ld(10, i + 1, j + 1, 1)));
            const R tny = R(0.5) * (ld(3, i, j - 1, 1) + ld(7, i - 1, j - 1, 1) + ld(8, i + 1, j - 1, 1) -
                                    (ld(4, i, j + 1, 1) + ld(10, i + 1, j + 1, 1) + ld(9, i - 1, j + 1, 1)));
            st(5, i, j, 0, sel<R>(ld(6, i, j, 2) + c3 * t, ld(5, i, j, 0), wi));
            st(11, i - 1, j, 0, sel<R>(ld(14, i + 1, j, 2) + c6 * t - tnx, ld(11, i - 1, j, 0), wi));
            st(12, i + 1, j, 0, sel<R>(ld(13, i - 1, j, 2) + c6 * t + tnx, ld(12, i + 1, j, 0), wi));
            st(15, i, j - 1, 0, sel<R>(ld(18, i, j + 1, 2) + c6 * t - tny, ld(15, i, j - 1, 0), wi));
            st(16, i, j + 1, 0, sel<R>(ld(17, i, j - 1, 2) + c6 * t + tny, ld(16, i, j + 1, 0), wi));
        } else {
            const R t = (R(rhos[s]) - (ld(0, i, j, 1) + ld(2, i, j, 1) + ld(1, i, j, 1) + ld(4, i, j, 1) + ld(3, i, j, 1) +
                                       ld(8, i, j, 1) + ld(7, i, j, 1) + ld(10, i, j, 1) + ld(9, i, j, 1) +
                                       R(2.0) * (ld(5, i, j, 1) + ld(11, i, j, 1) + ld(12, i, j, 1) + ld(15, i, j, 1) +
                                                 ld(16, i, j, 1)))) *
                        R(P.relaxation);
            const R tnx = R(0.5) * (ld(2, i, j, 1) + ld(8, i, j, 1) + ld(10, i, j, 1) - (ld(1, i, j, 1) + ld(7, i, j, 1) + ld(9, i, j, 1)));
            const R tny = R(0.5) * (ld(4, i, j, 1) + ld(9, i, j, 1) + ld(10, i, j, 1) - (ld(3, i, j, 1) + ld(8, i, j, 1) + ld(7, i, j, 1)));
            st(6, i, j, 1, sel<R>(ld(5, i, j, 1) + c3 * t, ld(6, i, j, 1), wi));
            st(13, i, j, 1, sel<R>(ld(12, i, j, 1) + c6 * t + tnx, ld(13, i, j, 1), wi));
            st(14, i, j, 1, sel<R>(ld(11, i, j, 1) + c6 * t - tnx, ld(14, i, j, 1), wi));
            st(17, i, j, 1, sel<R>(ld(16, i, j, 1) + c6 * t + tny, ld(17, i, j, 1), wi));
            st(18, i, j, 1, sel<R>(ld(15, i, j, 1) + c6 * t - tny, ld(18, i, j, 1), wi));
        }
    }
}

// convective outlet (Boundary_multiphase_outlet.F90:7-127; Boundary.F90:196-276)
template <class S>
__global__ void k_outlet_convective(S *__restrict__ f, S *__restrict__ g, typename Store<S>::R *__restrict__ phi,
                                    double *__restrict__ fconv, double *__restrict__ gconv, double *__restrict__ phiconv,
                                    const int8_t *__restrict__ walls, const Layout L, const PdfAt pa, const StepParams P, int before_odd,
                                    int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1;
    if (i > L.nx) return;
    const int nz = L.nz;
    const int wi = walls[L.i2(i, j, nz)];
    const double u_convec = P.uin_avg;
    const double temp = 1.0 / (1.0 + u_convec);
    if (multiphase) {
        const double p1 = ((phiconv[L.ip(i, j)] + u_convec * phi[L.i4(i, j, nz)]) * temp) * (double)(1 - wi) +
                          phi[L.i4(i, j, nz + 1)] * (double)wi;
        phi[L.i4(i, j, nz + 1)] = p1;
        phiconv[L.ip(i, j)] = p1;
        phi[L.i4(i, j, nz + 2)] = p1;
        phi[L.i4(i, j, nz + 3)] = p1;
        phi[L.i4(i, j, nz + 4)] = p1;
    }
    const R inv = R(1.0f / scale), sc = R(scale);
    const R uc = R(u_convec), tp = R(temp);
    for (int s = 0; s < (multiphase ? 2 : 1); ++s) {
        S *A = s == 0 ? f : g;
        double *C = s == 0 ? fconv : gconv;
        const float rf = ref;
        auto ld = [&](int q, int ii, int jj, int kk) { return St::ld(A, pa(L, q, ii, jj, kk), R(WREST(q) * rf), inv); };
        auto st = [&](int q, int ii, int jj, int kk, R v) { St::st(A, pa(L, q, ii, jj, kk), v, R(WREST(q) * rf), sc); };
        auto cv = [&](int q) -> double & { return C[L.ic(i, j, q)]; };
        if (before_odd) {
            st(6, i, j, nz + 1, sel<R>((R(cv(6)) + uc * ld(6, i, j, nz)) * tp, ld(6, i, j, nz + 1), wi));
            st(13, i - 1, j, nz + 1, sel<R>((R(cv(13)) + uc * ld(13, i - 1, j, nz)) * tp, ld(13, i - 1, j, nz + 1), wi));
            st(14, i + 1, j, nz + 1, sel<R>((R(cv(14)) + uc * ld(14, i + 1, j, nz)) * tp, ld(14, i + 1, j, nz + 1), wi));
            st(17, i, j - 1, nz + 1, sel<R>((R(cv(17)) + uc * ld(17, i, j - 1, nz)) * tp, ld(17, i, j - 1, nz + 1), wi));
            st(18, i, j + 1, nz + 1, sel<R>((R(cv(18)) + uc * ld(18, i, j + 1, nz)) * tp, ld(18, i, j + 1, nz + 1), wi));
            cv(6) = ld(6, i, j, nz + 1);
            cv(13) = ld(13, i - 1, j, nz + 1);
            cv(14) = ld(14, i + 1, j, nz + 1);
            cv(17) = ld(17, i, j - 1, nz + 1);
            cv(18) = ld(18, i, j + 1, nz + 1);
        } else {
            st(5, i, j, nz, sel<R>((R(cv(6)) + uc * ld(5, i, j, nz - 1)) * tp, ld(5, i, j, nz), wi));
            st(11, i, j, nz, sel<R>((R(cv(14)) + uc * ld(11, i, j, nz - 1)) * tp, ld(11, i, j, nz), wi));
            st(12, i, j, nz, sel<R>((R(cv(13)) + uc * ld(12, i, j, nz - 1)) * tp, ld(12, i, j, nz), wi));
            st(15, i, j, nz, sel<R>((R(cv(18)) + uc * ld(15, i, j, nz - 1)) * tp, ld(15, i, j, nz), wi));
            st(16, i, j, nz, sel<R>((R(cv(17)) + uc * ld(16, i, j, nz - 1)) * tp, ld(16, i, j, nz), wi));
            cv(6) = ld(5, i, j, nz);
            cv(14) = ld(11, i, j, nz);
            cv(13) = ld(12, i, j, nz);
            cv(18) = ld(15, i, j, nz);
            cv(17) = ld(16, i, j, nz);
        }
    }
}

// Zou-He pressure outlet (Boundary_multiphase_outlet.F90:139-311; Boundary.F90:284-389)
template <class S>
__global__ void k_outlet_zouhe(S *__restrict__ f, S *__restrict__ g, typename Store<S>::R *__restrict__ phi,
                               const int8_t *__restrict__ walls, const Layout L, const PdfAt pa, const StepParams P, int before_odd,
                               int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1;
    if (i > L.nx) return;
    const int nz = L.nz;
    const int wi = walls[L.i2(i, j, nz)];
    double phin = 0.0;
    if (multiphase) {
        phin = phi[L.i4(i, j, nz)];
        phi[L.i4(i, j, nz + 1)] = phin;
        phi[L.i4(i, j, nz + 2)] = phin;
        phi[L.i4(i, j, nz + 3)] = phin;
        phi[L.i4(i, j, nz + 4)] = phin;
    }
    const R inv = R(1.0f / scale), sc = R(scale);
    const float rf = ref;
    auto LD = [&](S *A, int q, int ii, int jj, int kk) { return St::ld(A, pa(L, q, ii, jj, kk), R(WREST(q) * rf), inv); };
    R t1;
    for (int s = 0; s < (multiphase ? 2 : 1); ++s) {
        S *A = s == 0 ? f : g;
        auto ld = [&](int q, int ii, int jj, int kk) { return LD(A, q, ii, jj, kk); };
        if (before_odd) {
            const R part = ld(0, i, j, nz) + ld(1, i - 1, j, nz) + ld(2, i + 1, j, nz) + ld(3, i, j - 1, nz);
            // keep one left-to-right chain across both species, as the reference writes it
            R acc = s == 0 ? part : t1 + ld(0, i, j, nz) + ld(1, i - 1, j, nz) + ld(2, i + 1, j, nz) + ld(3, i, j - 1, nz);
            acc = acc + ld(4, i, j + 1, nz) + ld(7, i - 1, j - 1, nz) + ld(8, i + 1, j - 1, nz) + ld(9, i - 1, j + 1, nz) +
                  ld(10, i + 1, j + 1, nz) +
                  R(2.0) * (ld(5, i, j, nz - 1) + ld(11, i - 1, j, nz - 1) + ld(12, i + 1, j, nz - 1) +
                            ld(15, i, j - 1, nz - 1) + ld(16, i, j + 1, nz - 1));
            t1 = acc;
        } else {
            const R part = ld(0, i, j, nz) + ld(2, i, j, nz) + ld(1, i, j, nz) + ld(4, i, j, nz);
            R acc = s == 0 ? part : t1 + ld(0, i, j, nz) + ld(2, i, j, nz) + ld(1, i, j, nz) + ld(4, i, j, nz);
            acc = acc + ld(3, i, j, nz) + ld(8, i, j, nz) + ld(7, i, j, nz) + ld(10, i, j, nz) + ld(9, i, j, nz) +
                  R(2.0) * (ld(6, i, j, nz) + ld(14, i, j, nz) + ld(13, i, j, nz) + ld(18, i, j, nz) + ld(17, i, j, nz));
            t1 = acc;
        }
    }
    t1 = t1 - R(P.rho_out);
    R t2 = R(0.0);
    if (multiphase) {
        t2 = t1 * R(0.5) * (R(1.0) - R(phin));
        t1 = t1 - t2;
    }
    const R c3 = R(0.333333333333333333), c6 = R(0.166666666666666667);
    const R w1 = R(1.0) - (R)wi, w0 = (R)wi;
    for (int s = 0; s < (multiphase ? 2 : 1); ++s) {
        S *A = s == 0 ? f : g;
        const R t = s == 0 ? t1 : t2;
        auto ld = [&](int q, int ii, int jj, int kk) { return LD(A, q, ii, jj, kk); };
        auto st = [&](int q, int ii, int jj, int kk, R v) { St::st(A, pa(L, q, ii, jj, kk), v, R(WREST(q) * rf), sc); };
        if (before_odd) {
            const R tnx = R(0.5) * (ld(1, i - 1, j, nz) + ld(7, i - 1, j - 1, nz) + ld(9, i - 1, j + 1, nz) -
                                    (ld(2, i + 1, j, nz) + ld(8, i + 1, j - 1, nz) + ld(10, i + 1, j + 1, nz)));
            const R tny = R(0.5) * (ld(3, i, j - 1, nz) + ld(7, i - 1, j - 1, nz) + ld(8, i + 1, j - 1, nz) -
                                    (ld(4, i, j + 1, nz) + ld(10, i + 1, j + 1, nz) + ld(9, i - 1, j + 1, nz)));
            st(6, i, j, nz + 1, (ld(5, i, j, nz - 1) - c3 * t) * w1 + ld(6, i, j, nz + 1) * w0);
            st(13, i - 1, j, nz + 1, (ld(12, i + 1, j, nz - 1) - c6 * t - tnx) * w1 + ld(13, i - 1, j, nz + 1) * w0);
            st(14, i + 1, j, nz + 1, (ld(11, i - 1, j, nz - 1) - c6 * t + tnx) * w1 + ld(14, i + 1, j, nz + 1) * w0);
            st(17, i, j - 1, nz + 1, (ld(16, i, j + 1, nz - 1) - c6 * t - tny) * w1 + ld(17, i, j - 1, nz + 1) * w0);
            st(18, i, j + 1, nz + 1, (ld(15, i, j - 1, nz - 1) - c6 * t + tny) * w1 + ld(18, i, j + 1, nz + 1) * w0);
        } else {
            const R tnx = R(0.5) * (ld(2, i, j, nz) + ld(8, i, j, nz) + ld(10, i, j, nz) - (ld(1, i, j, nz) + ld(7, i, j, nz) + ld(9, i, j, nz)));
            const R tny = R(0.5) * (ld(4, i, j, nz) + ld(10, i, j, nz) + ld(9, i, j, nz) - (ld(3, i, j, nz) + ld(7, i, j, nz) + ld(8, i, j, nz)));
            st(5, i, j, nz, (ld(6, i, j, nz) - c3 * t) * w1 + ld(5, i, j, nz) * w0);
            st(11, i, j, nz, (ld(14, i, j, nz) - c6 * t + tnx) * w1 + ld(11, i, j, nz) * w0);
            st(12, i, j, nz, (ld(13, i, j, nz) - c6 * t - tnx) * w1 + ld(12, i, j, nz) * w0);
            st(15, i, j, nz, (ld(18, i, j, nz) - c6 * t + tny) * w1 + ld(15, i, j, nz) * w0);
            st(16, i, j, nz, (ld(17, i, j, nz) - c6 * t - tny) * w1 + ld(16, i, j, nz) * w0);
        }
    }
}

// porous plate (Boundary_multiphase_other.F90:8-184); blocked = the species that is
// reflected, passing = the species copied across.
template <class T>
__global__ void k_porous_plate(T *__restrict__ blocked, T *__restrict__ passing, const Layout L, const PdfAt pa, int z,
                               int before_odd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1;
    if (i > L.nx) return;
    auto b = [&](int q, int ii, int jj, int kk) -> T & { return blocked[pa(L, q, ii, jj, kk)]; };
    auto c = [&](int q, int ii, int jj, int kk) -> T & { return passing[pa(L, q, ii, jj, kk)]; };
    if (before_odd) {
        b(6, i, j, z) = b(5, i, j, z - 1);
        b(13, i - 1, j, z) = b(12, i, j, z - 1);
        b(14, i + 1, j, z) = b(11, i, j, z - 1);
        b(17, i, j - 1, z) = b(16, i, j, z - 1);
        b(18, i, j + 1, z) = b(15, i, j, z - 1);
        b(5, i, j, z) = b(6, i, j, z + 1);
        b(12, i + 1, j, z) = b(13, i, j, z + 1);
        b(11, i - 1, j, z) = b(14, i, j, z + 1);
        b(16, i, j + 1, z) = b(17, i, j, z + 1);
        b(15, i, j - 1, z) = b(18, i, j, z + 1);
        c(6, i, j, z) = c(6, i, j, z + 1);
        c(13, i, j, z) = c(13, i, j, z + 1);
        c(14, i, j, z) = c(14, i, j, z + 1);
        c(17, i, j, z) = c(17, i, j, z + 1);
        c(18, i, j, z) = c(18, i, j, z + 1);
        c(5, i, j, z) = c(5, i, j, z - 1);
        c(12, i, j, z) = c(12, i, j, z - 1);
        c(11, i, j, z) = c(11, i, j, z - 1);
        c(16, i, j, z) = c(16, i, j, z - 1);
        c(15, i, j, z) = c(15, i, j, z - 1);
    } else {
        b(5, i, j, z - 1) = b(6, i, j, z);
        b(11, i, j, z - 1) = b(14, i + 1, j, z);
        b(12, i, j, z - 1) = b(13, i - 1, j, z);
        b(15, i, j, z - 1) = b(18, i, j + 1, z);
        b(16, i, j, z - 1) = b(17, i, j - 1, z);
        b(6, i, j, z + 1) = b(5, i, j, z);
        b(14, i, j, z + 1) = b(11, i - 1, j, z);
        b(13, i, j, z + 1) = b(12, i + 1, j, z);
        b(18, i, j, z + 1) = b(15, i, j - 1, z);
        b(17, i, j, z + 1) = b(16, i, j + 1, z);
        c(5, i, j, z - 1) = c(5, i, j, z);
        c(11, i, j, z - 1) = c(11, i, j, z);
        c(12, i, j, z - 1) = c(12, i, j, z);
        c(15, i, j, z - 1) = c(15, i, j, z);
        c(16, i, j, z - 1) = c(16, i, j, z);
        c(6, i, j, z + 1) = c(6, i, j, z);
        c(14, i, j, z + 1) = c(14, i, j, z);
        c(13, i, j, z + 1) = c(13, i, j, z);
        c(18, i, j, z + 1) = c(18, i, j, z);
        c(17, i, j, z + 1) = c(17, i, j, z);
    }
}

// ---------------------------------------------------------------------------------
// color_gradient (Phase_gradient.F90:5-265)
// ---------------------------------------------------------------------------------
// phi extrapolation to the solid-boundary list (:13-30)
template <class T>
__global__ void k_extrap_phi(T *__restrict__ phi, const SolidBnd *__restrict__ sb, int ns, const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const SolidBnd s = sb[t];
    T acc = T(0.0);
    for (int n = 0; n < s.i_fluid_num; ++n) {
        const int ie = s.nbr[n];
        // ie is 1..18 (validated on upload)
        const int dx = c_ex[ie], dy = c_ey[ie], dz = c_ez[ie];
        const T w = ie <= 6 ? T(w_equ_1) : T(w_equ_2);
        acc = acc + phi[L.i4(s.ix + dx, s.iy + dy, s.iz + dz)] * w;
    }
    phi[L.i4(s.ix, s.iy, s.iz)] = acc / T(s.la_weight);
}

// Register caps of the fluid-cell gradient kernels (256 threads) and of the compact-record
// normal extrapolation (128 threads): resident blocks per SM.  The FP32 gradient lists take 5
// (curvature 52 -> 48 registers, 5 blocks instead of 4; C3 packing FP32 step 2.4 % faster;
// 6 blocks spilled and gained less), the FP64 ones 3 (80 registers, as the compiler's own
// choice; 5 spilled).  The extrapolation keeps the compiler's choice (72 registers in FP32;
// caps of 8 and 10 blocks spilled and made the step slower), 0 below.
// Tuning parameters (MFLBM_NVCC_FLAGS=-DMFLBM_GRAD_MIN_BLOCKS_F32=n, -DMFLBM_EXTRAP_MIN_BLOCKS=n).
#ifndef MFLBM_GRAD_MIN_BLOCKS_F32
#define MFLBM_GRAD_MIN_BLOCKS_F32 5
#endif
#ifndef MFLBM_GRAD_MIN_BLOCKS_F64
#define MFLBM_GRAD_MIN_BLOCKS_F64 3
#endif
#ifndef MFLBM_EXTRAP_MIN_BLOCKS
#define MFLBM_EXTRAP_MIN_BLOCKS 0
#endif
template <class T> struct GradOcc { static constexpr int kMinBlocks = MFLBM_GRAD_MIN_BLOCKS_F64; };
template <> struct GradOcc<float> { static constexpr int kMinBlocks = MFLBM_GRAD_MIN_BLOCKS_F32; };
#define MFLBM_GRAD_BOUNDS __launch_bounds__(256, GradOcc<T>::kMinBlocks)
#if MFLBM_EXTRAP_MIN_BLOCKS > 0
#define MFLBM_EXTRAP_BOUNDS __launch_bounds__(128, MFLBM_EXTRAP_MIN_BLOCKS)
#else
#define MFLBM_EXTRAP_BOUNDS __launch_bounds__(128)
#endif

// The same two extrapolations over the compact solid-boundary records (SolidBndC: packed
// cell, bit mask of the fluid-neighbour directions, la_weight): 16 bytes read per node
// instead of 96.  The 18 directions are visited in ascending order, which is the order of
// the neighbour list whenever the context builds these records, so the sums are the same
// operations in the same order.  The loop is unrolled with one predicated gather per
// direction, so a node's loads are all in flight at once instead of one per iteration
// of a data-dependent loop.
template <class T>
__global__ void k_extrap_phi_c(T *__restrict__ phi, const SolidBndC *__restrict__ sb, int ns, const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const SolidBndC s = sb[t];
    int ix, iy, iz;
    unpack_cell(s.ijk, ix, iy, iz);
    const int64_t c = L.i4(ix, iy, iz);
    T v[18];
#pragma unroll
    for (int ie = 1; ie <= 18; ++ie)
        v[ie - 1] = (s.mask >> (ie - 1)) & 1u ? phi[c + EX(ie) + L.h4x * EY(ie) + L.h4xy * EZ(ie)] : T(0.0);
    T acc = T(0.0);
#pragma unroll
    for (int ie = 1; ie <= 18; ++ie)
        if ((s.mask >> (ie - 1)) & 1u) acc = acc + v[ie - 1] * (ie <= 6 ? T(w_equ_1) : T(w_equ_2));
    phi[c] = acc / T(s.la_weight);
}

template <class T>
__global__ void MFLBM_EXTRAP_BOUNDS k_extrap_normals_c(Nrm<T> *__restrict__ cn, const SolidBndC *__restrict__ sb, int ns,
                                                       const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const SolidBndC s = sb[t];
    int ix, iy, iz;
    unpack_cell(s.ijk, ix, iy, iz);
    if (!(ix >= 0 && ix <= L.nx + 1 && iy >= 0 && iy <= L.ny + 1 && iz >= 0 && iz <= L.nz + 1)) return;
    const int64_t id = L.i2(ix, iy, iz);
    T ax = T(0.0), ay = T(0.0), az = T(0.0);
    if constexpr (sizeof(T) == 4) {
        // FP32: the gathers in two groups of nine directions, each group's record loads in
        // flight together, then the sums in direction order
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            Nrm<T> v[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) {
                const int ie = 1 + 9 * h + e;
                const bool on = (s.mask >> (ie - 1)) & 1u;
                const int64_t nb = id + EX(ie) + L.h2x * EY(ie) + L.h2xy * EZ(ie);
                v[e] = on ? cn[nb] : Nrm<T>{T(0.0), T(0.0), T(0.0), T(0.0)};
            }
#pragma unroll
            for (int e = 0; e < 9; ++e) {
                const int ie = 1 + 9 * h + e;
                if ((s.mask >> (ie - 1)) & 1u) {
                    const T w = ie <= 6 ? T(w_equ_1) : T(w_equ_2);
                    ax = ax + v[e].x * w;
                    ay = ay + v[e].y * w;
                    az = az + v[e].z * w;
                }
            }
        }
    } else {
        // FP64: gather direction by direction (preloaded records would cost occupancy)
        for (uint32_t m = s.mask; m; m &= m - 1u) {
            const int ie = __ffs((int)m);
            const T w = ie <= 6 ? T(w_equ_1) : T(w_equ_2);
            const Nrm<T> v = cn[L.i2(ix + c_ex[ie], iy + c_ey[ie], iz + c_ez[ie])];
            ax = ax + v.x * w;
            ay = ay + v.y * w;
            az = az + v.z * w;
        }
    }
    const T lw = T(s.la_weight);
    cn[id].x = ax / lw;
    cn[id].y = ay / lw;
    cn[id].z = az / lw;
}

#include "wetting.cuh"

// ISO4 gradient and unit normal from a phi accessor P(a, b, c) = phi at offset (a, b, c)
// (:33-79); shared by the global-memory and shared-memory forms
template <class T, class PA>
__device__ __forceinline__ void normals_of(PA P, T &gx, T &gy, T &gz, T &cn) {
    const T c1 = T(ISO4_1), c2 = T(ISO4_2);
    gx = c1 * (P(1, 0, 0) - P(-1, 0, 0)) +
         c2 * (P(1, 1, 0) - P(-1, -1, 0) + P(1, -1, 0) - P(-1, 1, 0) + P(1, 0, 1) - P(-1, 0, -1) + P(1, 0, -1) - P(-1, 0, 1));
    gy = c1 * (P(0, 1, 0) - P(0, -1, 0)) +
         c2 * (P(1, 1, 0) - P(-1, -1, 0) + P(-1, 1, 0) - P(1, -1, 0) + P(0, 1, 1) - P(0, -1, -1) + P(0, 1, -1) - P(0, -1, 1));
    gz = c1 * (P(0, 0, 1) - P(0, 0, -1)) +
         c2 * (P(1, 0, 1) - P(-1, 0, -1) + P(-1, 0, 1) - P(1, 0, -1) + P(0, 1, 1) - P(0, -1, -1) + P(0, -1, 1) - P(0, 1, -1));
    cn = sqrt(gx * gx + gy * gy + gz * gz);
    if (cn < T(1e-6)) {
        gx = T(0.0); gy = T(0.0); gz = T(0.0); cn = T(0.0);
    } else {
#ifdef MFLBM_STRICT
        gx = gx / cn; gy = gy / cn; gz = gz / cn;
#else
        const T inv = T(1.0) / cn;
        gx = gx * inv; gy = gy * inv; gz = gz * inv;
#endif
    }
}

// ISO4 gradient and unit normal of one cell from global memory
template <class T>
__device__ __forceinline__ void normals_at(const T *__restrict__ phi, int i, int j, int k, int64_t id,
                                           Nrm<T> *__restrict__ out, const Layout &L) {
    auto P = [&](int a, int b, int c) { return phi[L.i4(i + a, j + b, k + c)]; };
    T gx, gy, gz, cn;
    normals_of<T>(P, gx, gy, gz, cn);
    out[id] = Nrm<T>{gx, gy, gz, cn};
}

// over [1-2, n+2]^3, every cell
template <class T>
__global__ void __launch_bounds__(256) k_normals(const T *__restrict__ phi, const int8_t *__restrict__ walls,
                                                 Nrm<T> *__restrict__ cn, const Layout L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > L.nx + 2 || j > L.ny + 2) return;
    const int64_t id = L.i2(i, j, k);
    if (walls[id] == 1) {  // the reference zeroes normals at wall nodes (Phase_gradient.F90:65-69)
        cn[id] = Nrm<T>{T(0.0), T(0.0), T(0.0), T(0.0)};
        return;
    }
    normals_at<T>(phi, i, j, k, id, cn, L);
}

// Fluid-cell forms of k_normals / k_curvature (default build): one thread per entry of a
// list of the cells that need the value, packed as (i+2) | (j+2) << 11 | (k+2) << 22 in
// ascending cell order (pack_cell in common.cuh).  Wall cells are never visited: they keep the zeros the context
// wrote when the geometry was set (the full-box kernels write the same zeros each call),
// and solid-boundary cells receive their extrapolated normals as before.  At porosity 0.22
// this skips about two thirds of the cells, and every lane of a warp does work.

// WET: the list starts with the nwet fluid-boundary nodes in record order; entry t < nwet
// applies the geometric wetting of record fb[t] to the normal it has just computed (the
// wetting kernel's operations on the same values, so it is not launched)
template <class T, bool WET = false>
__global__ void MFLBM_GRAD_BOUNDS k_normals_list(const T *__restrict__ phi, const uint32_t *__restrict__ cl, int n,
                                                      Nrm<T> *__restrict__ cn, const Layout L,
                                                      const FluidBnd *__restrict__ fb = nullptr, int nwet = 0,
                                                      T min_one_m = T(0.0)) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_cell(cl[t], i, j, k);
    if constexpr (WET) {
        auto P = [&](int a, int b, int c) { return phi[L.i4(i + a, j + b, k + c)]; };
        T gx, gy, gz, c;
        normals_of<T>(P, gx, gy, gz, c);
        if (t < nwet && c > T(1e-6)) {
            const FluidBnd b = fb[t];
            T nn[3] = {gx, gy, gz};
            wetting_normal<T>(nn, T(b.nwx), T(b.nwy), T(b.nwz), T(b.cos_t), T(b.sin_t), min_one_m);
            gx = nn[0];
            gy = nn[1];
            gz = nn[2];
        }
        cn[L.i2(i, j, k)] = Nrm<T>{gx, gy, gz, c};
    } else {
        normals_at<T>(phi, i, j, k, L.i2(i, j, k), cn, L);
    }
}

// The two stencils of the double-word form (MFLBM_FP64FF, multiphase): FP64 fields split on
// load, the default build's operations in FP32 pairs (ISO4 sums, norm, reciprocal), FP64
// results.  Fluid-cell lists only; without them the form uses the FP64 kernels.
template <int DUMMY = 0>
__global__ void __launch_bounds__(256) k_normals_list_ff(const double *__restrict__ phi, const uint32_t *__restrict__ cl,
                                                         int n, Nrm<double> *__restrict__ out,
                                                         const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_cell(cl[t], i, j, k);
    const int64_t id = L.i2(i, j, k);
    auto P = [&](int a, int b, int c) { return ff_from_f64(phi[L.i4(i + a, j + b, k + c)]); };
    constexpr ff c1 = ff_const(ISO4_1), c2 = ff_const(ISO4_2);
    ff gx = c1 * (P(1, 0, 0) - P(-1, 0, 0)) +
            c2 * (P(1, 1, 0) - P(-1, -1, 0) + P(1, -1, 0) - P(-1, 1, 0) + P(1, 0, 1) - P(-1, 0, -1) + P(1, 0, -1) - P(-1, 0, 1));
    ff gy = c1 * (P(0, 1, 0) - P(0, -1, 0)) +
            c2 * (P(1, 1, 0) - P(-1, -1, 0) + P(-1, 1, 0) - P(1, -1, 0) + P(0, 1, 1) - P(0, -1, -1) + P(0, 1, -1) - P(0, -1, 1));
    ff gz = c1 * (P(0, 0, 1) - P(0, 0, -1)) +
            c2 * (P(1, 0, 1) - P(-1, 0, -1) + P(-1, 0, 1) - P(1, 0, -1) + P(0, 1, 1) - P(0, -1, -1) + P(0, -1, 1) - P(0, 1, -1));
    ff cn = ff_sqrt(gx * gx + gy * gy + gz * gz);
    if (ff_less(cn, ff_const(1e-6))) {
        out[id] = Nrm<double>{0.0, 0.0, 0.0, 0.0};
        return;
    }
    const ff inv = ff(1.0f) / cn;
    out[id] = Nrm<double>{f64_of_ff(gx * inv), f64_of_ff(gy * inv), f64_of_ff(gz * inv), f64_of_ff(cn)};
}

template <int DUMMY = 0>
__global__ void __launch_bounds__(256) k_curvature_list_ff(const Nrm<double> *__restrict__ cn, double *__restrict__ curv,
                                                           const uint32_t *__restrict__ cl, int n, const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_cell(cl[t], i, j, k);
    constexpr ff c1 = ff_const(ISO4_1), c2 = ff_const(ISO4_2);
    auto X = [&](int a, int b, int c) { return ff_from_f64(cn[L.i2(i + a, j + b, k + c)].x); };
    auto Y = [&](int a, int b, int c) { return ff_from_f64(cn[L.i2(i + a, j + b, k + c)].y); };
    auto Z = [&](int a, int b, int c) { return ff_from_f64(cn[L.i2(i + a, j + b, k + c)].z); };
    const ff kxx = c1 * (X(1, 0, 0) - X(-1, 0, 0)) +
                   c2 * (X(1, 1, 0) - X(-1, -1, 0) + X(1, -1, 0) - X(-1, 1, 0) + X(1, 0, 1) - X(-1, 0, -1) + X(1, 0, -1) - X(-1, 0, 1));
    const ff kyy = c1 * (Y(0, 1, 0) - Y(0, -1, 0)) +
                   c2 * (Y(1, 1, 0) - Y(-1, -1, 0) + Y(-1, 1, 0) - Y(1, -1, 0) + Y(0, 1, 1) - Y(0, -1, -1) + Y(0, 1, -1) - Y(0, -1, 1));
    const ff kzz = c1 * (Z(0, 0, 1) - Z(0, 0, -1)) +
                   c2 * (Z(1, 0, 1) - Z(-1, 0, -1) + Z(-1, 0, 1) - Z(1, 0, -1) + Z(0, 1, 1) - Z(0, -1, -1) + Z(0, -1, 1) - Z(0, 1, -1));
    const ff kxy = c1 * (X(0, 1, 0) - X(0, -1, 0)) +
                   c2 * (X(1, 1, 0) - X(-1, -1, 0) + X(-1, 1, 0) - X(1, -1, 0) + X(0, 1, 1) - X(0, -1, -1) + X(0, 1, -1) - X(0, -1, 1));
    const ff kxz = c1 * (X(0, 0, 1) - X(0, 0, -1)) +
                   c2 * (X(1, 0, 1) - X(-1, 0, -1) + X(-1, 0, 1) - X(1, 0, -1) + X(0, 1, 1) - X(0, -1, -1) + X(0, -1, 1) - X(0, 1, -1));
    const ff kyx = c1 * (Y(1, 0, 0) - Y(-1, 0, 0)) +
                   c2 * (Y(1, 1, 0) - Y(-1, -1, 0) + Y(1, -1, 0) - Y(-1, 1, 0) + Y(1, 0, 1) - Y(-1, 0, -1) + Y(1, 0, -1) - Y(-1, 0, 1));
    const ff kyz = c1 * (Y(0, 0, 1) - Y(0, 0, -1)) +
                   c2 * (Y(1, 0, 1) - Y(-1, 0, -1) + Y(-1, 0, 1) - Y(1, 0, -1) + Y(0, 1, 1) - Y(0, -1, -1) + Y(0, -1, 1) - Y(0, 1, -1));
    const ff kzx = c1 * (Z(1, 0, 0) - Z(-1, 0, 0)) +
                   c2 * (Z(1, 1, 0) - Z(-1, -1, 0) + Z(1, -1, 0) - Z(-1, 1, 0) + Z(1, 0, 1) - Z(-1, 0, -1) + Z(1, 0, -1) - Z(-1, 0, 1));
    const ff kzy = c1 * (Z(0, 1, 0) - Z(0, -1, 0)) +
                   c2 * (Z(1, 1, 0) - Z(-1, -1, 0) + Z(-1, 1, 0) - Z(1, -1, 0) + Z(0, 1, 1) - Z(0, -1, -1) + Z(0, 1, -1) - Z(0, -1, 1));
    const ff cx = X(0, 0, 0), cy = Y(0, 0, 0), cz = Z(0, 0, 0);
    const ff one(1.0f);
    curv[L.i1(i, j, k)] = f64_of_ff((cx * cx - one) * kxx + (cy * cy - one) * kyy + (cz * cz - one) * kzz +
                                    cx * cy * (kxy + kyx) + cx * cz * (kxz + kzx) + cy * cz * (kzy + kyz));
}

// geometric wetting at fluid-boundary nodes (alter_color_gradient_solid_surface, :210-265)

template <class T>
__global__ void k_wetting(Nrm<T> *__restrict__ cn, const FluidBnd *__restrict__ fb, int nf, const Layout L,
                          const T min_one_m) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf) return;
    const FluidBnd b = fb[t];
    const int64_t id = L.i2(b.ix, b.iy, b.iz);
    const Nrm<T> v = cn[id];
    if (v.n > T(1e-6)) {
        T n[3] = {v.x, v.y, v.z};
        wetting_normal<T>(n, T(b.nwx), T(b.nwy), T(b.nwz), T(b.cos_t), T(b.sin_t), min_one_m);
        cn[id] = Nrm<T>{n[0], n[1], n[2], v.n};
    }
}

// normal extrapolation to solid-boundary nodes inside [0, n+1]^3 (:85-110)
template <class T>
__global__ void k_extrap_normals(Nrm<T> *__restrict__ cn,
                                 const SolidBnd *__restrict__ sb, int ns, const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const SolidBnd s = sb[t];
    if (!(s.ix >= 0 && s.ix <= L.nx + 1 && s.iy >= 0 && s.iy <= L.ny + 1 && s.iz >= 0 && s.iz <= L.nz + 1)) return;
    T ax = T(0.0), ay = T(0.0), az = T(0.0);
    for (int n = 0; n < s.i_fluid_num; ++n) {
        const int ie = s.nbr[n];
        // ie is 1..18 (validated on upload)
        const int dx = c_ex[ie], dy = c_ey[ie], dz = c_ez[ie];
        const T w = ie <= 6 ? T(w_equ_1) : T(w_equ_2);
        const int64_t nb = L.i2(s.ix + dx, s.iy + dy, s.iz + dz);
        const Nrm<T> v = cn[nb];
        ax = ax + v.x * w;
        ay = ay + v.y * w;
        az = az + v.z * w;
    }
    const int64_t id = L.i2(s.ix, s.iy, s.iz);
    const T lw = T(s.la_weight);
    cn[id].x = ax / lw;
    cn[id].y = ay / lw;
    cn[id].z = az / lw;
}

// FP32 arithmetic with every operation rounded on its own (never contracted into an FMA), so
// an expression gives the same bits in every kernel it is inlined into: the curvature is
// computed both inside the FP32 collision and by its own kernel (for the monitor and
// get_gradient), and the value a reader sees is the one the collision used
struct rnf {
    float v;
    __device__ __forceinline__ rnf(float f) : v(f) {}
    __device__ __forceinline__ explicit rnf(double d) : v((float)d) {}
};
__device__ __forceinline__ rnf operator+(rnf a, rnf b) { return rnf(__fadd_rn(a.v, b.v)); }
__device__ __forceinline__ rnf operator-(rnf a, rnf b) { return rnf(__fsub_rn(a.v, b.v)); }
__device__ __forceinline__ rnf operator*(rnf a, rnf b) { return rnf(__fmul_rn(a.v, b.v)); }

// curvature from accessors X, Y, Z of cn_x, cn_y, cn_z at offset (a, b, c) (:113-201)
template <class T, class FX, class FY, class FZ>
__device__ __forceinline__ T curvature_expr(FX X, FY Y, FZ Z);

template <class T, class FX, class FY, class FZ>
__device__ __forceinline__ T curvature_of(FX X, FY Y, FZ Z) {
    if constexpr (std::is_same<T, float>::value) {
        auto Xr = [&](int a, int b, int c) { return rnf(X(a, b, c)); };
        auto Yr = [&](int a, int b, int c) { return rnf(Y(a, b, c)); };
        auto Zr = [&](int a, int b, int c) { return rnf(Z(a, b, c)); };
        return curvature_expr<rnf>(Xr, Yr, Zr).v;
    } else {
        return curvature_expr<T>(X, Y, Z);
    }
}

template <class T, class FX, class FY, class FZ>
__device__ __forceinline__ T curvature_expr(FX X, FY Y, FZ Z) {
    const T c1 = T(ISO4_1), c2 = T(ISO4_2);
    const T kxx = c1 * (X(1, 0, 0) - X(-1, 0, 0)) +
                       c2 * (X(1, 1, 0) - X(-1, -1, 0) + X(1, -1, 0) - X(-1, 1, 0) + X(1, 0, 1) - X(-1, 0, -1) + X(1, 0, -1) - X(-1, 0, 1));
    const T kyy = c1 * (Y(0, 1, 0) - Y(0, -1, 0)) +
                       c2 * (Y(1, 1, 0) - Y(-1, -1, 0) + Y(-1, 1, 0) - Y(1, -1, 0) + Y(0, 1, 1) - Y(0, -1, -1) + Y(0, 1, -1) - Y(0, -1, 1));
    const T kzz = c1 * (Z(0, 0, 1) - Z(0, 0, -1)) +
                       c2 * (Z(1, 0, 1) - Z(-1, 0, -1) + Z(-1, 0, 1) - Z(1, 0, -1) + Z(0, 1, 1) - Z(0, -1, -1) + Z(0, -1, 1) - Z(0, 1, -1));
    const T kxy = c1 * (X(0, 1, 0) - X(0, -1, 0)) +
                       c2 * (X(1, 1, 0) - X(-1, -1, 0) + X(-1, 1, 0) - X(1, -1, 0) + X(0, 1, 1) - X(0, -1, -1) + X(0, 1, -1) - X(0, -1, 1));
    const T kxz = c1 * (X(0, 0, 1) - X(0, 0, -1)) +
                       c2 * (X(1, 0, 1) - X(-1, 0, -1) + X(-1, 0, 1) - X(1, 0, -1) + X(0, 1, 1) - X(0, -1, -1) + X(0, -1, 1) - X(0, 1, -1));
    const T kyx = c1 * (Y(1, 0, 0) - Y(-1, 0, 0)) +
                       c2 * (Y(1, 1, 0) - Y(-1, -1, 0) + Y(1, -1, 0) - Y(-1, 1, 0) + Y(1, 0, 1) - Y(-1, 0, -1) + Y(1, 0, -1) - Y(-1, 0, 1));
    const T kyz = c1 * (Y(0, 0, 1) - Y(0, 0, -1)) +
                       c2 * (Y(1, 0, 1) - Y(-1, 0, -1) + Y(-1, 0, 1) - Y(1, 0, -1) + Y(0, 1, 1) - Y(0, -1, -1) + Y(0, -1, 1) - Y(0, 1, -1));
    const T kzx = c1 * (Z(1, 0, 0) - Z(-1, 0, 0)) +
                       c2 * (Z(1, 1, 0) - Z(-1, -1, 0) + Z(1, -1, 0) - Z(-1, 1, 0) + Z(1, 0, 1) - Z(-1, 0, -1) + Z(1, 0, -1) - Z(-1, 0, 1));
    const T kzy = c1 * (Z(0, 1, 0) - Z(0, -1, 0)) +
                       c2 * (Z(1, 1, 0) - Z(-1, -1, 0) + Z(-1, 1, 0) - Z(1, -1, 0) + Z(0, 1, 1) - Z(0, -1, -1) + Z(0, 1, -1) - Z(0, -1, 1));
    const T cx = X(0, 0, 0), cy = Y(0, 0, 0), cz = Z(0, 0, 0);
    return (cx * cx - T(1.0)) * kxx + (cy * cy - T(1.0)) * kyy + (cz * cz - T(1.0)) * kzz + cx * cy * (kxy + kyx) +
           cx * cz * (kxz + kzx) + cy * cz * (kzy + kyz);
}

template <class T>
__device__ __forceinline__ void curvature_at(const Nrm<T> *__restrict__ cn, T *__restrict__ curv, int i, int j, int k,
                                             const Layout &L) {
    auto X = [&](int a, int b, int c) { return cn[L.i2(i + a, j + b, k + c)].x; };
    auto Y = [&](int a, int b, int c) { return cn[L.i2(i + a, j + b, k + c)].y; };
    auto Z = [&](int a, int b, int c) { return cn[L.i2(i + a, j + b, k + c)].z; };
    curv[L.i1(i, j, k)] = curvature_of<T>(X, Y, Z);
}

// over [1, n]^3, every cell
template <class T>
__global__ void __launch_bounds__(256) k_curvature(const Nrm<T> *__restrict__ cn, T *__restrict__ curv,
                                                   const int8_t *__restrict__ walls, const Layout L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > L.nx || j > L.ny) return;
#ifndef MFLBM_STRICT
    // curv is read only at fluid nodes (collision, compute_macro_vars masks walls); the
    // default build leaves 0 at wall nodes instead of the reference's unused value
    if (walls[L.i2(i, j, k)] != 0) {
        curv[L.i1(i, j, k)] = T(0.0);
        return;
    }
#endif
    curvature_at<T>(cn, curv, i, j, k, L);
}

template <class T>
__global__ void MFLBM_GRAD_BOUNDS k_curvature_list(const Nrm<T> *__restrict__ cn, T *__restrict__ curv,
                                                        const uint32_t *__restrict__ cl, int n, const Layout L) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_cell(cl[t], i, j, k);
    curvature_at<T>(cn, curv, i, j, k, L);
}

// Shared-memory forms of the two stencils (default build): a block of 32 x 8 threads owns
// a 32 x 8 column of cells and marches it up a chunk of GRAD_KCH planes.  The planes
// k-1, k, k+1 of the input field(s), with a one-cell halo in i and j, sit in a ring of
// three shared-memory planes; each step stores the plane that was prefetched into
// registers during the previous step, then issues the loads of the next one before
// computing, so global loads overlap the stencil arithmetic.  Every input value is read
// from global memory once per column (plus the halo) instead of once per neighbour, with
// coalesced rows.  Outputs go to the same cells as the fluid-cell lists (normals: walls != 1
// in [-1, n+2]^3; curvature: walls == 0 in [1, n]^3) with the same expressions.
constexpr int GRAD_TX = 32, GRAD_TY = 8, GRAD_KCH = 16;
constexpr int GRAD_PW = GRAD_TX + 2, GRAD_PH = GRAD_TY + 2, GRAD_PN = GRAD_PW * GRAD_PH;
constexpr int GRAD_LD = (GRAD_PN + GRAD_TX * GRAD_TY - 1) / (GRAD_TX * GRAD_TY);   // loads per thread per plane

// NF input fields of halo h (stride hx, hxy in elements, origin offset o so that cell
// (i, j, k) is at o + i + hx j + hxy k), valid for i in [-h+1, nx+h] etc.
template <class T, int NF>
struct GradPlanes {
    const T *src[NF];
    int64_t hx, hxy, o;
    int es;                 // elements between consecutive cells (1: a plain field, 4: a Nrm record component)
    int imax, jmax, kmax;   // largest valid index per axis
    __device__ __forceinline__ void fetch(T (&r)[NF][GRAD_LD], int i0, int j0, int k, int tid) const {
#pragma unroll
        for (int l = 0; l < GRAD_LD; ++l) {
            const int idx = tid + l * GRAD_TX * GRAD_TY;
            const int ii = idx % GRAD_PW, jj = idx / GRAD_PW;
            const int i = i0 - 1 + ii, j = j0 - 1 + jj;
            const bool ok = idx < GRAD_PN && i <= imax && j <= jmax && k <= kmax;
            const int64_t a = o + i + hx * j + hxy * k;
#pragma unroll
            for (int f = 0; f < NF; ++f) r[f][l] = ok ? src[f][a * es] : T(0.0);
        }
    }
    __device__ __forceinline__ void put(T (*sm)[3][GRAD_PN], const T (&r)[NF][GRAD_LD], int slot, int tid) const {
#pragma unroll
        for (int l = 0; l < GRAD_LD; ++l) {
            const int idx = tid + l * GRAD_TX * GRAD_TY;
            if (idx < GRAD_PN) {
#pragma unroll
                for (int f = 0; f < NF; ++f) sm[f][slot][idx] = r[f][l];
            }
        }
    }
};

template <class T>
__global__ void __launch_bounds__(GRAD_TX *GRAD_TY) k_normals_tile(const T *__restrict__ phi,
                                                                    const int8_t *__restrict__ walls,
                                                                    Nrm<T> *__restrict__ out, const Layout L) {
    __shared__ T sm[1][3][GRAD_PN];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + GRAD_TX * ty;
    const int i0 = -1 + (int)blockIdx.x * GRAD_TX, j0 = -1 + (int)blockIdx.y * GRAD_TY;
    const int kb = -1 + (int)blockIdx.z * GRAD_KCH;
    const int ke = min(kb + GRAD_KCH - 1, L.nz + 2);
    GradPlanes<T, 1> g;
    g.src[0] = phi;
    g.es = 1;
    g.hx = L.h4x; g.hxy = L.h4xy; g.o = 3 + 3 * L.h4x + 3 * L.h4xy;
    g.imax = L.nx + 4; g.jmax = L.ny + 4; g.kmax = L.nz + 4;
    T r[1][GRAD_LD];
    g.fetch(r, i0, j0, kb - 1, tid);
    g.put(sm, r, (kb - 1 + 3) % 3, tid);
    g.fetch(r, i0, j0, kb, tid);
    g.put(sm, r, (kb + 3) % 3, tid);
    g.fetch(r, i0, j0, kb + 1, tid);
    const int i = i0 + tx, j = j0 + ty;
    const bool in_ij = i <= L.nx + 2 && j <= L.ny + 2;
    for (int k = kb; k <= ke; ++k) {
        g.put(sm, r, (k + 1 + 3) % 3, tid);
        __syncthreads();
        if (k + 1 < ke + 1) g.fetch(r, i0, j0, k + 2, tid);
        if (in_ij) {
            const int64_t id = L.i2(i, j, k);
            if (walls[id] != 1) {
                auto P = [&](int a, int b, int c) { return sm[0][(k + c + 3) % 3][(tx + 1 + a) + GRAD_PW * (ty + 1 + b)]; };
                T gx, gy, gz, cn;
                normals_of<T>(P, gx, gy, gz, cn);
                out[id] = Nrm<T>{gx, gy, gz, cn};
            }
        }
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(GRAD_TX *GRAD_TY) k_curvature_tile(const Nrm<T> *__restrict__ cn, T *__restrict__ curv,
                                                                      const int8_t *__restrict__ walls, const Layout L) {
    __shared__ T sm[3][3][GRAD_PN];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + GRAD_TX * ty;
    const int i0 = 1 + (int)blockIdx.x * GRAD_TX, j0 = 1 + (int)blockIdx.y * GRAD_TY;
    const int kb = 1 + (int)blockIdx.z * GRAD_KCH;
    const int ke = min(kb + GRAD_KCH - 1, L.nz);
    GradPlanes<T, 3> g;
    g.src[0] = &cn[0].x; g.src[1] = &cn[0].y; g.src[2] = &cn[0].z;
    g.es = 4;
    g.hx = L.h2x; g.hxy = L.h2xy; g.o = 1 + L.h2x + L.h2xy;
    g.imax = L.nx + 2; g.jmax = L.ny + 2; g.kmax = L.nz + 2;
    T r[3][GRAD_LD];
    g.fetch(r, i0, j0, kb - 1, tid);
    g.put(sm, r, (kb - 1) % 3, tid);
    g.fetch(r, i0, j0, kb, tid);
    g.put(sm, r, kb % 3, tid);
    g.fetch(r, i0, j0, kb + 1, tid);
    const int i = i0 + tx, j = j0 + ty;
    const bool in_ij = i <= L.nx && j <= L.ny;
    for (int k = kb; k <= ke; ++k) {
        g.put(sm, r, (k + 1) % 3, tid);
        __syncthreads();
        if (k + 1 < ke + 1) g.fetch(r, i0, j0, k + 2, tid);
        if (in_ij && walls[L.i2(i, j, k)] == 0) {
            const int c0 = (tx + 1) + GRAD_PW * (ty + 1);
            auto X = [&](int a, int b, int c) { return sm[0][(k + c) % 3][c0 + a + GRAD_PW * b]; };
            auto Y = [&](int a, int b, int c) { return sm[1][(k + c) % 3][c0 + a + GRAD_PW * b]; };
            auto Z = [&](int a, int b, int c) { return sm[2][(k + c) % 3][c0 + a + GRAD_PW * b]; };
            curv[L.i1(i, j, k)] = curvature_of<T>(X, Y, Z);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------
// compute_macro_vars fused with the per-slice monitor reductions
// (Misc.F90:372-430; Monitor.F90:27-85; singlephase Misc.F90:368-423, Monitor.F90:18-59).
// One block per z slice.  Each block writes its slice sums and its umax/usq partials to
// out[nq][nz]; the host finishes the global max/sums in slice order, so the result is
// independent of scheduling.  Accumulation is FP64 for every storage type.
// ---------------------------------------------------------------------------------
constexpr int MON_THREADS = 256;
constexpr int MON_NQ = 10;  // fl1 fl2 vol1 vol2 mass1 mass2 pre | umax usq1 usq2

template <class S>
__global__ void __launch_bounds__(MON_THREADS) k_monitor(const S *__restrict__ f, const S *__restrict__ g,
                                                         typename Store<S>::R *__restrict__ phi, const int8_t *__restrict__ walls,
                                                         const Nrm<typename Store<S>::R> *__restrict__ cn,
                                                         const typename Store<S>::R *__restrict__ curv, double *__restrict__ u,
                                                         double *__restrict__ v, double *__restrict__ w, double *__restrict__ rho,
                                                         double *__restrict__ out, const Layout L, const PdfAt pa,
                                                         const StepParams P, int multiphase, int write_fields, float ref,
                                                         float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int k = blockIdx.x + 1;
    const int64_t n = (int64_t)L.nx * L.ny;
    double acc[MON_NQ];
#pragma unroll
    for (int m = 0; m < MON_NQ; ++m) acc[m] = 0.0;
    const R inv = R(1.0f / scale);
    for (int64_t t = threadIdx.x; t < n; t += MON_THREADS) {
        const int i = (int)(t % L.nx) + 1, j = (int)(t / L.nx) + 1;
        const int wi = walls[L.i2(i, j, k)];
        const int64_t c = pa.slot(L, i, j, k);
        double ft[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            double a = St::ld64(f, (int64_t)q * pa.qs + c, WREST(q) * ref, inv);
            if (multiphase) a = a + St::ld64(g, (int64_t)q * pa.qs + c, WREST(q) * ref, inv);
            ft[q] = a;
        }
        const double m = (double)(1 - wi);
        const double rr = (ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] + ft[11] +
                           ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18]) * m;
        double fx = 0.0, fy = 0.0, fz = P.force_z;
        const int64_t i1 = L.i1(i, j, k);
        if (multiphase) {
            const int64_t i2 = L.i2(i, j, k);
            const Nrm<typename Store<S>::R> nr = cn[i2];
            const double tmp = 0.5 * P.gamma * (double)curv[i1] * (double)nr.n;
            fx = tmp * (double)nr.x;
            fy = tmp * (double)nr.y;
            fz = tmp * (double)nr.z + P.force_z;
        }
        const double uu = (ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] - 0.5 * fx) * m;
        const double vv = (ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] - 0.5 * fy) * m;
        const double ww = (ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] - 0.5 * fz) * m;
        if (write_fields) { u[i1] = uu; v[i1] = vv; w[i1] = ww; rho[i1] = rr; }
        const double temp = multiphase ? (uu * uu + vv * vv + ww * ww) * m : uu * uu + vv * vv + ww * ww;
        acc[7] = (acc[7] < temp) ? temp : acc[7];
        if (multiphase) {
            const int64_t i4 = L.i4(i, j, k);
            const double ph = 0.0 * (double)wi + (double)phi[i4] * m;
            phi[i4] = (R)ph;
            if (ph > 0.999) acc[8] += temp;
            else if (ph < -0.999) acc[9] += temp;
            acc[2] += 0.5 * (1.0 + ph) * m;
            acc[3] += 0.5 * (1.0 - ph) * m;
            acc[4] += rr * 0.5 * (1.0 + ph) * m;
            acc[5] += rr * 0.5 * (1.0 - ph) * m;
            acc[0] += ww * 0.5 * (1.0 + ph) * m;
            acc[1] += ww * 0.5 * (1.0 - ph) * m;
            acc[6] += rr * m;
        } else {
            acc[0] += ww;
            acc[6] += rr;
        }
    }
    // warp shuffle, then shared memory across warps (fixed order -> deterministic)
    __shared__ double red[MON_THREADS / 32][MON_NQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int m = 0; m < MON_NQ; ++m) {
        double x = acc[m];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = m == 7 ? ((x < y) ? y : x) : x + y;
        }
        if (lane == 0) red[wid][m] = x;
    }
    __syncthreads();
    if (threadIdx.x < MON_NQ) {
        const int m = threadIdx.x;
        double x = red[0][m];
        for (int q = 1; q < MON_THREADS / 32; ++q) x = m == 7 ? ((x < red[q][m]) ? red[q][m] : x) : x + red[q][m];
        out[(int64_t)m * L.nz + (k - 1)] = x;
    }
}

// cal_saturation partial sums per slice (Monitor.F90:512-550)
template <class T>
__global__ void __launch_bounds__(MON_THREADS) k_saturation(const T *__restrict__ phi, const int8_t *__restrict__ walls,
                                                            double *__restrict__ out, const Layout L) {
    const int k = blockIdx.x + 1;
    const int64_t n = (int64_t)L.nx * L.ny;
    double v1 = 0.0, v2 = 0.0;
    for (int64_t t = threadIdx.x; t < n; t += MON_THREADS) {
        const int i = (int)(t % L.nx) + 1, j = (int)(t / L.nx) + 1;
        const double m = (double)(1 - walls[L.i2(i, j, k)]);
        const double ph = (double)phi[L.i4(i, j, k)];
        v1 += 0.5 * (1.0 + ph) * m;
        v2 += 0.5 * (1.0 - ph) * m;
    }
    __shared__ double red[2][MON_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
        v2 += __shfl_down_sync(0xffffffffu, v2, o);
    }
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = v1; red[1][threadIdx.x >> 5] = v2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < MON_THREADS / 32; ++q) { a += red[0][q]; b += red[1][q]; }
        out[k - 1] = a;
        out[L.nz + k - 1] = b;
    }
}

// ---------------------------------------------------------------------------------
// initialisation: equilibrium PDFs at rest, rho = 1 (Init_multiphase.F90:366-415;
// singlephase Initialization.F90:248-276), and the convective-outlet memory (:418-467)
// ---------------------------------------------------------------------------------
template <class S>
__global__ void k_init_eq(S *__restrict__ f, S *__restrict__ g, const typename Store<S>::R *__restrict__ phi, double *__restrict__ u,
                          double *__restrict__ v, double *__restrict__ w, double *__restrict__ rho, const Layout L,
                          const PdfAt pa, int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb) return;
    const int i = (int)(t % (L.nx + 2));
    const int j = (int)((t / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    // t enumerates the halo-1 box in Fortran order, so it is also the u/v/w/rho index
    u[t] = 0.0;
    v[t] = 0.0;
    w[t] = 0.0;
    rho[t] = 1.0;
    if (!pa.owned(L, i, j, k)) return;   // fluid list: the cell has no slot of its own
    const int64_t c = pa.slot(L, i, j, k);
    const double usqrt = 0.0;
    double r0, r1 = 0.0;
    if (multiphase) {
        const double ph = (double)phi[L.i4(i, j, k)];
        r0 = 1.0 * (1.0 + ph) * 0.5;
        r1 = 1.0 * (1.0 - ph) * 0.5;
    } else {
        r0 = 1.0;
    }
    const R sc = R(scale);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const double wq = WEQ(q);
        const double cu = 0.0;
        const double a = q == 0 ? r0 * wq + r0 * wq * (-1.5 * usqrt) : r0 * wq + r0 * wq * (3.0 * cu + 4.5 * cu * cu - 1.5 * usqrt);
        St::st64(f, (int64_t)q * pa.qs + c, a, WREST(q) * ref, scale);
        if (multiphase) {
            const double b = q == 0 ? r1 * wq + r1 * wq * (-1.5 * usqrt) : r1 * wq + r1 * wq * (3.0 * cu + 4.5 * cu * cu - 1.5 * usqrt);
            St::st64(g, (int64_t)q * pa.qs + c, b, WREST(q) * ref, scale);
        }
    }
}

template <class S>
__global__ void k_init_convec(const S *__restrict__ f, const S *__restrict__ g, const typename Store<S>::R *__restrict__ phi,
                              double *__restrict__ fconv, double *__restrict__ gconv, double *__restrict__ phiconv,
                              const Layout L, const PdfAt pa, int multiphase, float ref, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t np = (int64_t)(L.nx + 2) * (L.ny + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np) return;
    const int i = (int)(t % (L.nx + 2)), j = (int)(t / (L.nx + 2));
    const R inv = R(1.0f / scale);
    for (int q = 0; q < 19; ++q) {
        fconv[L.ic(i, j, q)] = St::ld64(f, pa(L, q, i, j, L.nz), WREST(q) * ref, inv);
        if (multiphase)
            gconv[L.ic(i, j, q)] = St::ld64(g, pa(L, q, i, j, L.nz), WREST(q) * ref, inv);
    }
    if (multiphase) phiconv[L.ip(i, j)] = (double)phi[L.i4(i, j, L.nz)];
}

// FP64 <-> storage conversion of one direction plane (upload/download of FP32/FP16 state)
template <class S>
__global__ void k_convert_in(S *__restrict__ dst, const double *__restrict__ src, const Layout L, int q, float ref,
                             float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb) return;
    const int i = (int)(t % (L.nx + 2));
    const int j = (int)((t / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    St::st64(dst, L.cell(i, j, k), src[t], WREST(q) * ref, scale);
}

template <class S>
__global__ void k_convert_out(double *__restrict__ dst, const S *__restrict__ src, const Layout L, int q, float ref,
                              float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb) return;
    const int i = (int)(t % (L.nx + 2));
    const int j = (int)((t / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    dst[t] = St::ld64(src, L.cell(i, j, k), WREST(q) * ref, 1.0f / scale);
}

// ---------------------------------------------------------------------------------
// Fluid-list layout (singlephase samples whose every direction is periodic or walled).
// A_q = A + q*stride holds the fluid nodes [0, nf) and the bounce-back link slots;
// nb[(d-1)*nf + x] is the slot of x + e_d (see listlayout.h).  The arithmetic is the
// dense kernel's (k_sp_step), so the strict flavour stays bit-identical to the oracle.
// ---------------------------------------------------------------------------------
// the singlephase collision of one node in the sweep's arithmetic type (shared by the list
// sweeps): the double-word form, the reference's order (strict build) or the pair form
template <class S, bool UNIT>
__device__ __forceinline__ void sp_collide(typename Store<S>::RS (&ft)[19], const StepParams &P,
                                           const MrtFold<typename Store<S>::RS> &cf) {
    using R = typename Store<S>::RS;
    if constexpr (std::is_same<R, ff>::value) {
        mrt_collide_ff<UNIT>(ft, cf);
    } else {
#ifdef MFLBM_STRICT
        const R den = ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] + ft[11] +
                      ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
        mrt_collide<R>(ft, den, R(0.0), R(0.0), R(P.force_z), R(P.s_e), R(P.s_e2), R(P.s_q), R(P.s_nu), R(P.s_pi),
                       R(P.s_t));
#else
        mrt_collide_pairs<R, false, true, UNIT>(ft, R(0.0), R(0.0), R(0.0), cf.fz, cf);
#endif
    }
}

// the odd step of one fluid node whose 18 neighbour slots are known
template <class S, bool UNIT>
__device__ __forceinline__ void sp_list_odd_node(S *__restrict__ A, const int64_t stride, const int64_t t,
                                                 const int32_t (&nbr)[18], const StepParams &P,
                                                 const MrtFold<typename Store<S>::RS> &cf, const float scale) {
    using R = typename Store<S>::RS;
    const R inv_scale = R(1.0f / scale);
    R ft[19];
    ld_node<S>(ft, A, [&](int q) -> int64_t { return q == 0 ? t : (int64_t)q * stride + nbr[OPP(q) - 1]; },
               inv_scale);
    sp_collide<S, UNIT>(ft, P, cf);
    const R sc = R(scale);
    st_sweep<S>(A, t, 0, ft[0], sc);
#pragma unroll
    for (int q = 1; q < 19; ++q) st_sweep<S>(A, (int64_t)OPP(q) * stride + nbr[q - 1], q, ft[q], sc);
}

// How many blocks ahead the odd list step prefetches the neighbour table into L2 (0: no
// prefetch).  Measured on the 256^3 packing (MLUPS without / 512 / 1024 / 2048 blocks
// ahead): FP16 40,668 / 42,056 / 42,151 / 41,763, double-word storage 15,720 / 15,985 /
// 15,886 / 15,759; FP32 (30,513 without) and FP64 storage with the double-word collision
// (13,072 without) lost about 1 % at every distance, so they do not prefetch.
template <class S> struct TablePrefetch { static constexpr int kAhead = 0; };
template <> struct TablePrefetch<__half> { static constexpr int kAhead = 1024; };
template <> struct TablePrefetch<ffs> { static constexpr int kAhead = 512; };

// one fluid node of the list sweep (shared by the single-sample and ensemble kernels)
template <class S, bool ODD, bool UNIT>
__device__ __forceinline__ void sp_list_node(S *__restrict__ A, const int64_t stride, const int32_t *__restrict__ nb,
                                             const int64_t nf, const int64_t t, const StepParams &P,
                                             const MrtFold<typename Store<S>::RS> &cf, const float scale) {
    if constexpr (ODD) {
        int32_t nbr[18];
#pragma unroll
        for (int d = 0; d < 18; ++d) nbr[d] = __ldcs(nb + (int64_t)d * nf + t);   // streamed: read once per step
        sp_list_odd_node<S, UNIT>(A, stride, t, nbr, P, cf, scale);
    } else {
        using R = typename Store<S>::RS;
        const R inv_scale = R(1.0f / scale);
        R ft[19];
        ld_node<S>(ft, A, [&](int q) -> int64_t { return (int64_t)OPP(q) * stride + t; }, inv_scale);
        sp_collide<S, UNIT>(ft, P, cf);
        const R sc = R(scale);
#pragma unroll
        for (int q = 0; q < 19; ++q) st_sweep<S>(A, (int64_t)q * stride + t, q, ft[q], sc);
    }
}

template <class S, bool ODD, bool UNIT>
__global__ void __launch_bounds__(128, SweepOcc<S>::kMinBlocks) k_sp_list(S *__restrict__ A, const int64_t stride, const int32_t *__restrict__ nb,
                                                 const int nf, const StepParams P,
                                                 const MrtFold<typename Store<S>::RS> cf, const float scale) {
    if constexpr (ODD && TablePrefetch<S>::kAhead > 0) {
        // L2 prefetch of the neighbour-table rows of the block kAhead blocks ahead, so its
        // table reads wait on L2, not DRAM: 72 threads, one 128-byte line each (4 lines of
        // each of the 18 rows)
        const int64_t first = ((int64_t)blockIdx.x + TablePrefetch<S>::kAhead) * 128 + (threadIdx.x & 3) * 32;
        if (threadIdx.x < 72 && first < nf)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(nb + (int64_t)(threadIdx.x >> 2) * nf + first));
    }
    const int t = list_node_index<ODD>();
    if (t >= nf) return;
    sp_list_node<S, ODD, UNIT>(A, stride, nb, nf, t, P, cf, scale);
}


// ---------------------------------------------------------------------------------
// The even step of the list sweep through the tensor memory accelerator (TMA).  The even
// step reads A_opp(q)[x] and writes A_q[x] over a contiguous range of fluid nodes, so one
// tiled load brings a 19 x 128 box (every direction array, 128 consecutive nodes) into
// shared memory, the collision runs from there, and one tiled store writes the box back.
// A persistent grid walks the tiles.  In each block one thread of warp 4 issues the copies
// and warps 0-3 compute, one node per thread; two shared-memory stages let the load of the
// next tile and the store of the last one overlap the arithmetic.  Stage hand-over uses
// mbarriers: `full` completes with the load's byte count, `empty` when all 128 computing
// threads have written their results (and fenced them for the async proxy).  Only whole
// tiles go through the copies, so no box reaches past the nf fluid nodes into the link
// slots that follow them (a store clipped at the tensor's extent is clipped at 16-byte
// granularity, which would reach the first link slot when nf * element size is not a
// multiple of 16); the last block updates the nf % 128 remaining nodes with plain loads
// and stores.  Every wait is bounded; a wait that runs out sets *err, and the copy thread
// waits (bounded again) for the loads it issued before the block exits.
// ---------------------------------------------------------------------------------
constexpr int kTmaNodes = 128;            // nodes per tile = computing threads per block
constexpr long long kTmaWait = 1ll << 26; // probes of one wait before it gives up

// bytes of one tile and shared-memory stages per block: two for 8-byte populations (the
// arithmetic is long, two tiles in flight cover the copies), four for 4- and 2-byte ones
// (short arithmetic: more tiles in flight keep HBM busy; FP16 with 2 / 4 / 8 stages:
// 40,775 / 41,873 / 42,173 MLUPS on the 256^3 packing)
template <class S> struct TmaTile {
    static constexpr int bytes = 19 * kTmaNodes * (int)sizeof(S);
    static constexpr int stages = sizeof(S) >= 8 ? 2 : 4;
};

template <class S, bool UNIT>
__global__ void __launch_bounds__(kTmaNodes + 32, 4)
    k_sp_list_even_tma(const __grid_constant__ CUtensorMap map, S *__restrict__ A, const int64_t stride, const int nf,
                       const StepParams P, const MrtFold<typename Store<S>::RS> cf, const float scale,
                       int32_t *__restrict__ err) {
    constexpr int NS = TmaTile<S>::stages;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t full[NS], empty[NS];
    S *tiles = reinterpret_cast<S *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x;
    const int ntiles = nf / kTmaNodes;   // whole tiles only
    const int m = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    // the n-th tile of this block (last tile first when the even steps walk backwards)
    auto tile_of = [&](int n) -> int {
        const int k = (int)blockIdx.x + n * (int)gridDim.x;
        return MFLBM_EVEN_REVERSE ? ntiles - 1 - k : k;
    };
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            bulk::mbar_init(&full[s], 1);
            bulk::mbar_init(&empty[s], kTmaNodes);
        }
        bulk::fence_mbar_init();
    }
    __syncthreads();
    if (tid >= kTmaNodes) {
        if (tid != kTmaNodes) return;
        // copy thread: tile n goes to stage n % NS; before reloading a stage, the
        // results of the tile it held are stored and the store has read them out
        int last_load[NS];
        for (int s = 0; s < NS; ++s) last_load[s] = -1;
        bool ok = true;
        for (int n = 0; n < m + NS; ++n) {
            const int s = n % NS;
            S *buf = tiles + s * 19 * kTmaNodes;
            if (n >= NS) {
                const int np = n - NS;
                if (!bulk::mbar_wait(&empty[s], (uint32_t)((np / NS) & 1), kTmaWait)) {
                    ok = false;
                    break;
                }
                bulk::tma_store_2d(&map, tile_of(np) * kTmaNodes, 0, buf);
                bulk::bulk_commit();
                bulk::bulk_wait_read0();
            }
            if (n < m) {
                bulk::mbar_arrive_expect_tx(&full[s], (uint32_t)TmaTile<S>::bytes);
                bulk::tma_load_2d(buf, &map, tile_of(n) * kTmaNodes, 0, &full[s]);
                last_load[s] = n;
            }
        }
        bulk::bulk_wait0();
        if (!ok) {
            atomicExch(err, 1);
            for (int s = 0; s < NS; ++s)
                if (last_load[s] >= 0)
                    (void)bulk::mbar_wait(&full[s], (uint32_t)((last_load[s] / NS) & 1), kTmaWait);
        }
        return;
    }
    using R = typename Store<S>::RS;
    const R inv_scale = R(1.0f / scale);
    const R sc = R(scale);
    for (int n = 0; n < m; ++n) {
        const int s = n % NS;
        S *buf = tiles + s * 19 * kTmaNodes;
        if (!bulk::mbar_wait(&full[s], (uint32_t)((n / NS) & 1), kTmaWait)) {
            atomicExch(err, 1);
            break;
        }
        R ft[19];
        ld_node<S>(ft, buf, [&](int q) -> int64_t { return (int64_t)OPP(q) * kTmaNodes + tid; }, inv_scale);
        sp_collide<S, UNIT>(ft, P, cf);
#pragma unroll
        for (int q = 0; q < 19; ++q) st_sweep<S>(buf, (int64_t)q * kTmaNodes + tid, q, ft[q], sc);
        bulk::fence_async_smem();
        bulk::mbar_arrive(&empty[s]);
    }
    // the nodes after the last whole tile, by the last block, from global memory
    if (blockIdx.x == gridDim.x - 1) {
        const int t = ntiles * kTmaNodes + tid;
        if (t < nf) sp_list_node<S, false, UNIT>(A, stride, nullptr, nf, t, P, cf, scale);
    }
}

// ---------------------------------------------------------------------------------
// Ensembles: many samples share one fluid-list arena (fluid nodes of all samples first,
// then all link slots); a tile is a run of at most blockDim fluid nodes of one sample.
// The tile table and its length live in device memory, so a captured graph keeps
// working when the host drops converged samples from the table.
// ---------------------------------------------------------------------------------
template <class R> __device__ __forceinline__ const MrtFold<R> &ens_fold(const EnsArgs &a);
template <> __device__ __forceinline__ const MrtFold<double> &ens_fold<double>(const EnsArgs &a) { return a.fold; }
template <> __device__ __forceinline__ const MrtFold<float> &ens_fold<float>(const EnsArgs &a) { return a.fold32; }
template <> __device__ __forceinline__ const MrtFold<ff> &ens_fold<ff>(const EnsArgs &a) { return a.foldff; }

template <class S, bool ODD, bool UNIT>
__device__ __forceinline__ void ens_sweep(const EnsArgs &a) {
    const int nt = *a.ntiles;
    for (int tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        const EnsTile T = a.tiles[tile];
        if ((int)threadIdx.x < T.count)
            sp_list_node<S, ODD, UNIT>(reinterpret_cast<S *>(a.A), a.stride, a.nb, a.nf, (int64_t)T.start + threadIdx.x, a.P,
                                 ens_fold<typename Store<S>::RS>(a), a.scale);
    }
}

// one step over the active tiles (grid-stride over the tile table)
template <class S, bool ODD, bool UNIT>
__global__ void k_ens_step(const EnsArgs a) {
    ens_sweep<S, ODD, UNIT>(a);
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident).  Sense by
// generation counter; the wait is bounded: after `limit` polls the block sets *err and
// every other block leaves at its next poll.  The last of gridDim.x + extra arrivals
// opens the barrier; extra is 0 except in the timeout test, where nobody can open it.
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, int32_t *err, long long limit, unsigned int extra) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int *vgen = bar + 1;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1 + extra) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                if (++it > limit || *(volatile int32_t *)err) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// nsteps AA steps in one cooperative launch, a grid barrier between consecutive steps
template <class S, bool UNIT>
__global__ void k_ens_persistent(const EnsArgs a) {
    for (int s = 0; s < a.nsteps; ++s) {
        if (((a.ntime0 + s) & 1) != 0) ens_sweep<S, true, UNIT>(a);
        else ens_sweep<S, false, UNIT>(a);
        if (s + 1 < a.nsteps && !grid_barrier(a.bar, a.err, a.spin_limit, a.bar_extra)) return;
    }
}

// equilibrium at rest (r0 = 1, u = 0: f_q = w_q) in every slot of the list arrays
template <class S>
__global__ void k_list_init(S *__restrict__ A, const int64_t stride, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 19 * stride) return;
    const int q = (int)(t / stride);
    St::st64(A, t, WEQ(q), WREST(q), scale);
}

// dense FP64 plane q (halo-1 Fortran order, in stage) -> list slots of direction q
template <class S>
__global__ void k_list_in(S *__restrict__ A, const int64_t stride, const int q, const int32_t *__restrict__ cell1,
                          const int nf, const int32_t *__restrict__ link, const int64_t nlink,
                          const double *__restrict__ stage, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    S *Aq = A + (int64_t)q * stride;
    if (t < nf) {
        St::st64(Aq, t, stage[cell1[t]], WREST(q), scale);
    } else if (t - nf < nlink) {
        const int64_t l = t - nf;
        if (link[3 * l] == q) St::st64(Aq, link[3 * l + 1], stage[link[3 * l + 2]], WREST(q), scale);
    }
}

// list slots of direction q -> dense FP64 plane (stage): every cell first gets the rest
// equilibrium w_q (the value the reference's untouched slots keep after
// initialisation), then the fluid nodes and link slots are scattered, then the ghost
// layers of periodic directions receive their periodic images.
static __global__ void k_list_plane_fill(double *__restrict__ stage, int64_t n, double v) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) stage[t] = v;
}

template <class S>
__global__ void k_list_out(const S *__restrict__ A, const int64_t stride, const int q, const int32_t *__restrict__ cell1,
                           const int nf, const int32_t *__restrict__ link, const int64_t nlink,
                           double *__restrict__ stage, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const S *Aq = A + (int64_t)q * stride;
    const R inv = R(1.0f / scale);
    if (t < nf) {
        stage[cell1[t]] = St::ld64(Aq, t, WREST(q), 1.0f / scale);
    } else if (t - nf < nlink) {
        const int64_t l = t - nf;
        if (link[3 * l] == q) stage[link[3 * l + 2]] = St::ld64(Aq, link[3 * l + 1], WREST(q), 1.0f / scale);
    }
}

// ---------------------------------------------------------------------------------
// The multiphase fluid list (listlayout.h, MpListLayout): the boundary planes' private slots
// (map >= nf) against a dense FP64 image of one direction in `stage` (halo-1 Fortran
// order), the equilibrium of the link slots, and change_inlet_fluid_phase on them.  Fluid
// nodes and link slots move through k_list_in / k_list_out as in the singlephase list.
// ---------------------------------------------------------------------------------
template <class S>
__global__ void k_mp_planes_in(S *__restrict__ A, const int64_t stride, const int q, const int32_t *__restrict__ map,
                               const int nf, const int64_t n1, const double *__restrict__ stage, float scale) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1) return;
    const int32_t m = map[t];
    if (m >= nf) Store<S>::st64(A + (int64_t)q * stride, m, stage[t], WREST(q), scale);
}

template <class S>
__global__ void k_mp_planes_out(const S *__restrict__ A, const int64_t stride, const int q,
                                const int32_t *__restrict__ map, const int nf, const int64_t n1,
                                double *__restrict__ stage, float scale) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1) return;
    const int32_t m = map[t];
    if (m >= nf) stage[t] = Store<S>::ld64(A + (int64_t)q * stride, m, WREST(q), 1.0f / scale);
}

// the equilibrium at rest of every link slot, from phi at its solid cell: k_init_eq's
// expression for that cell and direction
template <class S>
__global__ void k_mp_init_links(S *__restrict__ f, S *__restrict__ g, const typename Store<S>::R *__restrict__ phi,
                                const int64_t stride, const int32_t *__restrict__ link, const int64_t nlink,
                                const Layout L) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlink) return;
    const int q = link[3 * l];
    const int64_t slot = link[3 * l + 1], h = link[3 * l + 2];
    const int k = (int)(h / L.h1xy);
    const int64_t r = h - (int64_t)k * L.h1xy;
    const int j = (int)(r / L.h1x), i = (int)(r - (int64_t)j * L.h1x);
    const double ph = (double)phi[L.i4(i, j, k)];
    const double r0 = 1.0 * (1.0 + ph) * 0.5, r1 = 1.0 * (1.0 - ph) * 0.5;
    const double usqrt = 0.0, cu = 0.0, wq = WEQ(q);
    const double a = q == 0 ? r0 * wq + r0 * wq * (-1.5 * usqrt) : r0 * wq + r0 * wq * (3.0 * cu + 4.5 * cu * cu - 1.5 * usqrt);
    const double b = q == 0 ? r1 * wq + r1 * wq * (-1.5 * usqrt) : r1 * wq + r1 * wq * (3.0 * cu + 4.5 * cu * cu - 1.5 * usqrt);
    Store<S>::st64(f, (int64_t)q * stride + slot, a, WREST(q), 1.0f);
    Store<S>::st64(g, (int64_t)q * stride + slot, b, WREST(q), 1.0f);
}

// the y-face exchange of the porous-plate planes' private ghosts (the dense k_wrap_faces for
// dim 1 over those planes): one thread per (i, k) entry {ghost 0, image ny, ghost ny+1,
// image 1} and species; pull after an even step (ghosts from images), push after an odd
// step (images from the ghosts the odd step wrote)
template <class S>
__global__ void k_mp_wrap_ghosts(S *__restrict__ f, S *__restrict__ g, const int64_t stride,
                                 const int32_t *__restrict__ wrap, const int64_t nwrap, int pull) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nwrap) return;
    S *A = t < nwrap ? f : g;
    const int64_t e = t < nwrap ? t : t - nwrap;
    const int64_t g0 = wrap[4 * e], in_n = wrap[4 * e + 1], g1 = wrap[4 * e + 2], in_1 = wrap[4 * e + 3];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const int64_t qp = (int64_t)c_plus[1][m] * stride, qm = (int64_t)c_minus[1][m] * stride;
        if (pull) {
            A[qp + g0] = A[qp + in_n];
            A[qm + g1] = A[qm + in_1];
        } else {
            A[qm + in_1] = A[qm + g1];
            A[qp + in_n] = A[qp + g0];
        }
    }
}

static __global__ void k_list_ghosts(double *__restrict__ stage, const Layout L, int px, int py, int pz) {
    const int64_t n = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i = (int)(t % (L.nx + 2)), j = (int)((t / (L.nx + 2)) % (L.ny + 2)), k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    const bool gx = i == 0 || i == L.nx + 1, gy = j == 0 || j == L.ny + 1, gz = k == 0 || k == L.nz + 1;
    if (!(gx || gy || gz)) return;
    if ((gx && !px) || (gy && !py) || (gz && !pz)) return;
    if (gx) i = i == 0 ? L.nx : 1;
    if (gy) j = j == 0 ? L.ny : 1;
    if (gz) k = k == 0 ? L.nz : 1;
    stage[t] = stage[L.i1(i, j, k)];
}

// compute_macro_vars + monitor reductions over the fluid list (singlephase): one block
// per segment [seg0[b], seg1[b]) of fluid indices (a z slice of one sample, or a whole
// sample of an ensemble).  out[m * nseg + b]: m = 0 sum w, 6 sum rho, 7 max |u|^2
// (the rows of the dense k_monitor).  Fields u, v, w, rho are scattered to the halo-1
// arrays when write_fields (solid cells keep the zeros written before).
template <class S>
__global__ void __launch_bounds__(MON_THREADS) k_list_monitor(const S *__restrict__ A, const int64_t stride,
                                                              const int32_t *__restrict__ seg0,
                                                              const int32_t *__restrict__ seg1, const int nseg,
                                                              const int32_t *__restrict__ cell1, double *__restrict__ u,
                                                              double *__restrict__ v, double *__restrict__ w,
                                                              double *__restrict__ rho, double *__restrict__ out,
                                                              const StepParams P, int write_fields, float scale) {
    using St = Store<S>;
    using R = typename St::R;
    const int b = blockIdx.x;
    const int x0 = seg0[b], x1 = seg1[b];
    const R inv = R(1.0f / scale);
    double sw = 0.0, sr = 0.0, um = 0.0;
    for (int x = x0 + (int)threadIdx.x; x < x1; x += MON_THREADS) {
        double ft[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) ft[q] = St::ld64(A, (int64_t)q * stride + x, WREST(q), 1.0f / scale);
        const double rr = ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] + ft[11] +
                          ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
        const double uu = ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] - 0.5 * 0.0;
        const double vv = ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] - 0.5 * 0.0;
        const double ww = ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] - 0.5 * P.force_z;
        if (write_fields) {
            const int32_t c = cell1[x];
            u[c] = uu; v[c] = vv; w[c] = ww; rho[c] = rr;
        }
        const double temp = uu * uu + vv * vv + ww * ww;
        um = (um < temp) ? temp : um;
        sw += ww;
        sr += rr;
    }
    __shared__ double red[3][MON_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        sw += __shfl_down_sync(0xffffffffu, sw, o);
        sr += __shfl_down_sync(0xffffffffu, sr, o);
        const double y = __shfl_down_sync(0xffffffffu, um, o);
        um = (um < y) ? y : um;
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = sw; red[1][threadIdx.x >> 5] = sr; red[2][threadIdx.x >> 5] = um;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, r = 0.0, m = 0.0;
        for (int q = 0; q < MON_THREADS / 32; ++q) {
            a += red[0][q];
            r += red[1][q];
            m = (m < red[2][q]) ? red[2][q] : m;
        }
        out[b] = a;
        out[(int64_t)6 * nseg + b] = r;
        out[(int64_t)7 * nseg + b] = m;
    }
}

// ---------------------------------------------------------------------------------
// Singlephase state from density and velocity fields (warm start): every fluid slot gets
//   f_q = rho (base_q + w_q (3 e.u + 4.5 (e.u)^2 - 1.5 u^2))
// with base_q = w_q (the reference's equilibrium) or the MRT rest state W_q
// (rest_base = 1), rho and u from the halo-1 arrays (rho NULL: 1).  A solid slot that a
// fluid node pushes into (bounce-back link: slot q of solid s, pushed by the fluid node
// s + e_q in direction opp(q)) gets that node's f_opp(q), the value it holds in a settled
// flow; every other solid slot gets base_q.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double feq_vel(int q, double rho, double ux, double uy, double uz, int rest_base) {
    const double wq = WEQ(q);
    const double cu = (double)c_ex[q] * ux + (double)c_ey[q] * uy + (double)c_ez[q] * uz;
    const double usq = ux * ux + uy * uy + uz * uz;
    const double base = rest_base ? WREST(q) : wq;
    return rho * (base + wq * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq));
}

template <class S>
__global__ void k_init_vel_dense(S *__restrict__ f, const double *__restrict__ rho, const double *__restrict__ u,
                                 const double *__restrict__ v, const double *__restrict__ w,
                                 const int8_t *__restrict__ walls, const Layout L, int rest_base, float scale) {
    using St = Store<S>;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb) return;
    const int i = (int)(t % (L.nx + 2));
    const int j = (int)((t / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    const int64_t c = L.cell(i, j, k);
    if (walls[L.i2(i, j, k)] == 0) {
        const double r = rho ? rho[t] : 1.0;
        for (int q = 0; q < 19; ++q)
            St::st64(f, (int64_t)q * L.qs + c, feq_vel(q, r, u[t], v[t], w[t], rest_base), WREST(q), scale);
        return;
    }
    for (int q = 0; q < 19; ++q) {
        double val = rest_base ? WREST(q) : WEQ(q);
        const int ni = i + c_ex[q], nj = j + c_ey[q], nk = k + c_ez[q];
        if (q > 0 && ni >= 0 && ni <= L.nx + 1 && nj >= 0 && nj <= L.ny + 1 && nk >= 0 && nk <= L.nz + 1 &&
            walls[L.i2(ni, nj, nk)] == 0) {
            const int64_t m = L.i1(ni, nj, nk);
            val = feq_vel(OPP_RT(q), rho ? rho[m] : 1.0, u[m], v[m], w[m], rest_base);
        }
        St::st64(f, (int64_t)q * L.qs + c, val, WREST(q), scale);
    }
}

// list layout, pass 1: every slot of every direction array (fluid nodes from their cell,
// links and padding base_q)
template <class S>
__global__ void k_init_vel_list(S *__restrict__ A, const int64_t stride, const int32_t *__restrict__ cell1, const int nf,
                                const double *__restrict__ rho, const double *__restrict__ u,
                                const double *__restrict__ v, const double *__restrict__ w, int rest_base, float scale) {
    using St = Store<S>;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= stride) return;
    double r = 1.0, ux = 0.0, uy = 0.0, uz = 0.0;
    if (t < nf) {
        const int32_t c = cell1[t];
        r = rho ? rho[c] : 1.0;
        ux = u[c]; uy = v[c]; uz = w[c];
        for (int q = 0; q < 19; ++q) St::st64(A, (int64_t)q * stride + t, feq_vel(q, r, ux, uy, uz, rest_base), WREST(q), scale);
    } else {
        for (int q = 0; q < 19; ++q) St::st64(A, (int64_t)q * stride + t, rest_base ? WREST(q) : WEQ(q), WREST(q), scale);
    }
}

// list layout, pass 2: the link slots a fluid node pushes into (nb[d][x] >= nf holds
// that node's f_d in array opp(d))
template <class S>
__global__ void k_init_vel_links(S *__restrict__ A, const int64_t stride, const int32_t *__restrict__ nb,
                                 const int32_t *__restrict__ cell1, const int nf, const double *__restrict__ rho,
                                 const double *__restrict__ u, const double *__restrict__ v,
                                 const double *__restrict__ w, int rest_base, float scale) {
    using St = Store<S>;
    const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nf) return;
    const int32_t c = cell1[x];
    const double r = rho ? rho[c] : 1.0;
    for (int d = 1; d < 19; ++d) {
        const int32_t slot = nb[(int64_t)(d - 1) * nf + x];
        if (slot >= nf)
            St::st64(A, (int64_t)OPP_RT(d) * stride + slot, feq_vel(d, r, u[c], v[c], w[c], rest_base), WREST(d), scale);
    }
}

// list layout with boundary-plane slots, pass 3: every cell that owns a plane slot, as
// k_init_vel_dense writes that cell (after pass 2, which also reaches plane slots through
// the neighbour table)
template <class S>
__global__ void k_init_vel_planes(S *__restrict__ A, const PdfAt pa, const int nf, const double *__restrict__ rho,
                                  const double *__restrict__ u, const double *__restrict__ v,
                                  const double *__restrict__ w, const int8_t *__restrict__ walls, const Layout L,
                                  int rest_base, float scale) {
    using St = Store<S>;
    const int64_t n1 = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1) return;
    const int32_t m = pa.map[t];
    if (m < nf) return;   // a fluid node, a periodic ghost or a cell without a slot
    const int i = (int)(t % (L.nx + 2));
    const int j = (int)((t / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(t / ((int64_t)(L.nx + 2) * (L.ny + 2)));
    if (walls[L.i2(i, j, k)] == 0) {
        const double r = rho ? rho[t] : 1.0;
        for (int q = 0; q < 19; ++q)
            St::st64(A, (int64_t)q * pa.qs + m, feq_vel(q, r, u[t], v[t], w[t], rest_base), WREST(q), scale);
        return;
    }
    for (int q = 0; q < 19; ++q) {
        double val = rest_base ? WREST(q) : WEQ(q);
        const int ni = i + c_ex[q], nj = j + c_ey[q], nk = k + c_ez[q];
        if (q > 0 && ni >= 0 && ni <= L.nx + 1 && nj >= 0 && nj <= L.ny + 1 && nk >= 0 && nk <= L.nz + 1 &&
            walls[L.i2(ni, nj, nk)] == 0) {
            const int64_t mm = L.i1(ni, nj, nk);
            val = feq_vel(OPP_RT(q), rho ? rho[mm] : 1.0, u[mm], v[mm], w[mm], rest_base);
        }
        St::st64(A, (int64_t)q * pa.qs + m, val, WREST(q), scale);
    }
}

// ---------------------------------------------------------------------------------
// Steady-state and breakthrough monitors of the multiphase model
// (multiphase_3D/0.src/Monitor.F90:287-507); one block per z slice, partials
// out[m * nz + k - 1]: m = 0 max |phi - phi_old|, 1 max |u|^2, 2 sum rho (phi < -0.99),
// 3 count (phi < -0.99), 4 sum rho (phi > 0.99), 5 count (phi > 0.99), 6 count of fluid
// nodes with phi > 0 (only slice obs_z).  Fluid nodes only; u, v, w, rho from
// compute_macro_vars.  copy_old: phi_old <- phi afterwards (interior).
// ---------------------------------------------------------------------------------
constexpr int STEADY_NQ = 7;

template <class T>
__global__ void __launch_bounds__(MON_THREADS) k_steady(const T *__restrict__ phi, T *__restrict__ phi_old,
                                                        const double *__restrict__ rho, const double *__restrict__ u,
                                                        const double *__restrict__ v, const double *__restrict__ w,
                                                        const int8_t *__restrict__ walls, double *__restrict__ out,
                                                        const Layout L, int obs_z, int copy_old) {
    const int k = blockIdx.x + 1;
    const int64_t n = (int64_t)L.nx * L.ny;
    double acc[STEADY_NQ];
#pragma unroll
    for (int m = 0; m < STEADY_NQ; ++m) acc[m] = 0.0;
    for (int64_t t = threadIdx.x; t < n; t += MON_THREADS) {
        const int i = (int)(t % L.nx) + 1, j = (int)(t / L.nx) + 1;
        const int wi = walls[L.i2(i, j, k)];
        const int64_t i4 = L.i4(i, j, k), i1 = L.i1(i, j, k);
        const double ph = (double)phi[i4];
        if (wi == 0) {
            if (phi_old) {
                const double d = fabs(ph - (double)phi_old[i4]);
                acc[0] = acc[0] < d ? d : acc[0];
            }
            const double uu = u[i1] * u[i1] + v[i1] * v[i1] + w[i1] * w[i1];
            acc[1] = acc[1] < uu ? uu : acc[1];
            if (ph < -0.99) { acc[2] += rho[i1]; acc[3] += 1.0; }
            if (ph > 0.99) { acc[4] += rho[i1]; acc[5] += 1.0; }
            if (k == obs_z && ph > 0.0) acc[6] += 1.0;
        }
        if (copy_old && phi_old) phi_old[i4] = phi[i4];
    }
    __shared__ double red[MON_THREADS / 32][STEADY_NQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int m = 0; m < STEADY_NQ; ++m) {
        double x = acc[m];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = m <= 1 ? ((x < y) ? y : x) : x + y;
        }
        if (lane == 0) red[wid][m] = x;
    }
    __syncthreads();
    if (threadIdx.x < STEADY_NQ) {
        const int m = threadIdx.x;
        double x = red[0][m];
        for (int q = 1; q < MON_THREADS / 32; ++q) x = m <= 1 ? ((x < red[q][m]) ? red[q][m] : x) : x + red[q][m];
        out[(int64_t)m * L.nz + (k - 1)] = x;
    }
}

// change_inlet_fluid_phase (multiphase_3D/0.src/Misc.F90:507-621): in every slot of the
// halo-1 box with k <= kmax (z <= interface_z0 on one rank) one species takes the sum of
// both populations and the other is emptied; to_f = 1 (cmd 1): f <- f + g, g <- 0;
// to_f = 0 (cmd 2): g <- f + g, f <- 0.  One thread per (q, cell).
template <class T>
__global__ void k_change_inlet_phase(T *__restrict__ f, T *__restrict__ g, const Layout L, const PdfAt pa, int kmax,
                                     int to_f) {
    const int64_t nrow = L.nx + 2, nplane = nrow * (L.ny + 2), ncell = nplane * (kmax + 1);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 19 * ncell) return;
    const int q = (int)(t / ncell);
    const int64_t r = t - q * ncell;
    const int k = (int)(r / nplane);
    const int64_t r2 = r - k * nplane;
    const int j = (int)(r2 / nrow), i = (int)(r2 - j * nrow);
    if (!pa.owned(L, i, j, k)) return;   // fluid list: link slots are updated from the link table
    const int64_t id = pa(L, q, i, j, k);
    if constexpr (std::is_same<T, ffs>::value) {
        // double-word storage: join both to FP64, add, split
        const double a = Store<ffs>::ld(f, id, 0.0, 0.0), b = Store<ffs>::ld(g, id, 0.0, 0.0);
        Store<ffs>::st(to_f ? f : g, id, a + b, 0.0, 0.0);
        Store<ffs>::st(to_f ? g : f, id, 0.0, 0.0, 0.0);
    } else {
        const T a = f[id], b = g[id];
        if (to_f) {
            f[id] = a + b;
            g[id] = T(0);
        } else {
            g[id] = a + b;
            f[id] = T(0);
        }
    }
}

// the same for the link slots of the multiphase fluid list whose solid cell has k <= kmax
template <class T>
__global__ void k_change_inlet_links(T *__restrict__ f, T *__restrict__ g, const int64_t stride,
                                     const int32_t *__restrict__ link, const int64_t nlink, const Layout L, int kmax,
                                     int to_f) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlink) return;
    const int k = (int)(link[3 * l + 2] / L.h1xy);
    if (k > kmax) return;
    const int64_t id = (int64_t)link[3 * l] * stride + link[3 * l + 1];
    if constexpr (std::is_same<T, ffs>::value) {
        const double a = Store<ffs>::ld(f, id, 0.0, 0.0), b = Store<ffs>::ld(g, id, 0.0, 0.0);
        Store<ffs>::st(to_f ? f : g, id, a + b, 0.0, 0.0);
        Store<ffs>::st(to_f ? g : f, id, 0.0, 0.0, 0.0);
    } else {
        const T a = f[id], b = g[id];
        if (to_f) {
            f[id] = a + b;
            g[id] = T(0);
        } else {
            g[id] = a + b;
            f[id] = T(0);
        }
    }
}

// FP64 host image <-> field array of type T (phi, gradient fields of the mixed form)
template <class T>
__global__ void k_field_in(T *__restrict__ dst, const double *__restrict__ src, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (T)src[t];
}

template <class T>
__global__ void k_field_out(double *__restrict__ dst, const T *__restrict__ src, int64_t n, int stride) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (double)src[t * stride];
}

}  // namespace MFLBM_NS
}  // namespace mflbm
