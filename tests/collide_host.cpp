// Host build of the MRT collision forms (mf-lbm_gb300/csrc/collide.cuh) for the CPU tests:
// the pair form in FP64 and the double-word forms (the singlephase mrt_collide_ff and the
// pair form instantiated with the double-word type, as the multiphase double-word kernel
// uses it), with the folded coefficients of common.cuh.  The CUDA intrinsics of the
// double-word arithmetic come from cuda_host_shim.h.
#include <cuda_runtime.h>

#include "cuda_host_shim.h"

#include "../mf-lbm_gb300/csrc/common.cuh"

namespace mflbm {
namespace hostchk {
#include "../mf-lbm_gb300/csrc/collide.cuh"
}  // namespace hostchk
}  // namespace mflbm

using mflbm::ff;
using mflbm::MrtFold;

static double join(ff x) { return (double)x.hi + (double)x.lo; }

extern "C" {
// singlephase collision of one node: rates as the context derives them from (la_nu1, mrt
// preset 1), body force fz; out64 = FP64 pair form, outff = mrt_collide_ff; unit selects the
// unit-rate specialisation (valid when the rates make the zero coefficients vanish)
void ch_sp(const double *f, double s_e, double s_e2, double s_q, double s_nu, double s_pi, double s_t, double fz,
           int unit, double *out64, double *outff) {
    MrtFold<double> c = mflbm::fold_rates<double>(s_e, s_e2, s_q, s_nu, s_pi, s_t);
    c.fz = fz;
    const MrtFold<ff> cf = mflbm::fold_to_ff(c);
    double a[19];
    ff b[19];
    for (int q = 0; q < 19; ++q) {
        a[q] = f[q];
        b[q] = ff(f[q]);
    }
    if (unit) {
        mflbm::hostchk::mrt_collide_pairs<double, false, true, true>(a, 0.0, 0.0, 0.0, c.fz, c);
        mflbm::hostchk::mrt_collide_ff<true>(b, cf);
    } else {
        mflbm::hostchk::mrt_collide_pairs<double, false, true, false>(a, 0.0, 0.0, 0.0, c.fz, c);
        mflbm::hostchk::mrt_collide_ff<false>(b, cf);
    }
    for (int q = 0; q < 19; ++q) {
        out64[q] = a[q];
        outff[q] = join(b[q]);
    }
}

// multiphase collision of one node with a general force and per-node rates folded at run
// time (fold_rates_dev), MRT preset 1: s_q = s_t = 8 (2 - omega) / (8 - omega)
void ch_mp(const double *f, double den, double fx, double fy, double fz, double omega, double *out64,
           double *outff) {
    const double sq = 8.0 * (2.0 - omega) / (8.0 - omega);
    const MrtFold<double> c = mflbm::fold_rates_dev<double>(omega, omega, sq, omega, omega, sq);
    const ff om(omega);
    const ff sqf = mflbm::ff_mulf(ff(2.0f) - om, 8.0f) / (ff(8.0f) - om);
    const MrtFold<ff> cf = mflbm::fold_rates_dev<ff>(om, om, sqf, om, om, sqf);
    double a[19];
    ff b[19];
    for (int q = 0; q < 19; ++q) {
        a[q] = f[q];
        b[q] = ff(f[q]);
    }
    mflbm::hostchk::mrt_collide_pairs<double, true, false>(a, den, fx, fy, fz, c);
    mflbm::hostchk::mrt_collide_pairs<ff, true, false>(b, ff(den), ff(fx), ff(fy), ff(fz), cf);
    for (int q = 0; q < 19; ++q) {
        out64[q] = a[q];
        outff[q] = join(b[q]);
    }
}
}
