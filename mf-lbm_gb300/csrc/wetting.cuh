// wetting.cuh -- the per-node step of the geometric wetting (the colour gradient replaced
// at fluid-boundary nodes).  Included by kernels.cuh inside the kernel flavour's namespace
// (each flavour compiles it with its own contraction rule) and by the host tests; it
// includes nothing itself.
#pragma once

// geometric wetting at a fluid-boundary node (alter_color_gradient_solid_surface,
// Phase_gradient.F90:210-265): the phase normal n (in/out) replaced by the candidate at
// contact angle theta to the wall normal nw that lies closer to n.
// The reference writes the two candidates as (cos - s t/sqrt(1-t^2)) nw + (s/sqrt(1-t^2)) n
// with t = nw.n, i.e. cos nw +- s (n - t nw)/sqrt(1 - t^2): for a unit n, sqrt(1 - t^2) is the
// length of the perpendicular part n - t nw.  Where the phase normal is nearly parallel to
// the wall normal, that length is tiny and the formula divides any departure of |n| from 1
// by it: FP64-normalised normals rarely meet it, but FP32 or double-word normals (unit to
// 1e-7 / 1e-14) gave |n| of 1.01-1.05 at such nodes, which grew into NaN on large packings.
// With min_one_m > 0 (FP32: 1e-6, double-word form: 1e-12) the perpendicular part is
// normalised by its own length, bounded below by sqrt(min_one_m): the same formula for a
// unit n, with a unit result while the perpendicular part is longer than the bound and a
// result of length between cos(theta) and 1 below it (no division by a vanishing length);
// min_one_m = 0 keeps the reference's expression (FP64 drop-in).
template <class T>
__host__ __device__ __forceinline__ void wetting_normal(T (&n)[3], const T nwx, const T nwy, const T nwz,
                                                       const T tmpCos, const T sin_t, const T min_one_m) {
    const T cnx0 = n[0], cny0 = n[1], cnz0 = n[2];
    const T tmp1 = nwx * cnx0 + nwy * cny0 + nwz * cnz0;
    T cnxp, cnyp, cnzp, cnxm, cnym, cnzm;
    if (min_one_m > T(0.0)) {
        // cos nw +- sin (n - t nw) / |n - t nw|
        const T px = cnx0 - tmp1 * nwx, py = cny0 - tmp1 * nwy, pz = cnz0 - tmp1 * nwz;
        T pp = px * px + py * py + pz * pz;
        if (pp < min_one_m) pp = min_one_m;
        const T coe2 = sin_t / sqrt(pp);
        cnxp = tmpCos * nwx + coe2 * px; cnyp = tmpCos * nwy + coe2 * py; cnzp = tmpCos * nwz + coe2 * pz;
        cnxm = tmpCos * nwx - coe2 * px; cnym = tmpCos * nwy - coe2 * py; cnzm = tmpCos * nwz - coe2 * pz;
    } else {
        const T tmp2 = T(1.0) / sqrt(T(1.0) - tmp1 * tmp1);
        const T coe1 = sin_t * tmp1 * tmp2;
        const T coe2 = sin_t * tmp2;
        cnxp = (tmpCos - coe1) * nwx + coe2 * cnx0;
        cnyp = (tmpCos - coe1) * nwy + coe2 * cny0;
        cnzp = (tmpCos - coe1) * nwz + coe2 * cnz0;
        cnxm = (tmpCos + coe1) * nwx - coe2 * cnx0;
        cnym = (tmpCos + coe1) * nwy - coe2 * cny0;
        cnzm = (tmpCos + coe1) * nwz - coe2 * cnz0;
    }
    const T distP = (cnxp - cnx0) * (cnxp - cnx0) + (cnyp - cny0) * (cnyp - cny0) + (cnzp - cnz0) * (cnzp - cnz0);
    const T distM = (cnxm - cnx0) * (cnxm - cnx0) + (cnym - cny0) * (cnym - cny0) + (cnzm - cnz0) * (cnzm - cnz0);
    if (distP <= distM) {
        n[0] = cnxp; n[1] = cnyp; n[2] = cnzp;
    } else {
        n[0] = cnxm; n[1] = cnym; n[2] = cnzm;
    }
}
