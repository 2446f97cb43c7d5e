// collide.cuh -- the pair form of the MRT collision (any arithmetic type R) and its
// double-word form.  Included by kernels.cuh inside the kernel flavour's namespace (so each
// flavour compiles it with its own contraction rule) and by the host tests of the
// double-word arithmetic; it needs MrtFold (common.cuh) and the ff operations (ffloat.cuh)
// in scope and includes nothing itself.
#pragma once

// ---------------------------------------------------------------------------------
// The same MRT collision re-associated for fewer FP64 instructions (default build).
//
// Opposite directions form 9 pairs (q, q').  Every even-order moment of the D3Q19 basis
// (rho, e, e2, 3pxx, 3pixx, pww, piww, pxy, pyz, pzx) depends only on f0 and the pair
// sums p = f_q + f_q'; every odd-order moment (j, q, t) only on the pair differences
// d = f_q - f_q'.  The back-transform likewise yields a symmetric part S and an
// antisymmetric part A per pair, f_q = S + A, f_q' = S - A.  Relaxation, equilibrium,
// forcing and the back-transform norms (1/19, 1/2394, ...) are folded into one
// coefficient set (MrtFold).  Mathematically this is the reference's collision
// (Kernel_multiphase.F90:158-267) with mrt_e2_coef1 = mrt_omega_xx = 0 substituted.
// ---------------------------------------------------------------------------------
// FXY = false: the force has only a z component (singlephase body force).
// OWN_DEN = true: the density is the sum of the 19 PDFs (singlephase); otherwise the
// caller supplies it (rho1 + rho2 of the colour model).
// UNIT = true: s_e = s_e2 = s_pi = s_nu = 1 (tau = 1 with MRT preset 1), so the
// coefficients of the non-conserved even-order moments (e_m, e2_m, x3_m, xi_m, w_m, wi_m,
// o_m) are zero and those moments are not formed.
template <class R, bool FXY, bool OWN_DEN, bool UNIT = false>
__device__ __forceinline__ void mrt_collide_pairs(R (&ft)[19], R den_in, R fx, R fy, R fz, const MrtFold<R> &c) {
    const R f0 = ft[0];
    const R p1 = ft[1] + ft[2], d1 = ft[1] - ft[2];
    const R p2 = ft[3] + ft[4], d2 = ft[3] - ft[4];
    const R p3 = ft[5] + ft[6], d3 = ft[5] - ft[6];
    const R p4 = ft[7] + ft[10], d4 = ft[7] - ft[10];
    const R p5 = ft[8] + ft[9], d5 = ft[8] - ft[9];
    const R p6 = ft[11] + ft[14], d6 = ft[11] - ft[14];
    const R p7 = ft[12] + ft[13], d7 = ft[12] - ft[13];
    const R p8 = ft[15] + ft[18], d8 = ft[15] - ft[18];
    const R p9 = ft[16] + ft[17], d9 = ft[16] - ft[17];
    // momentum; velocity with the half-step force
    const R jx = d1 + d4 - d5 + d6 - d7;
    const R jy = d2 + d4 + d5 + d8 - d9;
    const R jz = d3 + d6 + d7 + d8 + d9;
    const R ux = FXY ? jx + R(0.5) * fx : jx;
    const R uy = FXY ? jy + R(0.5) * fy : jy;
    const R uz = jz + R(0.5) * fz;
    const R uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
    const R u2 = uxx + uyy + uzz;
    const R fux = FXY ? fx * ux : R(0.0);
    const R fuy = FXY ? fy * uy : R(0.0);
    const R fuz = fz * uz;
    const R Fu = FXY ? fux + fuy + fuz : fuz;
    // even-order moments from the pair sums
    const R a = p1 + p2 + p3;
    const R dxy = p4 + p5, dxz = p6 + p7, dyz = p8 + p9;
    const R ds = dxy + dxz + dyz;
    const R den = OWN_DEN ? f0 + a + ds : den_in;
    const R m_e = UNIT ? R(0.0) : R(-30.0) * f0 - R(11.0) * a + R(8.0) * ds;
    const R m_e2 = UNIT ? R(0.0) : R(12.0) * f0 - R(4.0) * a + ds;
    const R s6 = UNIT ? R(0.0) : R(2.0) * p1 - p2 - p3;
    const R s7 = UNIT ? R(0.0) : dxy + dxz - R(2.0) * dyz;
    const R s8 = UNIT ? R(0.0) : p2 - p3, s9 = UNIT ? R(0.0) : dxy - dxz;
    // odd-order non-conserved moments from the pair differences
    const R qx = jx - R(5.0) * d1, qy = jy - R(5.0) * d2, qz = jz - R(5.0) * d3;
    const R tx = d4 - d5 - d6 + d7;
    const R ty = -d4 - d5 + d8 - d9;
    const R tz = d6 + d7 - d8 - d9;
    // relaxed, forced and scaled moments
    const R rho_s = den * R(1.0 / 19.0);
    const R e_s = UNIT ? c.e_den * den + c.e_u2 * u2 + c.e_f * Fu : c.e_m * m_e + c.e_den * den + c.e_u2 * u2 + c.e_f * Fu;
    const R e2_s = UNIT ? c.e2_u2 * u2 + c.e2_f * Fu : c.e2_m * m_e2 + c.e2_u2 * u2 + c.e2_f * Fu;
    const R jx_s = R(0.1) * (FXY ? jx + fx : jx);
    const R jy_s = R(0.1) * (FXY ? jy + fy : jy);
    const R jz_s = R(0.1) * (jz + fz);
    const R qx_s = FXY ? c.q_m * qx + c.q_u * ux + c.q_f * fx : c.q_m * qx + c.q_u * ux;
    const R qy_s = FXY ? c.q_m * qy + c.q_u * uy + c.q_f * fy : c.q_m * qy + c.q_u * uy;
    const R qz_s = c.q_m * qz + c.q_u * uz + c.q_f * fz;
    const R x3_s = (UNIT ? R(0.0) : c.x3_m * (s6 + s7)) + c.x3_eq * (R(3.0) * uxx - u2) + c.x3_f * (R(2.0) * fux - fuy - fuz);
    const R xi_s = (UNIT ? R(0.0) : c.xi_m * (R(-2.0) * s6 + s7)) + c.xi_f * (R(-2.0) * fux + fuy + fuz);
    const R w_s = (UNIT ? R(0.0) : c.w_m * (s8 + s9)) + c.w_eq * (uyy - uzz) + c.w_f * (fuy - fuz);
    const R wi_s = (UNIT ? R(0.0) : c.wi_m * (R(-2.0) * s8 + s9)) + c.wi_f * (fuz - fuy);
    const R om_xy = UNIT ? R(0.0) : c.o_m * (p4 - p5);
    const R om_yz = UNIT ? R(0.0) : c.o_m * (p8 - p9);
    const R om_zx = UNIT ? R(0.0) : c.o_m * (p6 - p7);
    const R xy_s = FXY ? om_xy + c.o_eq * (ux * uy) + c.o_f * (fx * uy + fy * ux) : om_xy + c.o_eq * (ux * uy);
    const R yz_s = FXY ? om_yz + c.o_eq * (uy * uz) + c.o_f * (fy * uz + fz * uy) : om_yz + c.o_eq * (uy * uz) + c.o_f * (fz * uy);
    const R zx_s = FXY ? om_zx + c.o_eq * (ux * uz) + c.o_f * (fx * uz + fz * ux) : om_zx + c.o_eq * (ux * uz) + c.o_f * (fz * ux);
    const R tx_s = c.t_m * tx, ty_s = c.t_m * ty, tz_s = c.t_m * tz;
    // back-transform
    const R sum1 = rho_s - R(11.0) * e_s - R(4.0) * e2_s;
    const R sum2 = R(2.0) * x3_s - R(4.0) * xi_s;
    const R sum3 = w_s - R(2.0) * wi_s;
    const R sum4 = rho_s + R(8.0) * e_s + e2_s;
    const R sum5 = jx_s + qx_s, sum6 = jy_s + qy_s, sum7 = jz_s + qz_s;
    const R sum8 = x3_s + xi_s, sum9 = w_s + wi_s;
    ft[0] = rho_s - R(30.0) * e_s + R(12.0) * e2_s;
    {
        const R S = sum1 + sum2, A = jx_s - R(4.0) * qx_s;
        ft[1] = S + A;
        ft[2] = S - A;
    }
    {
        const R Syz = sum1 - R(0.5) * sum2;
        const R Sy = Syz + sum3, Ay = jy_s - R(4.0) * qy_s;
        const R Sz = Syz - sum3, Az = jz_s - R(4.0) * qz_s;
        ft[3] = Sy + Ay;
        ft[4] = Sy - Ay;
        ft[5] = Sz + Az;
        ft[6] = Sz - Az;
    }
    {
        const R b = sum4 + sum8 + sum9;
        const R Sp = b + xy_s, Ap = sum5 + sum6 + tx_s - ty_s;
        const R Sm = b - xy_s, Am = sum6 - sum5 - tx_s - ty_s;
        ft[7] = Sp + Ap;
        ft[10] = Sp - Ap;
        ft[8] = Sm + Am;
        ft[9] = Sm - Am;
    }
    {
        const R b = sum4 + sum8 - sum9;
        const R Sp = b + zx_s, Ap = sum5 + sum7 - tx_s + tz_s;
        const R Sm = b - zx_s, Am = sum7 - sum5 + tx_s + tz_s;
        ft[11] = Sp + Ap;
        ft[14] = Sp - Ap;
        ft[12] = Sm + Am;
        ft[13] = Sm - Am;
    }
    {
        const R b = sum4 - R(2.0) * sum8;
        const R Sp = b + yz_s, Ap = sum6 + sum7 + ty_s - tz_s;
        const R Sm = b - yz_s, Am = sum7 - sum6 - ty_s - tz_s;
        ft[15] = Sp + Ap;
        ft[18] = Sp - Ap;
        ft[16] = Sm + Am;
        ft[17] = Sm - Am;
    }
}

// ---------------------------------------------------------------------------------
// The same singlephase collision (mrt_collide_pairs with FXY = false, OWN_DEN = true) in
// double-word arithmetic (ffloat.cuh) for FP64 storage: every sum, difference and product
// of the FP64 form, with multiplications by small integers as FP32-factor products and by
// powers of two exactly.  With the force along z only, the forcing combinations of the
// FP64 form reduce to +-F_z u_z (2 fux - fuy - fuz = -fuz, -2 fux + fuy + fuz = fuz,
// fuy - fuz = -fuz, fuz - fuy = fuz).
// ---------------------------------------------------------------------------------
template <bool UNIT>
__device__ __forceinline__ void mrt_collide_ff(ff (&ft)[19], const MrtFold<ff> &c) {
    const ff f0 = ft[0];
    const ff p1 = ft[1] + ft[2], d1 = ft[1] - ft[2];
    const ff p2 = ft[3] + ft[4], d2 = ft[3] - ft[4];
    const ff p3 = ft[5] + ft[6], d3 = ft[5] - ft[6];
    const ff p4 = ft[7] + ft[10], d4 = ft[7] - ft[10];
    const ff p5 = ft[8] + ft[9], d5 = ft[8] - ft[9];
    const ff p6 = ft[11] + ft[14], d6 = ft[11] - ft[14];
    const ff p7 = ft[12] + ft[13], d7 = ft[12] - ft[13];
    const ff p8 = ft[15] + ft[18], d8 = ft[15] - ft[18];
    const ff p9 = ft[16] + ft[17], d9 = ft[16] - ft[17];
    const ff jx = d1 + d4 - d5 + d6 - d7;
    const ff jy = d2 + d4 + d5 + d8 - d9;
    const ff jz = d3 + d6 + d7 + d8 + d9;
    const ff &ux = jx, &uy = jy;
    const ff uz = jz + ff_pow2(c.fz, 0.5f);
    const ff uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
    const ff u2 = uxx + uyy + uzz;
    const ff fuz = c.fz * uz;
    const ff a = p1 + p2 + p3;
    const ff dxy = p4 + p5, dxz = p6 + p7, dyz = p8 + p9;
    const ff ds = dxy + dxz + dyz;
    const ff den = f0 + a + ds;
    const ff qx = jx - ff_mulf(d1, 5.0f), qy = jy - ff_mulf(d2, 5.0f), qz = jz - ff_mulf(d3, 5.0f);
    const ff tx = d4 - d5 - d6 + d7;
    const ff ty = d8 - d4 - d5 - d9;
    const ff tz = d6 + d7 - d8 - d9;
    constexpr ff k19 = ff_const(1.0 / 19.0), k01 = ff_const(0.1);
    const ff rho_s = den * k19;
    ff e_s = c.e_den * den + c.e_u2 * u2 + c.e_f * fuz;
    ff e2_s = c.e2_u2 * u2 + c.e2_f * fuz;
    const ff jx_s = jx * k01, jy_s = jy * k01, jz_s = (jz + c.fz) * k01;
    const ff qx_s = c.q_m * qx + c.q_u * ux;
    const ff qy_s = c.q_m * qy + c.q_u * uy;
    const ff qz_s = c.q_m * qz + c.q_u * uz + c.q_f * c.fz;
    ff x3_s = c.x3_eq * (ff_mulf(uxx, 3.0f) - u2) - c.x3_f * fuz;
    ff xi_s = c.xi_f * fuz;
    ff w_s = c.w_eq * (uyy - uzz) - c.w_f * fuz;
    ff wi_s = c.wi_f * fuz;
    ff xy_s = c.o_eq * (ux * uy);
    ff yz_s = c.o_eq * (uy * uz) + c.o_f * (c.fz * uy);
    ff zx_s = c.o_eq * (ux * uz) + c.o_f * (c.fz * ux);
    if constexpr (!UNIT) {
        const ff m_e = ff_mulf(f0, -30.0f) - ff_mulf(a, 11.0f) + ff_pow2(ds, 8.0f);
        const ff m_e2 = ff_mulf(f0, 12.0f) - ff_pow2(a, 4.0f) + ds;
        const ff s6 = ff_pow2(p1, 2.0f) - p2 - p3;
        const ff s7 = dxy + dxz - ff_pow2(dyz, 2.0f);
        const ff s8 = p2 - p3, s9 = dxy - dxz;
        e_s = e_s + c.e_m * m_e;
        e2_s = e2_s + c.e2_m * m_e2;
        x3_s = x3_s + c.x3_m * (s6 + s7);
        xi_s = xi_s + c.xi_m * (s7 - ff_pow2(s6, 2.0f));
        w_s = w_s + c.w_m * (s8 + s9);
        wi_s = wi_s + c.wi_m * (s9 - ff_pow2(s8, 2.0f));
        xy_s = xy_s + c.o_m * (p4 - p5);
        yz_s = yz_s + c.o_m * (p8 - p9);
        zx_s = zx_s + c.o_m * (p6 - p7);
    }
    const ff tx_s = c.t_m * tx, ty_s = c.t_m * ty, tz_s = c.t_m * tz;
    // back-transform
    const ff sum1 = rho_s - ff_mulf(e_s, 11.0f) - ff_pow2(e2_s, 4.0f);
    const ff sum2 = ff_pow2(x3_s, 2.0f) - ff_pow2(xi_s, 4.0f);
    const ff sum3 = w_s - ff_pow2(wi_s, 2.0f);
    const ff sum4 = rho_s + ff_pow2(e_s, 8.0f) + e2_s;
    const ff sum5 = jx_s + qx_s, sum6 = jy_s + qy_s, sum7 = jz_s + qz_s;
    const ff sum8 = x3_s + xi_s, sum9 = w_s + wi_s;
    ft[0] = rho_s - ff_mulf(e_s, 30.0f) + ff_mulf(e2_s, 12.0f);
    {
        const ff S = sum1 + sum2, A = jx_s - ff_pow2(qx_s, 4.0f);
        ft[1] = S + A;
        ft[2] = S - A;
    }
    {
        const ff Syz = sum1 - ff_pow2(sum2, 0.5f);
        const ff Sy = Syz + sum3, Ay = jy_s - ff_pow2(qy_s, 4.0f);
        const ff Sz = Syz - sum3, Az = jz_s - ff_pow2(qz_s, 4.0f);
        ft[3] = Sy + Ay;
        ft[4] = Sy - Ay;
        ft[5] = Sz + Az;
        ft[6] = Sz - Az;
    }
    {
        const ff b = sum4 + sum8 + sum9;
        const ff Sp = b + xy_s, Ap = sum5 + sum6 + tx_s - ty_s;
        const ff Sm = b - xy_s, Am = sum6 - sum5 - tx_s - ty_s;
        ft[7] = Sp + Ap;
        ft[10] = Sp - Ap;
        ft[8] = Sm + Am;
        ft[9] = Sm - Am;
    }
    {
        const ff b = sum4 + sum8 - sum9;
        const ff Sp = b + zx_s, Ap = sum5 + sum7 - tx_s + tz_s;
        const ff Sm = b - zx_s, Am = sum7 - sum5 + tx_s + tz_s;
        ft[11] = Sp + Ap;
        ft[14] = Sp - Ap;
        ft[12] = Sm + Am;
        ft[13] = Sm - Am;
    }
    {
        const ff b = sum4 - ff_pow2(sum8, 2.0f);
        const ff Sp = b + yz_s, Ap = sum6 + sum7 + ty_s - tz_s;
        const ff Sm = b - yz_s, Am = sum7 - sum6 - ty_s - tz_s;
        ft[15] = Sp + Ap;
        ft[18] = Sp - Ap;
        ft[16] = Sm + Am;
        ft[17] = Sm - Am;
    }
}

