// mflbm_oracle.cpp -- CPU FP64 restatement of MF-LBM's per-time-step lattice update.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300 library
// (libmflbm.so).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// may load it, and only as the checker or the timed CPU baseline -- never as the thing
// measured or shipped.
//
// The reference (lanl/MF-LBM) is Fortran 90 + MPI + OpenACC and cannot be compiled in
// this environment (no Fortran compiler, no MPI).  This file restates, for a single
// rank and in the same operation order, the reference routines listed beside each
// function below.  Array shapes, halos and index maps are the reference's own
// (column-major, i fastest).  Built with -ffp-contract=off it evaluates every
// expression left to right exactly as written in the Fortran, so it is bit-identical
// to any IEEE-754 FP64 implementation that keeps that order (the GPU "strict" build).
//
// Parity unpinned: the reference ships no golden vectors, tests or fixtures (its
// test_suites/ hold only input decks), and it cannot be run here to produce outputs.
// The oracle is therefore pinned only by the restatement itself plus analytic
// known-answer properties that the reference's own decks are built around (rest state,
// mass conservation, Poiseuille duct flow, Laplace drop, static contact angle); see
// tests/test_oracle_*.py and tests/test_kat_oracle.py.
//
// Single-rank semantics of the reference's MPI halo exchange: with one rank and a
// periodic direction the Cartesian communicator sends each halo message to the rank
// itself (multiphase_3D/0.src/Mpi_misc.F90:19-38).  The pack/unpack index maps of
// Mpi.F90 then reduce to the on-node copies in periodic_pull / periodic_push /
// periodic_phi below, applied after the whole kernel has run; this equals the
// reference whenever MPI_async_layers_num >= 4 (the template default is 0,4,4).

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mflbm.h"

namespace {

// D3Q19 lattice (multiphase_3D/0.src/Module.F90:111-114)
const int ex[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int ez[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

// MRT constants (Module.F90:116-122)
const double mrt_coef1 = 1.0 / 19.0;
const double mrt_coef2 = 1.0 / 2394.0;
const double mrt_coef3 = 1.0 / 252.0;
const double mrt_coef4 = 1.0 / 72.0;
const double mrt_e2_coef1 = 0.0;
const double mrt_e2_coef2 = -475.0 / 63.0;
const double mrt_omega_xx = 0.0;
// weights (Module.F90:127-131)
const double w_equ_0 = 1.0 / 3.0;
const double w_equ_1 = 1.0 / 18.0;
const double w_equ_2 = 1.0 / 36.0;
const double w_equ[19] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                          1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                          1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
// R-K recolouring weight and ISO4 gradient weights (Module.F90:225-227)
const double rk_weight2 = 1.0 / std::sqrt(2.0) / 36.0;
const double ISO4_1 = 1.0 / 6.0;
const double ISO4_2 = 1.0 / 12.0;
const double eps14 = 1e-14;  // Misc_module eps (Module.F90:6)

struct Orc {
    mflbm_params p{};
    int nx = 0, ny = 0, nz = 0;
    bool mp = false;
    std::vector<double> f[19], g[19];
    std::vector<double> phi, cnx, cny, cnz, cnorm, curv, u, v, w, rho;
    std::vector<double> phi_old;   // steady_state_option 2 (Monitor.F90:287-365)
    std::vector<int8_t> walls;
    std::vector<double> w_in, fconv, gconv, phiconv;
    std::vector<mflbm_solid_bnd> sb;
    std::vector<mflbm_fluid_bnd> fb;
    bool geometry = false;
    double la_nui1 = 0, la_nui2 = 0, phi_inlet = 0;
    double s_e = 0, s_e2 = 0, s_q = 0, s_nu = 0, s_pi = 0, s_t = 0;  // singlephase rates
    std::string err;

    // halo'd index maps
    inline int64_t I1(int i, int j, int k) const { return (int64_t)i + (int64_t)(nx + 2) * ((int64_t)j + (int64_t)(ny + 2) * k); }
    inline int64_t I2(int i, int j, int k) const { return (int64_t)(i + 1) + (int64_t)(nx + 4) * ((int64_t)(j + 1) + (int64_t)(ny + 4) * (k + 1)); }
    inline int64_t I4(int i, int j, int k) const { return (int64_t)(i + 3) + (int64_t)(nx + 8) * ((int64_t)(j + 3) + (int64_t)(ny + 8) * (k + 3)); }
    inline int64_t IP(int i, int j) const { return (int64_t)i + (int64_t)(nx + 2) * j; }
    inline int64_t IC(int i, int j, int q) const { return (int64_t)i + (int64_t)(nx + 2) * ((int64_t)j + (int64_t)(ny + 2) * q); }
    int64_t n1() const { return (int64_t)(nx + 2) * (ny + 2) * (nz + 2); }
    int64_t n2() const { return (int64_t)(nx + 4) * (ny + 4) * (nz + 4); }
    int64_t n4() const { return (int64_t)(nx + 8) * (ny + 8) * (nz + 8); }
    int64_t nplane() const { return (int64_t)(nx + 2) * (ny + 2); }

    inline double &F(int q, int i, int j, int k) { return f[q][I1(i, j, k)]; }
    inline double &G(int q, int i, int j, int k) { return g[q][I1(i, j, k)]; }
    inline double &PHI(int i, int j, int k) { return phi[I4(i, j, k)]; }
    inline int8_t WALL(int i, int j, int k) const { return walls[I2(i, j, k)]; }
};

thread_local std::string g_create_err;

// -----------------------------------------------------------------------------------
// MRT collision, "MRT kernel, repeated part":
//   multiphase_3D/0.src/Kernel_multiphase.F90:158-267 (odd) / 525-634 (even)
//   singlephase_3D/0.src/Kernel.F90:60-169 (odd) / 261-370 (even)
// ft[] holds the 19 pre-collision bulk PDFs on entry and the post-collision PDFs on
// exit.  den is supplied by the caller (sum of ft for singlephase, rho1+rho2 for the
// colour model).
// -----------------------------------------------------------------------------------
inline void mrt_collide(double *ft, double den, double fx, double fy, double fz,
                        double s_e, double s_e2, double s_q, double s_nu, double s_pi, double s_t) {
    const double ux = ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] + 0.5 * fx;
    const double uy = ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] + 0.5 * fy;
    const double uz = ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] + 0.5 * fz;
    const double u2 = ux * ux + uy * uy + uz * uz;

    double sum1 = ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6];
    double sum2 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
    double sum3 = ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14];
    double sum4 = ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    double sum5 = ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18];
    double sum6 = 2.0 * (ft[1] + ft[2]) - ft[3] - ft[4] - ft[5] - ft[6];
    double sum7 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] - 2.0 * (ft[15] + ft[16] + ft[17] + ft[18]);
    double sum8 = ft[3] + ft[4] - ft[5] - ft[6];
    double sum9 = ft[7] + ft[8] + ft[9] + ft[10] - ft[11] - ft[12] - ft[13] - ft[14];

    double m_rho = den;
    double m_e = -30.0 * ft[0] - 11.0 * sum1 + 8.0 * sum2;
    double m_e2 = 12.0 * ft[0] - 4.0 * sum1 + sum2;
    double m_jx = ft[1] - ft[2] + sum3;
    double m_qx = -4.0 * (ft[1] - ft[2]) + sum3;
    double m_jy = ft[3] - ft[4] + sum4;
    double m_qy = -4.0 * (ft[3] - ft[4]) + sum4;
    double m_jz = ft[5] - ft[6] + sum5;
    double m_qz = -4.0 * (ft[5] - ft[6]) + sum5;
    double m_3pxx = sum6 + sum7;
    double m_3pixx = -2.0 * sum6 + sum7;
    double m_pww = sum8 + sum9;
    double m_piww = -2.0 * sum8 + sum9;
    double m_pxy = ft[7] - ft[8] - ft[9] + ft[10];
    double m_pyz = ft[15] - ft[16] - ft[17] + ft[18];
    double m_pzx = ft[11] - ft[12] - ft[13] + ft[14];
    double m_tx = ft[7] - ft[8] + ft[9] - ft[10] - ft[11] + ft[12] - ft[13] + ft[14];
    double m_ty = -ft[7] - ft[8] + ft[9] + ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    double m_tz = ft[11] + ft[12] - ft[13] - ft[14] - ft[15] - ft[16] + ft[17] + ft[18];

    // relaxation in moment space
    m_e = m_e - s_e * (m_e - (-11.0 * den + 19.0 * u2)) + (38.0 - 19.0 * s_e) * (fx * ux + fy * uy + fz * uz);
    m_e2 = m_e2 - s_e2 * (m_e2 - (mrt_e2_coef1 * den + mrt_e2_coef2 * u2)) + (-11.0 + 5.5 * s_e2) * (fx * ux + fy * uy + fz * uz);
    m_jx = m_jx + fx;
    m_qx = m_qx - s_q * (m_qx - (-0.666666666666666667 * ux)) + (-0.666666666666666667 + 0.333333333333333333 * s_q) * fx;
    m_jy = m_jy + fy;
    m_qy = m_qy - s_q * (m_qy - (-0.666666666666666667 * uy)) + (-0.666666666666666667 + 0.333333333333333333 * s_q) * fy;
    m_jz = m_jz + fz;
    m_qz = m_qz - s_q * (m_qz - (-0.666666666666666667 * uz)) + (-0.666666666666666667 + 0.333333333333333333 * s_q) * fz;

    m_3pxx = m_3pxx - s_nu * (m_3pxx - (3.0 * ux * ux - u2)) + (2.0 - s_nu) * (2.0 * fx * ux - fy * uy - fz * uz);
    m_3pixx = m_3pixx - s_pi * (m_3pixx - mrt_omega_xx * (3.0 * ux * ux - u2)) + (1.0 - 0.5 * s_pi) * (-2.0 * fx * ux + fy * uy + fz * uz);
    m_pww = m_pww - s_nu * (m_pww - (uy * uy - uz * uz)) + (2.0 - s_nu) * (fy * uy - fz * uz);
    m_piww = m_piww - s_pi * (m_piww - mrt_omega_xx * (uy * uy - uz * uz)) + (1.0 - 0.5 * s_pi) * (-fy * uy + fz * uz);
    m_pxy = m_pxy - s_nu * (m_pxy - (ux * uy)) + (1.0 - 0.5 * s_nu) * (fx * uy + fy * ux);
    m_pyz = m_pyz - s_nu * (m_pyz - (uy * uz)) + (1.0 - 0.5 * s_nu) * (fy * uz + fz * uy);
    m_pzx = m_pzx - s_nu * (m_pzx - (ux * uz)) + (1.0 - 0.5 * s_nu) * (fx * uz + fz * ux);
    m_tx = m_tx - s_t * (m_tx);
    m_ty = m_ty - s_t * (m_ty);
    m_tz = m_tz - s_t * (m_tz);

    // back to PDFs
    m_rho = mrt_coef1 * m_rho;
    m_e = mrt_coef2 * m_e;
    m_e2 = mrt_coef3 * m_e2;
    m_jx = 0.1 * m_jx;
    m_qx = 0.025 * m_qx;
    m_jy = 0.1 * m_jy;
    m_qy = 0.025 * m_qy;
    m_jz = 0.1 * m_jz;
    m_qz = 0.025 * m_qz;
    m_3pxx = 2.0 * mrt_coef4 * m_3pxx;
    m_3pixx = mrt_coef4 * m_3pixx;
    m_pww = 6.0 * mrt_coef4 * m_pww;
    m_piww = 3.0 * mrt_coef4 * m_piww;
    m_pxy = 0.25 * m_pxy;
    m_pyz = 0.25 * m_pyz;
    m_pzx = 0.25 * m_pzx;
    m_tx = 0.125 * m_tx;
    m_ty = 0.125 * m_ty;
    m_tz = 0.125 * m_tz;
    sum1 = m_rho - 11.0 * m_e - 4.0 * m_e2;
    sum2 = 2.0 * m_3pxx - 4.0 * m_3pixx;
    sum3 = m_pww - 2.0 * m_piww;
    sum4 = m_rho + 8.0 * m_e + m_e2;
    sum5 = m_jx + m_qx;
    sum6 = m_jy + m_qy;
    sum7 = m_jz + m_qz;
    sum8 = m_3pxx + m_3pixx;
    sum9 = m_pww + m_piww;

    ft[0] = m_rho - 30.0 * m_e + 12.0 * m_e2;
    ft[1] = sum1 + m_jx - 4.0 * m_qx + sum2;
    ft[2] = sum1 - m_jx + 4.0 * m_qx + sum2;
    ft[3] = sum1 + m_jy - 4.0 * m_qy - 0.5 * sum2 + sum3;
    ft[4] = sum1 - m_jy + 4.0 * m_qy - 0.5 * sum2 + sum3;
    ft[5] = sum1 + m_jz - 4.0 * m_qz - 0.5 * sum2 - sum3;
    ft[6] = sum1 - m_jz + 4.0 * m_qz - 0.5 * sum2 - sum3;
    ft[7] = sum4 + sum5 + sum6 + sum8 + sum9 + m_pxy + m_tx - m_ty;
    ft[8] = sum4 - sum5 + sum6 + sum8 + sum9 - m_pxy - m_tx - m_ty;
    ft[9] = sum4 + sum5 - sum6 + sum8 + sum9 - m_pxy + m_tx + m_ty;
    ft[10] = sum4 - sum5 - sum6 + sum8 + sum9 + m_pxy - m_tx + m_ty;
    ft[11] = sum4 + sum5 + sum7 + sum8 - sum9 + m_pzx - m_tx + m_tz;
    ft[12] = sum4 - sum5 + sum7 + sum8 - sum9 - m_pzx + m_tx + m_tz;
    ft[13] = sum4 + sum5 - sum7 + sum8 - sum9 - m_pzx - m_tx - m_tz;
    ft[14] = sum4 - sum5 - sum7 + sum8 - sum9 + m_pzx + m_tx - m_tz;
    ft[15] = sum4 + sum6 + sum7 - sum8 * 2.0 + m_pyz + m_ty - m_tz;
    ft[16] = sum4 - sum6 + sum7 - sum8 * 2.0 - m_pyz - m_ty - m_tz;
    ft[17] = sum4 + sum6 - sum7 - sum8 * 2.0 - m_pyz + m_ty + m_tz;
    ft[18] = sum4 - sum6 - sum7 - sum8 * 2.0 + m_pyz - m_ty + m_tz;
}

// AA-pattern slot maps.
// odd step (Kernel.F90:35-53, 173-191; Kernel_multiphase.F90:46-84, 318-354):
//   read  ft_q <- f_q(x - e_q),  write ft_q -> f_opp(q)(x + e_q)
// even step (Kernel.F90:237-255, 374-392; Kernel_multiphase.F90:410-448, 681-717):
//   read  ft_q <- f_opp(q)(x),   write ft_q -> f_q(x)
const int opc[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

// -----------------------------------------------------------------------------------
// singlephase kernel_odd / kernel_even (singlephase_3D/0.src/Kernel.F90:5-400)
// -----------------------------------------------------------------------------------
void sp_kernel(Orc &o, bool odd) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k) {
        double ft[19];
        for (int j = 1; j <= ny; ++j) {
            for (int i = 1; i <= nx; ++i) {
                if (o.WALL(i, j, k) != 0) continue;
                if (odd) {
                    for (int q = 0; q < 19; ++q) ft[q] = o.F(q, i - ex[q], j - ey[q], k - ez[q]);
                } else {
                    for (int q = 0; q < 19; ++q) ft[q] = o.F(opc[q], i, j, k);
                }
                const double fx = 0.0, fy = 0.0, fz = o.p.force_z;
                const double den = ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] +
                                   ft[11] + ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
                mrt_collide(ft, den, fx, fy, fz, o.s_e, o.s_e2, o.s_q, o.s_nu, o.s_pi, o.s_t);
                if (odd) {
                    o.F(0, i, j, k) = ft[0];
                    for (int q = 1; q < 19; ++q) o.F(opc[q], i + ex[q], j + ey[q], k + ez[q]) = ft[q];
                } else {
                    for (int q = 0; q < 19; ++q) o.F(q, i, j, k) = ft[q];
                }
            }
        }
    }
}

// -----------------------------------------------------------------------------------
// multiphase kernel_odd_color / kernel_even_color
// (multiphase_3D/0.src/Kernel_multiphase.F90:6-362, 371-725)
// -----------------------------------------------------------------------------------
void mp_kernel(Orc &o, bool odd) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const int mrt = o.p.mrt;
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k) {
        double ft[19], a[19], b[19];
        for (int j = 1; j <= ny; ++j) {
            for (int i = 1; i <= nx; ++i) {
                if (o.WALL(i, j, k) != 0) continue;
                if (odd) {
                    for (int q = 0; q < 19; ++q) a[q] = o.F(q, i - ex[q], j - ey[q], k - ez[q]);
                    for (int q = 0; q < 19; ++q) b[q] = o.G(q, i - ex[q], j - ey[q], k - ez[q]);
                } else {
                    for (int q = 0; q < 19; ++q) a[q] = o.F(opc[q], i, j, k);
                    for (int q = 0; q < 19; ++q) b[q] = o.G(opc[q], i, j, k);
                }
                for (int q = 0; q < 19; ++q) ft[q] = a[q] + b[q];
                // order parameter (:108-110)
                const double rho1 = a[0] + a[1] + a[2] + a[3] + a[4] + a[5] + a[6] + a[7] + a[8] + a[9] + a[10] + a[11] +
                                    a[12] + a[13] + a[14] + a[15] + a[16] + a[17] + a[18];
                const double rho2 = b[0] + b[1] + b[2] + b[3] + b[4] + b[5] + b[6] + b[7] + b[8] + b[9] + b[10] + b[11] +
                                    b[12] + b[13] + b[14] + b[15] + b[16] + b[17] + b[18];
                const double ph = (rho1 - rho2) / (rho1 + rho2);
                o.PHI(i, j, k) = ph;
                const int64_t i2 = o.I2(i, j, k);
                const double cnx = o.cnx[i2], cny = o.cny[i2], cnz = o.cnz[i2];
                // CSF force (:116-119)
                double tmp = 0.5 * o.p.gamma * o.curv[o.I1(i, j, k)] * o.cnorm[i2];
                const double fx = tmp * cnx;
                const double fy = tmp * cny;
                const double fz = tmp * cnz + o.p.force_z;
                // viscosity by harmonic interpolation and MRT rates (:124-156)
                const double omega = 1.0 / (6.0 / ((1.0 + ph) * o.la_nui1 + (1.0 - ph) * o.la_nui2) + 0.5);
                const double s_nu = omega;
                double s_e, s_e2, s_pi, s_q, s_t;
                if (mrt == 1) {
                    s_e = omega; s_e2 = omega; s_pi = omega;
                    s_q = 8.0 * (2.0 - omega) / (8.0 - omega);
                    s_t = s_q;
                } else if (mrt == 3) {
                    s_e = omega; s_e2 = omega; s_pi = omega; s_q = omega; s_t = omega;
                } else if (mrt == 4) {
                    s_e = omega; s_e2 = omega; s_pi = omega;
                    s_q = (6.0 - 3.0 * omega) / (3.0 - omega);
                    s_t = omega;
                } else {  // mrt == 2, the reference default (preprocessor.h:2)
                    s_e = 1.19; s_e2 = 1.4; s_pi = 1.4; s_q = 1.2; s_t = 1.98;
                }
                const double den = rho1 + rho2;
                mrt_collide(ft, den, fx, fy, fz, s_e, s_e2, s_q, s_nu, s_pi, s_t);
                // recolouring (:272-315)
                const double tmp1 = rho1 / den;
                a[0] = tmp1 * ft[0];
                b[0] = ft[0] * (1.0 - tmp1);
                tmp = rho1 * rho2 * o.p.beta / den;
                a[1] = tmp1 * ft[1] + w_equ_1 * tmp * (cnx);
                a[2] = tmp1 * ft[2] + w_equ_1 * tmp * (-cnx);
                a[3] = tmp1 * ft[3] + w_equ_1 * tmp * (cny);
                a[4] = tmp1 * ft[4] + w_equ_1 * tmp * (-cny);
                a[5] = tmp1 * ft[5] + w_equ_1 * tmp * (cnz);
                a[6] = tmp1 * ft[6] + w_equ_1 * tmp * (-cnz);
                a[7] = tmp1 * ft[7] + rk_weight2 * tmp * (cnx + cny);
                a[8] = tmp1 * ft[8] + rk_weight2 * tmp * (-cnx + cny);
                a[9] = tmp1 * ft[9] + rk_weight2 * tmp * (cnx - cny);
                a[10] = tmp1 * ft[10] + rk_weight2 * tmp * (-cnx - cny);
                a[11] = tmp1 * ft[11] + rk_weight2 * tmp * (cnx + cnz);
                a[12] = tmp1 * ft[12] + rk_weight2 * tmp * (-cnx + cnz);
                a[13] = tmp1 * ft[13] + rk_weight2 * tmp * (cnx - cnz);
                a[14] = tmp1 * ft[14] + rk_weight2 * tmp * (-cnx - cnz);
                a[15] = tmp1 * ft[15] + rk_weight2 * tmp * (cny + cnz);
                a[16] = tmp1 * ft[16] + rk_weight2 * tmp * (-cny + cnz);
                a[17] = tmp1 * ft[17] + rk_weight2 * tmp * (cny - cnz);
                a[18] = tmp1 * ft[18] + rk_weight2 * tmp * (-cny - cnz);
                for (int q = 1; q < 19; ++q) b[q] = ft[q] - a[q];
                if (odd) {
                    o.F(0, i, j, k) = a[0];
                    o.G(0, i, j, k) = b[0];
                    for (int q = 1; q < 19; ++q) o.F(opc[q], i + ex[q], j + ey[q], k + ez[q]) = a[q];
                    for (int q = 1; q < 19; ++q) o.G(opc[q], i + ex[q], j + ey[q], k + ez[q]) = b[q];
                } else {
                    for (int q = 0; q < 19; ++q) o.F(q, i, j, k) = a[q];
                    for (int q = 0; q < 19; ++q) o.G(q, i, j, k) = b[q];
                }
            }
        }
    }
}

// -----------------------------------------------------------------------------------
// Periodic halo exchange, single-rank form of the Mpi.F90 pack/unpack maps.
// Faces copy 5 PDFs per species over the interior tangential range, then the
// x-edges (y and z periodic) copy one PDF per species, as the reference does
// (multiphase_3D/0.src/Mpi.F90:101-598; singlephase_3D/0.src/Mpi.F90:73-448).
// x-direction periodicity is an extension (the reference rejects iper=1,
// IO_multiphase.F90:472-475); it follows the same pattern, with edges along y and z.
// -----------------------------------------------------------------------------------
struct FaceSet { int out[5]; int in[5]; };
// directions leaving through the +face (e_d = +1) and through the -face (e_d = -1)
const int plusx[5] = {1, 7, 9, 11, 13}, minusx[5] = {2, 8, 10, 12, 14};
const int plusy[5] = {3, 7, 8, 15, 17}, minusy[5] = {4, 10, 9, 16, 18};
const int plusz[5] = {5, 11, 12, 15, 16}, minusz[5] = {6, 14, 13, 18, 17};

void wrap_species(Orc &o, std::vector<double> *A, bool pull) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    auto at = [&](int q, int i, int j, int k) -> double & { return A[q][o.I1(i, j, k)]; };
    const bool px = o.p.iper != 0, py = o.p.jper != 0, pz = o.p.kper != 0;
    if (pull) {
        // after even: ghost slots that the next odd step reads get the periodic image
        if (pz) {  // Mpi.F90:111-130 -> 177-197
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i)
                    for (int n = 0; n < 5; ++n) {
                        at(plusz[n], i, j, 0) = at(plusz[n], i, j, nz);
                        at(minusz[n], i, j, nz + 1) = at(minusz[n], i, j, 1);
                    }
        }
        if (py) {  // Mpi.F90:136-157 -> 207-229
            for (int k = 1; k <= nz; ++k)
                for (int i = 1; i <= nx; ++i)
                    for (int n = 0; n < 5; ++n) {
                        at(plusy[n], i, 0, k) = at(plusy[n], i, ny, k);
                        at(minusy[n], i, ny + 1, k) = at(minusy[n], i, 1, k);
                    }
        }
        if (px) {  // extension
            for (int k = 1; k <= nz; ++k)
                for (int j = 1; j <= ny; ++j)
                    for (int n = 0; n < 5; ++n) {
                        at(plusx[n], 0, j, k) = at(plusx[n], nx, j, k);
                        at(minusx[n], nx + 1, j, k) = at(minusx[n], 1, j, k);
                    }
        }
        if (py && pz) {  // x-edges, Mpi.F90:160-175 -> 240-254
            for (int i = 1; i <= nx; ++i) {
                at(18, i, ny + 1, nz + 1) = at(18, i, 1, 1);
                at(16, i, ny + 1, 0) = at(16, i, 1, nz);
                at(17, i, 0, nz + 1) = at(17, i, ny, 1);
                at(15, i, 0, 0) = at(15, i, ny, nz);
            }
        }
        if (px && pz) {  // y-edges (extension)
            for (int j = 1; j <= ny; ++j) {
                at(11, 0, j, 0) = at(11, nx, j, nz);
                at(12, nx + 1, j, 0) = at(12, 1, j, nz);
                at(13, 0, j, nz + 1) = at(13, nx, j, 1);
                at(14, nx + 1, j, nz + 1) = at(14, 1, j, 1);
            }
        }
        if (px && py) {  // z-edges (extension)
            for (int k = 1; k <= nz; ++k) {
                at(7, 0, 0, k) = at(7, nx, ny, k);
                at(8, nx + 1, 0, k) = at(8, 1, ny, k);
                at(9, 0, ny + 1, k) = at(9, nx, 1, k);
                at(10, nx + 1, ny + 1, k) = at(10, 1, 1, k);
            }
        }
    } else {
        // after odd: slots pushed into ghosts go back to their periodic image
        if (pz) {  // Mpi.F90:364-390 -> 497-519
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i)
                    for (int n = 0; n < 5; ++n) {
                        at(minusz[n], i, j, 1) = at(minusz[n], i, j, nz + 1);
                        at(plusz[n], i, j, nz) = at(plusz[n], i, j, 0);
                    }
        }
        if (py) {  // Mpi.F90:392-414 -> 529-551
            for (int k = 1; k <= nz; ++k)
                for (int i = 1; i <= nx; ++i)
                    for (int n = 0; n < 5; ++n) {
                        at(minusy[n], i, 1, k) = at(minusy[n], i, ny + 1, k);
                        at(plusy[n], i, ny, k) = at(plusy[n], i, 0, k);
                    }
        }
        if (px) {  // extension
            for (int k = 1; k <= nz; ++k)
                for (int j = 1; j <= ny; ++j)
                    for (int n = 0; n < 5; ++n) {
                        at(minusx[n], 1, j, k) = at(minusx[n], nx + 1, j, k);
                        at(plusx[n], nx, j, k) = at(plusx[n], 0, j, k);
                    }
        }
        if (py && pz) {  // Mpi.F90:417-431 -> 570-592 (applied after the faces)
            for (int i = 1; i <= nx; ++i) {
                at(15, i, ny, nz) = at(15, i, 0, 0);
                at(17, i, ny, 1) = at(17, i, 0, nz + 1);
                at(16, i, 1, nz) = at(16, i, ny + 1, 0);
                at(18, i, 1, 1) = at(18, i, ny + 1, nz + 1);
            }
        }
        if (px && pz) {
            for (int j = 1; j <= ny; ++j) {
                at(11, nx, j, nz) = at(11, 0, j, 0);
                at(12, 1, j, nz) = at(12, nx + 1, j, 0);
                at(13, nx, j, 1) = at(13, 0, j, nz + 1);
                at(14, 1, j, 1) = at(14, nx + 1, j, nz + 1);
            }
        }
        if (px && py) {
            for (int k = 1; k <= nz; ++k) {
                at(7, nx, ny, k) = at(7, 0, 0, k);
                at(8, 1, ny, k) = at(8, nx + 1, 0, k);
                at(9, nx, 1, k) = at(9, 0, ny + 1, k);
                at(10, 1, 1, k) = at(10, nx + 1, ny + 1, k);
            }
        }
    }
}

// phi halo (4 layers), MPI_phi_async_pack / MPI_phi_sync_update (Mpi.F90:608-867)
void wrap_phi(Orc &o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const bool py = o.p.jper != 0, pz = o.p.kper != 0;
    if (pz) {
        for (int k = 1; k <= 4; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) {
                    o.PHI(i, j, k - 4) = o.PHI(i, j, nz + k - 4);
                    o.PHI(i, j, k + nz) = o.PHI(i, j, k);
                }
    }
    if (py) {
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= 4; ++j)
                for (int i = 1; i <= nx; ++i) {
                    o.PHI(i, j - 4, k) = o.PHI(i, ny + j - 4, k);
                    o.PHI(i, j + ny, k) = o.PHI(i, j, k);
                }
    }
    if (py && pz) {
        for (int k = 1; k <= 4; ++k)
            for (int j = 1; j <= 4; ++j)
                for (int i = 1; i <= nx; ++i) {
                    o.PHI(i, j - 4, k - 4) = o.PHI(i, ny + j - 4, nz + k - 4);
                    o.PHI(i, j + ny, k - 4) = o.PHI(i, j, nz + k - 4);
                    o.PHI(i, j + ny, k + nz) = o.PHI(i, j, k);
                    o.PHI(i, j - 4, k + nz) = o.PHI(i, ny + j - 4, k);
                }
    }
}

// -----------------------------------------------------------------------------------
// Inlet / outlet / porous-plate boundary conditions.
// multiphase: Boundary_multiphase_inlet.F90, Boundary_multiphase_outlet.F90,
//             Boundary_multiphase_other.F90;  singlephase: Boundary.F90.
// wall_indicator arithmetic is kept literally: x*(1-w) + y*w.
// -----------------------------------------------------------------------------------
inline double sel(double x, double y, int w) { return x * (double)(1 - w) + y * (double)w; }

// velocity inlet (bounce-back type); before_odd: Boundary_multiphase_inlet.F90:6-53,
// singlephase Boundary.F90:5-40; after_odd: :56-102 / Boundary.F90:43-73
void inlet_velocity(Orc &o, bool before_odd) {
    const int nx = o.nx, ny = o.ny;
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const int wi = o.WALL(i, j, 1);
            if (o.mp) {
                o.PHI(i, j, 0) = o.phi_inlet * (double)(1 - wi) + o.PHI(i, j, 0) * (double)wi;
                o.PHI(i, j, -1) = o.PHI(i, j, 0);
                o.PHI(i, j, -2) = o.PHI(i, j, 0);
                o.PHI(i, j, -3) = o.PHI(i, j, 0);
            }
            double tmp2 = o.w_in[o.IP(i, j)] * o.p.relaxation;
            double tmp1;
            if (o.mp) {
                tmp1 = tmp2 * o.p.sa_inject;
                tmp2 = tmp2 - tmp1;
            } else {
                tmp1 = tmp2;
            }
            const int nsp = o.mp ? 2 : 1;
            for (int s = 0; s < nsp; ++s) {
                std::vector<double> *A = s == 0 ? o.f : o.g;
                const double t = s == 0 ? tmp1 : tmp2;
                auto at = [&](int q, int ii, int jj, int kk) -> double & { return A[q][o.I1(ii, jj, kk)]; };
                if (before_odd) {
                    at(5, i, j, 0) = sel(at(6, i, j, 1) + 6.0 * w_equ_1 * t, at(5, i, j, 0), wi);
                    at(11, i - 1, j, 0) = sel(at(14, i, j, 1) + 6.0 * w_equ_2 * t, at(11, i - 1, j, 0), wi);
                    at(12, i + 1, j, 0) = sel(at(13, i, j, 1) + 6.0 * w_equ_2 * t, at(12, i + 1, j, 0), wi);
                    at(15, i, j - 1, 0) = sel(at(18, i, j, 1) + 6.0 * w_equ_2 * t, at(15, i, j - 1, 0), wi);
                    at(16, i, j + 1, 0) = sel(at(17, i, j, 1) + 6.0 * w_equ_2 * t, at(16, i, j + 1, 0), wi);
                } else {
                    at(6, i, j, 1) = sel(at(5, i, j, 0) + 6.0 * w_equ_1 * t, at(6, i, j, 1), wi);
                    at(13, i, j, 1) = sel(at(12, i + 1, j, 0) + 6.0 * w_equ_2 * t, at(13, i, j, 1), wi);
                    at(14, i, j, 1) = sel(at(11, i - 1, j, 0) + 6.0 * w_equ_2 * t, at(14, i, j, 1), wi);
                    at(17, i, j, 1) = sel(at(16, i, j + 1, 0) + 6.0 * w_equ_2 * t, at(17, i, j, 1), wi);
                    at(18, i, j, 1) = sel(at(15, i, j - 1, 0) + 6.0 * w_equ_2 * t, at(18, i, j, 1), wi);
                }
            }
        }
}

// Zou-He pressure inlet; before_odd: Boundary_multiphase_inlet.F90:115-209,
// singlephase Boundary.F90:80-135; after_odd: :212-294 / Boundary.F90:138-187
void inlet_zouhe(Orc &o, bool before_odd) {
    const int nx = o.nx, ny = o.ny;
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const int wi = o.WALL(i, j, 1);
            double rhos[2];
            if (o.mp) {
                o.PHI(i, j, 0) = o.phi_inlet * (double)(1 - wi) + o.PHI(i, j, 0) * (double)wi;
                o.PHI(i, j, -1) = o.PHI(i, j, 0);
                o.PHI(i, j, -2) = o.PHI(i, j, 0);
                o.PHI(i, j, -3) = o.PHI(i, j, 0);
                double tmpRho2 = o.p.rho_in;
                const double tmpRho1 = o.p.rho_in * o.p.sa_inject;
                tmpRho2 = tmpRho2 - tmpRho1;
                rhos[0] = tmpRho1;
                rhos[1] = tmpRho2;
            } else {
                rhos[0] = o.p.rho_in;
            }
            const int nsp = o.mp ? 2 : 1;
            for (int s = 0; s < nsp; ++s) {
                std::vector<double> *A = s == 0 ? o.f : o.g;
                auto at = [&](int q, int ii, int jj, int kk) -> double & { return A[q][o.I1(ii, jj, kk)]; };
                if (before_odd) {
                    const double t = (rhos[s] - (at(0, i, j, 1) + at(1, i - 1, j, 1) + at(2, i + 1, j, 1) + at(3, i, j - 1, 1) +
                                                 at(4, i, j + 1, 1) + at(7, i - 1, j - 1, 1) + at(8, i + 1, j - 1, 1) +
                                                 at(9, i - 1, j + 1, 1) + at(10, i + 1, j + 1, 1) +
                                                 2.0 * (at(6, i, j, 2) + at(14, i + 1, j, 2) + at(13, i - 1, j, 2) +
                                                        at(18, i, j + 1, 2) + at(17, i, j - 1, 2)))) *
                                     o.p.relaxation;
                    const double tnx = 0.5 * (at(1, i - 1, j, 1) + at(7, i - 1, j - 1, 1) + at(9, i - 1, j + 1, 1) -
                                              (at(2, i + 1, j, 1) + at(8, i + 1, j - 1, 1) + at(10, i + 1, j + 1, 1)));
                    const double tny = 0.5 * (at(3, i, j - 1, 1) + at(7, i - 1, j - 1, 1) + at(8, i + 1, j - 1, 1) -
                                              (at(4, i, j + 1, 1) + at(10, i + 1, j + 1, 1) + at(9, i - 1, j + 1, 1)));
                    at(5, i, j, 0) = sel(at(6, i, j, 2) + 0.333333333333333333 * t, at(5, i, j, 0), wi);
                    at(11, i - 1, j, 0) = sel(at(14, i + 1, j, 2) + 0.166666666666666667 * t - tnx, at(11, i - 1, j, 0), wi);
                    at(12, i + 1, j, 0) = sel(at(13, i - 1, j, 2) + 0.166666666666666667 * t + tnx, at(12, i + 1, j, 0), wi);
                    at(15, i, j - 1, 0) = sel(at(18, i, j + 1, 2) + 0.166666666666666667 * t - tny, at(15, i, j - 1, 0), wi);
                    at(16, i, j + 1, 0) = sel(at(17, i, j - 1, 2) + 0.166666666666666667 * t + tny, at(16, i, j + 1, 0), wi);
                } else {
                    const double t = (rhos[s] - (at(0, i, j, 1) + at(2, i, j, 1) + at(1, i, j, 1) + at(4, i, j, 1) +
                                                 at(3, i, j, 1) + at(8, i, j, 1) + at(7, i, j, 1) + at(10, i, j, 1) +
                                                 at(9, i, j, 1) +
                                                 2.0 * (at(5, i, j, 1) + at(11, i, j, 1) + at(12, i, j, 1) + at(15, i, j, 1) +
                                                        at(16, i, j, 1)))) *
                                     o.p.relaxation;
                    const double tnx = 0.5 * (at(2, i, j, 1) + at(8, i, j, 1) + at(10, i, j, 1) -
                                              (at(1, i, j, 1) + at(7, i, j, 1) + at(9, i, j, 1)));
                    const double tny = 0.5 * (at(4, i, j, 1) + at(9, i, j, 1) + at(10, i, j, 1) -
                                              (at(3, i, j, 1) + at(8, i, j, 1) + at(7, i, j, 1)));
                    at(6, i, j, 1) = sel(at(5, i, j, 1) + 0.333333333333333333 * t, at(6, i, j, 1), wi);
                    at(13, i, j, 1) = sel(at(12, i, j, 1) + 0.166666666666666667 * t + tnx, at(13, i, j, 1), wi);
                    at(14, i, j, 1) = sel(at(11, i, j, 1) + 0.166666666666666667 * t - tnx, at(14, i, j, 1), wi);
                    at(17, i, j, 1) = sel(at(16, i, j, 1) + 0.166666666666666667 * t + tny, at(17, i, j, 1), wi);
                    at(18, i, j, 1) = sel(at(15, i, j, 1) + 0.166666666666666667 * t - tny, at(18, i, j, 1), wi);
                }
            }
        }
}

// convective outlet; before_odd: Boundary_multiphase_outlet.F90:7-65, singlephase
// Boundary.F90:196-237; after_odd: :68-127 / Boundary.F90:240-276
void outlet_convective(Orc &o, bool before_odd) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    const double u_convec = o.p.uin_avg;
    const double temp = 1.0 / (1.0 + u_convec);
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const int wi = o.WALL(i, j, nz);
            if (o.mp) {
                o.PHI(i, j, nz + 1) = ((o.phiconv[o.IP(i, j)] + u_convec * o.PHI(i, j, nz)) * temp) * (double)(1 - wi) +
                                      o.PHI(i, j, nz + 1) * (double)wi;
                o.phiconv[o.IP(i, j)] = o.PHI(i, j, nz + 1);
                o.PHI(i, j, nz + 2) = o.PHI(i, j, nz + 1);
                o.PHI(i, j, nz + 3) = o.PHI(i, j, nz + 1);
                o.PHI(i, j, nz + 4) = o.PHI(i, j, nz + 1);
            }
            const int nsp = o.mp ? 2 : 1;
            for (int s = 0; s < nsp; ++s) {
                std::vector<double> *A = s == 0 ? o.f : o.g;
                std::vector<double> &C = s == 0 ? o.fconv : o.gconv;
                auto at = [&](int q, int ii, int jj, int kk) -> double & { return A[q][o.I1(ii, jj, kk)]; };
                auto cv = [&](int q) -> double & { return C[o.IC(i, j, q)]; };
                if (before_odd) {
                    at(6, i, j, nz + 1) = sel((cv(6) + u_convec * at(6, i, j, nz)) * temp, at(6, i, j, nz + 1), wi);
                    at(13, i - 1, j, nz + 1) = sel((cv(13) + u_convec * at(13, i - 1, j, nz)) * temp, at(13, i - 1, j, nz + 1), wi);
                    at(14, i + 1, j, nz + 1) = sel((cv(14) + u_convec * at(14, i + 1, j, nz)) * temp, at(14, i + 1, j, nz + 1), wi);
                    at(17, i, j - 1, nz + 1) = sel((cv(17) + u_convec * at(17, i, j - 1, nz)) * temp, at(17, i, j - 1, nz + 1), wi);
                    at(18, i, j + 1, nz + 1) = sel((cv(18) + u_convec * at(18, i, j + 1, nz)) * temp, at(18, i, j + 1, nz + 1), wi);
                    cv(6) = at(6, i, j, nz + 1);
                    cv(13) = at(13, i - 1, j, nz + 1);
                    cv(14) = at(14, i + 1, j, nz + 1);
                    cv(17) = at(17, i, j - 1, nz + 1);
                    cv(18) = at(18, i, j + 1, nz + 1);
                } else {
                    at(5, i, j, nz) = sel((cv(6) + u_convec * at(5, i, j, nz - 1)) * temp, at(5, i, j, nz), wi);
                    at(11, i, j, nz) = sel((cv(14) + u_convec * at(11, i, j, nz - 1)) * temp, at(11, i, j, nz), wi);
                    at(12, i, j, nz) = sel((cv(13) + u_convec * at(12, i, j, nz - 1)) * temp, at(12, i, j, nz), wi);
                    at(15, i, j, nz) = sel((cv(18) + u_convec * at(15, i, j, nz - 1)) * temp, at(15, i, j, nz), wi);
                    at(16, i, j, nz) = sel((cv(17) + u_convec * at(16, i, j, nz - 1)) * temp, at(16, i, j, nz), wi);
                    cv(6) = at(5, i, j, nz);
                    cv(14) = at(11, i, j, nz);
                    cv(13) = at(12, i, j, nz);
                    cv(18) = at(15, i, j, nz);
                    cv(17) = at(16, i, j, nz);
                }
            }
        }
}

// Zou-He pressure outlet; before_odd: Boundary_multiphase_outlet.F90:139-228,
// singlephase Boundary.F90:284-334; after_odd: :231-311 / Boundary.F90:337-389
void outlet_zouhe(Orc &o, bool before_odd) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const int wi = o.WALL(i, j, nz);
            if (o.mp) {
                o.PHI(i, j, nz + 1) = o.PHI(i, j, nz);
                o.PHI(i, j, nz + 2) = o.PHI(i, j, nz);
                o.PHI(i, j, nz + 3) = o.PHI(i, j, nz);
                o.PHI(i, j, nz + 4) = o.PHI(i, j, nz);
            }
            auto F = [&](int q, int ii, int jj, int kk) -> double & { return o.f[q][o.I1(ii, jj, kk)]; };
            auto G = [&](int q, int ii, int jj, int kk) -> double & { return o.g[q][o.I1(ii, jj, kk)]; };
            double t1;
            if (before_odd) {
                t1 = F(0, i, j, nz) + F(1, i - 1, j, nz) + F(2, i + 1, j, nz) + F(3, i, j - 1, nz) + F(4, i, j + 1, nz) +
                     F(7, i - 1, j - 1, nz) + F(8, i + 1, j - 1, nz) + F(9, i - 1, j + 1, nz) + F(10, i + 1, j + 1, nz) +
                     2.0 * (F(5, i, j, nz - 1) + F(11, i - 1, j, nz - 1) + F(12, i + 1, j, nz - 1) + F(15, i, j - 1, nz - 1) +
                            F(16, i, j + 1, nz - 1));
                if (o.mp) {
                    t1 = t1 + G(0, i, j, nz) + G(1, i - 1, j, nz) + G(2, i + 1, j, nz) + G(3, i, j - 1, nz) + G(4, i, j + 1, nz) +
                         G(7, i - 1, j - 1, nz) + G(8, i + 1, j - 1, nz) + G(9, i - 1, j + 1, nz) + G(10, i + 1, j + 1, nz) +
                         2.0 * (G(5, i, j, nz - 1) + G(11, i - 1, j, nz - 1) + G(12, i + 1, j, nz - 1) + G(15, i, j - 1, nz - 1) +
                                G(16, i, j + 1, nz - 1));
                }
            } else {
                t1 = F(0, i, j, nz) + F(2, i, j, nz) + F(1, i, j, nz) + F(4, i, j, nz) + F(3, i, j, nz) + F(8, i, j, nz) +
                     F(7, i, j, nz) + F(10, i, j, nz) + F(9, i, j, nz) +
                     2.0 * (F(6, i, j, nz) + F(14, i, j, nz) + F(13, i, j, nz) + F(18, i, j, nz) + F(17, i, j, nz));
                if (o.mp) {
                    t1 = t1 + G(0, i, j, nz) + G(2, i, j, nz) + G(1, i, j, nz) + G(4, i, j, nz) + G(3, i, j, nz) + G(8, i, j, nz) +
                         G(7, i, j, nz) + G(10, i, j, nz) + G(9, i, j, nz) +
                         2.0 * (G(6, i, j, nz) + G(14, i, j, nz) + G(13, i, j, nz) + G(18, i, j, nz) + G(17, i, j, nz));
                }
            }
            t1 = t1 - o.p.rho_out;
            double t2 = 0.0;
            if (o.mp) {
                t2 = t1 * 0.5 * (1.0 - o.PHI(i, j, nz));
                t1 = t1 - t2;
            }
            const int nsp = o.mp ? 2 : 1;
            for (int s = 0; s < nsp; ++s) {
                std::vector<double> *A = s == 0 ? o.f : o.g;
                const double t = s == 0 ? t1 : t2;
                auto at = [&](int q, int ii, int jj, int kk) -> double & { return A[q][o.I1(ii, jj, kk)]; };
                const double w1 = 1.0 - (double)wi;
                const double w0 = (double)wi;
                if (before_odd) {
                    const double tnx = 0.5 * (at(1, i - 1, j, nz) + at(7, i - 1, j - 1, nz) + at(9, i - 1, j + 1, nz) -
                                              (at(2, i + 1, j, nz) + at(8, i + 1, j - 1, nz) + at(10, i + 1, j + 1, nz)));
                    const double tny = 0.5 * (at(3, i, j - 1, nz) + at(7, i - 1, j - 1, nz) + at(8, i + 1, j - 1, nz) -
                                              (at(4, i, j + 1, nz) + at(10, i + 1, j + 1, nz) + at(9, i - 1, j + 1, nz)));
                    at(6, i, j, nz + 1) = (at(5, i, j, nz - 1) - 0.333333333333333333 * t) * w1 + at(6, i, j, nz + 1) * w0;
                    at(13, i - 1, j, nz + 1) = (at(12, i + 1, j, nz - 1) - 0.166666666666666667 * t - tnx) * w1 + at(13, i - 1, j, nz + 1) * w0;
                    at(14, i + 1, j, nz + 1) = (at(11, i - 1, j, nz - 1) - 0.166666666666666667 * t + tnx) * w1 + at(14, i + 1, j, nz + 1) * w0;
                    at(17, i, j - 1, nz + 1) = (at(16, i, j + 1, nz - 1) - 0.166666666666666667 * t - tny) * w1 + at(17, i, j - 1, nz + 1) * w0;
                    at(18, i, j + 1, nz + 1) = (at(15, i, j - 1, nz - 1) - 0.166666666666666667 * t + tny) * w1 + at(18, i, j + 1, nz + 1) * w0;
                } else {
                    const double tnx = 0.5 * (at(2, i, j, nz) + at(8, i, j, nz) + at(10, i, j, nz) -
                                              (at(1, i, j, nz) + at(7, i, j, nz) + at(9, i, j, nz)));
                    const double tny = 0.5 * (at(4, i, j, nz) + at(10, i, j, nz) + at(9, i, j, nz) -
                                              (at(3, i, j, nz) + at(7, i, j, nz) + at(8, i, j, nz)));
                    at(5, i, j, nz) = (at(6, i, j, nz) - 0.333333333333333333 * t) * w1 + at(5, i, j, nz) * w0;
                    at(11, i, j, nz) = (at(14, i, j, nz) - 0.166666666666666667 * t + tnx) * w1 + at(11, i, j, nz) * w0;
                    at(12, i, j, nz) = (at(13, i, j, nz) - 0.166666666666666667 * t - tnx) * w1 + at(12, i, j, nz) * w0;
                    at(15, i, j, nz) = (at(18, i, j, nz) - 0.166666666666666667 * t + tny) * w1 + at(15, i, j, nz) * w0;
                    at(16, i, j, nz) = (at(17, i, j, nz) - 0.166666666666666667 * t - tny) * w1 + at(16, i, j, nz) * w0;
                }
            }
        }
}

// porous plate (Boundary_multiphase_other.F90:8-184)
void porous_plate(Orc &o, bool before_odd) {
    const int nx = o.nx, ny = o.ny;
    const int z = o.p.z_porous_plate;
    if (z < 1 || z > o.nz) return;
    // cmd 1 blocks fluid 1 (f), cmd 2 blocks fluid 2 (g)
    std::vector<double> *B = o.p.porous_plate_cmd == 1 ? o.f : o.g;  // blocked species
    std::vector<double> *P = o.p.porous_plate_cmd == 1 ? o.g : o.f;  // passing species
    auto b = [&](int q, int i, int j, int k) -> double & { return B[q][o.I1(i, j, k)]; };
    auto c = [&](int q, int i, int j, int k) -> double & { return P[q][o.I1(i, j, k)]; };
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
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
}

// -----------------------------------------------------------------------------------
// color_gradient (multiphase_3D/0.src/Phase_gradient.F90:5-204) and
// alter_color_gradient_solid_surface (:210-265)
// -----------------------------------------------------------------------------------
void color_gradient(Orc &o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    // phi extrapolation to solid boundary nodes (:13-30)
    for (const auto &s : o.sb) {
        double acc = 0.0;
        for (int n = 0; n < s.i_fluid_num; ++n) {
            const int ie = s.neighbor_list[n];
            acc = acc + o.PHI(s.ix + ex[ie], s.iy + ey[ie], s.iz + ez[ie]) * w_equ[ie];
        }
        o.PHI(s.ix, s.iy, s.iz) = acc / s.la_weight;
    }
    // normals from the ISO4 phi gradient over [1-2, n+2]^3 (:33-79)
#pragma omp parallel for schedule(static)
    for (int k = -1; k <= nz + 2; ++k)
        for (int j = -1; j <= ny + 2; ++j)
            for (int i = -1; i <= nx + 2; ++i) {
                auto P = [&](int a, int b, int c) { return o.phi[o.I4(a, b, c)]; };
                double gx = ISO4_1 * (P(i + 1, j, k) - P(i - 1, j, k)) +
                            ISO4_2 * (P(i + 1, j + 1, k) - P(i - 1, j - 1, k) + P(i + 1, j - 1, k) - P(i - 1, j + 1, k) +
                                      P(i + 1, j, k + 1) - P(i - 1, j, k - 1) + P(i + 1, j, k - 1) - P(i - 1, j, k + 1));
                double gy = ISO4_1 * (P(i, j + 1, k) - P(i, j - 1, k)) +
                            ISO4_2 * (P(i + 1, j + 1, k) - P(i - 1, j - 1, k) + P(i - 1, j + 1, k) - P(i + 1, j - 1, k) +
                                      P(i, j + 1, k + 1) - P(i, j - 1, k - 1) + P(i, j + 1, k - 1) - P(i, j - 1, k + 1));
                double gz = ISO4_1 * (P(i, j, k + 1) - P(i, j, k - 1)) +
                            ISO4_2 * (P(i + 1, j, k + 1) - P(i - 1, j, k - 1) + P(i - 1, j, k + 1) - P(i + 1, j, k - 1) +
                                      P(i, j + 1, k + 1) - P(i, j - 1, k - 1) + P(i, j - 1, k + 1) - P(i, j + 1, k - 1));
                double cn = std::sqrt(gx * gx + gy * gy + gz * gz);
                const int64_t id = o.I2(i, j, k);
                if (cn < 1e-6 || o.walls[id] == 1) {
                    gx = 0.0; gy = 0.0; gz = 0.0; cn = 0.0;
                } else {
                    gx = gx / cn; gy = gy / cn; gz = gz / cn;
                }
                o.cnx[id] = gx; o.cny[id] = gy; o.cnz[id] = gz; o.cnorm[id] = cn;
            }
    // wetting (:223-262): theta per node; cos/sin evaluated per node as the reference does
    const double local_eps = 1e-6;
    for (const auto &fbn : o.fb) {
        const int64_t id = o.I2(fbn.ix, fbn.iy, fbn.iz);
        if (o.cnorm[id] > local_eps) {
            const double th = fbn.theta;
            const double nwx = fbn.nwx, nwy = fbn.nwy, nwz = fbn.nwz;
            const double cnx0 = o.cnx[id], cny0 = o.cny[id], cnz0 = o.cnz[id];
            const double tmpCos = std::cos(th);
            const double tmp1 = nwx * cnx0 + nwy * cny0 + nwz * cnz0;
            const double tmp2 = 1.0 / std::sqrt(1.0 - tmp1 * tmp1);
            const double sn = std::sin(th);
            const double coe1 = sn * tmp1 * tmp2;
            const double coe2 = sn * tmp2;
            const double cnxp = (tmpCos - coe1) * nwx + coe2 * cnx0;
            const double cnyp = (tmpCos - coe1) * nwy + coe2 * cny0;
            const double cnzp = (tmpCos - coe1) * nwz + coe2 * cnz0;
            const double cnxm = (tmpCos + coe1) * nwx - coe2 * cnx0;
            const double cnym = (tmpCos + coe1) * nwy - coe2 * cny0;
            const double cnzm = (tmpCos + coe1) * nwz - coe2 * cnz0;
            const double distP = (cnxp - cnx0) * (cnxp - cnx0) + (cnyp - cny0) * (cnyp - cny0) + (cnzp - cnz0) * (cnzp - cnz0);
            const double distM = (cnxm - cnx0) * (cnxm - cnx0) + (cnym - cny0) * (cnym - cny0) + (cnzm - cnz0) * (cnzm - cnz0);
            if (distP <= distM) {
                o.cnx[id] = cnxp; o.cny[id] = cnyp; o.cnz[id] = cnzp;
            } else {
                o.cnx[id] = cnxm; o.cny[id] = cnym; o.cnz[id] = cnzm;
            }
        }
    }
    // normal extrapolation to solid boundary nodes in [0, n+1]^3 (:85-110)
    for (const auto &s : o.sb) {
        const int i = s.ix, j = s.iy, k = s.iz;
        if (i >= 0 && i <= nx + 1 && j >= 0 && j <= ny + 1 && k >= 0 && k <= nz + 1) {
            double ax = 0.0, ay = 0.0, az = 0.0;
            for (int n = 0; n < s.i_fluid_num; ++n) {
                const int ie = s.neighbor_list[n];
                const int64_t nb = o.I2(i + ex[ie], j + ey[ie], k + ez[ie]);
                ax = ax + o.cnx[nb] * w_equ[ie];
                ay = ay + o.cny[nb] * w_equ[ie];
                az = az + o.cnz[nb] * w_equ[ie];
            }
            const int64_t id = o.I2(i, j, k);
            o.cnx[id] = ax / s.la_weight;
            o.cny[id] = ay / s.la_weight;
            o.cnz[id] = az / s.la_weight;
        }
    }
    // curvature over [1, n]^3 (:113-201)
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                auto X = [&](int a, int b, int c) { return o.cnx[o.I2(a, b, c)]; };
                auto Y = [&](int a, int b, int c) { return o.cny[o.I2(a, b, c)]; };
                auto Z = [&](int a, int b, int c) { return o.cnz[o.I2(a, b, c)]; };
                const double kxx = ISO4_1 * (X(i + 1, j, k) - X(i - 1, j, k)) +
                                   ISO4_2 * (X(i + 1, j + 1, k) - X(i - 1, j - 1, k) + X(i + 1, j - 1, k) - X(i - 1, j + 1, k) +
                                             X(i + 1, j, k + 1) - X(i - 1, j, k - 1) + X(i + 1, j, k - 1) - X(i - 1, j, k + 1));
                const double kyy = ISO4_1 * (Y(i, j + 1, k) - Y(i, j - 1, k)) +
                                   ISO4_2 * (Y(i + 1, j + 1, k) - Y(i - 1, j - 1, k) + Y(i - 1, j + 1, k) - Y(i + 1, j - 1, k) +
                                             Y(i, j + 1, k + 1) - Y(i, j - 1, k - 1) + Y(i, j + 1, k - 1) - Y(i, j - 1, k + 1));
                const double kzz = ISO4_1 * (Z(i, j, k + 1) - Z(i, j, k - 1)) +
                                   ISO4_2 * (Z(i + 1, j, k + 1) - Z(i - 1, j, k - 1) + Z(i - 1, j, k + 1) - Z(i + 1, j, k - 1) +
                                             Z(i, j + 1, k + 1) - Z(i, j - 1, k - 1) + Z(i, j - 1, k + 1) - Z(i, j + 1, k - 1));
                const double kxy = ISO4_1 * (X(i, j + 1, k) - X(i, j - 1, k)) +
                                   ISO4_2 * (X(i + 1, j + 1, k) - X(i - 1, j - 1, k) + X(i - 1, j + 1, k) - X(i + 1, j - 1, k) +
                                             X(i, j + 1, k + 1) - X(i, j - 1, k - 1) + X(i, j + 1, k - 1) - X(i, j - 1, k + 1));
                const double kxz = ISO4_1 * (X(i, j, k + 1) - X(i, j, k - 1)) +
                                   ISO4_2 * (X(i + 1, j, k + 1) - X(i - 1, j, k - 1) + X(i - 1, j, k + 1) - X(i + 1, j, k - 1) +
                                             X(i, j + 1, k + 1) - X(i, j - 1, k - 1) + X(i, j - 1, k + 1) - X(i, j + 1, k - 1));
                const double kyx = ISO4_1 * (Y(i + 1, j, k) - Y(i - 1, j, k)) +
                                   ISO4_2 * (Y(i + 1, j + 1, k) - Y(i - 1, j - 1, k) + Y(i + 1, j - 1, k) - Y(i - 1, j + 1, k) +
                                             Y(i + 1, j, k + 1) - Y(i - 1, j, k - 1) + Y(i + 1, j, k - 1) - Y(i - 1, j, k + 1));
                const double kyz = ISO4_1 * (Y(i, j, k + 1) - Y(i, j, k - 1)) +
                                   ISO4_2 * (Y(i + 1, j, k + 1) - Y(i - 1, j, k - 1) + Y(i - 1, j, k + 1) - Y(i + 1, j, k - 1) +
                                             Y(i, j + 1, k + 1) - Y(i, j - 1, k - 1) + Y(i, j - 1, k + 1) - Y(i, j + 1, k - 1));
                const double kzx = ISO4_1 * (Z(i + 1, j, k) - Z(i - 1, j, k)) +
                                   ISO4_2 * (Z(i + 1, j + 1, k) - Z(i - 1, j - 1, k) + Z(i + 1, j - 1, k) - Z(i - 1, j + 1, k) +
                                             Z(i + 1, j, k + 1) - Z(i - 1, j, k - 1) + Z(i + 1, j, k - 1) - Z(i - 1, j, k + 1));
                const double kzy = ISO4_1 * (Z(i, j + 1, k) - Z(i, j - 1, k)) +
                                   ISO4_2 * (Z(i + 1, j + 1, k) - Z(i - 1, j - 1, k) + Z(i - 1, j + 1, k) - Z(i + 1, j - 1, k) +
                                             Z(i, j + 1, k + 1) - Z(i, j - 1, k - 1) + Z(i, j + 1, k - 1) - Z(i, j - 1, k + 1));
                const double cx = X(i, j, k), cy = Y(i, j, k), cz = Z(i, j, k);
                o.curv[o.I1(i, j, k)] = (cx * cx - 1.0) * kxx + (cy * cy - 1.0) * kyy + (cz * cz - 1.0) * kzz +
                                        cx * cy * (kxy + kyx) + cx * cz * (kxz + kzx) + cy * cz * (kzy + kyz);
            }
}

// compute_macro_vars (multiphase_3D/0.src/Misc.F90:372-430; singlephase Misc.F90:368-423)
void macro_vars(Orc &o) {
    const int nx = o.nx, ny = o.ny, nz = o.nz;
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const int wi = o.WALL(i, j, k);
                const int64_t id = o.I1(i, j, k);
                double ft[19];
                if (o.mp) {
                    for (int q = 0; q < 19; ++q) ft[q] = o.f[q][id] + o.g[q][id];
                } else {
                    for (int q = 0; q < 19; ++q) ft[q] = o.f[q][id];
                }
                const double m = (double)(1 - wi);
                o.rho[id] = (ft[0] + ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6] + ft[7] + ft[8] + ft[9] + ft[10] + ft[11] +
                             ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18]) * m;
                double fx = 0.0, fy = 0.0, fz = o.p.force_z;
                if (o.mp) {
                    const int64_t i2 = o.I2(i, j, k);
                    const double tmp = 0.5 * o.p.gamma * o.curv[id] * o.cnorm[i2];
                    fx = tmp * o.cnx[i2];
                    fy = tmp * o.cny[i2];
                    fz = tmp * o.cnz[i2] + o.p.force_z;
                }
                o.u[id] = (ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] - 0.5 * fx) * m;
                o.v[id] = (ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] - 0.5 * fy) * m;
                o.w[id] = (ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] - 0.5 * fz) * m;
                if (o.mp) {
                    const int64_t i4 = o.I4(i, j, k);
                    o.phi[i4] = 0.0 * (double)wi + o.phi[i4] * m;
                }
            }
}

bool open_z(const Orc &o) {
    return o.p.kper == 0 && o.p.wall_z_min == 0 && o.p.wall_z_max == 0;
}

// main_iteration_kernel (multiphase_3D/0.src/Main_multiphase.F90:341-486;
// singlephase_3D/0.src/Main.F90:291-422)
void step(Orc &o, int ntime) {
    const bool even = (ntime % 2) == 0;
    if (o.mp) mp_kernel(o, !even); else sp_kernel(o, !even);
    // periodic halo exchange: pull after even, push after odd; phi after both
    wrap_species(o, o.f, even);
    if (o.mp) {
        wrap_species(o, o.g, even);
        wrap_phi(o);
    }
    if (open_z(o)) {
        if (o.p.inlet_bc == 1) inlet_velocity(o, even);
        else if (o.p.inlet_bc == 2) inlet_zouhe(o, even);
        if (o.p.outlet_bc == 1) outlet_convective(o, even);
        else if (o.p.outlet_bc == 2) outlet_zouhe(o, even);
    }
    if (o.mp && o.p.porous_plate_cmd != 0) porous_plate(o, even);
    if (o.mp) color_gradient(o);
}

int validate(const mflbm_params *p, std::string &err) {
    if (!p) { err = "params is NULL"; return MFLBM_EINVAL; }
    if (p->abi_version != MFLBM_ABI_VERSION) { err = "abi_version mismatch"; return MFLBM_EINVAL; }
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) { err = "lattice dimensions must be >= 3"; return MFLBM_EINVAL; }
    if (p->multiphase) {
        // IO_multiphase.F90:472-475: x must be walled and non-periodic
        if (p->iper == 1 || p->wall_x_max == 0 || p->wall_x_min == 0) {
            err = "X direction periodic BC enabled or non-slip BC not applied at x = xmin or x = xmax";
            return MFLBM_EINVAL;
        }
    } else if (p->iper == 1 && (p->wall_x_max == 1 || p->wall_x_min == 1)) {
        err = "non-slip BC applied at x = xmin or x = xmax while x direction periodic BC enabled";
        return MFLBM_EINVAL;
    }
    if (!p->multiphase && p->iper == 0 && (p->wall_x_max == 0 || p->wall_x_min == 0)) {
        err = "non-slip BC not applied at x = xmin or x = xmax while x direction periodic BC not enabled";
        return MFLBM_EINVAL;
    }
    if (p->jper == 0 && (p->wall_y_max == 0 || p->wall_y_min == 0)) {
        err = "non-slip BC not applied at y = ymin or y = ymax while y direction periodic BC not enabled";
        return MFLBM_EINVAL;
    }
    if (p->jper == 1 && (p->wall_y_max == 1 || p->wall_y_min == 1)) {
        err = "non-slip BC applied at y = ymin or y = ymax while y direction periodic BC enabled";
        return MFLBM_EINVAL;
    }
    if (p->kper == 1 && (p->wall_z_max == 1 || p->wall_z_min == 1)) {
        err = "non-slip BC applied at z = zmin or z = zmax while z direction periodic BC enabled";
        return MFLBM_EINVAL;
    }
    if (p->outlet_bc == 1 && p->inlet_bc == 2) {
        err = "Inlet pressure + outlet convective BC is not supported";
        return MFLBM_EINVAL;
    }
    if (p->multiphase && (p->mrt < 1 || p->mrt > 4)) { err = "mrt must be 1..4"; return MFLBM_EINVAL; }
    return MFLBM_OK;
}

}  // namespace

// ===================================================================================
// C API of the oracle (mirrors include/mflbm.h with the orc_ prefix)
// ===================================================================================
extern "C" {

int32_t orc_create(const mflbm_params *p, void **out) {
    std::string err;
    int rc = validate(p, err);
    if (rc != MFLBM_OK) { g_create_err = err; return rc; }
    Orc *o = new Orc();
    o->p = *p;
    o->nx = p->nx; o->ny = p->ny; o->nz = p->nz;
    o->mp = p->multiphase != 0;
    const int64_t n1 = o->n1();
    for (int q = 0; q < 19; ++q) {
        o->f[q].assign(n1, 0.0);
        if (o->mp) o->g[q].assign(n1, 0.0);
    }
    o->walls.assign(o->n2(), 0);
    o->curv.assign(n1, 0.0); o->u.assign(n1, 0.0); o->v.assign(n1, 0.0); o->w.assign(n1, 0.0); o->rho.assign(n1, 0.0);
    o->w_in.assign(o->nplane(), 0.0);
    o->fconv.assign(o->nplane() * 19, 0.0);
    if (o->mp) {
        o->phi.assign(o->n4(), 0.0);
        o->cnx.assign(o->n2(), 0.0); o->cny.assign(o->n2(), 0.0); o->cnz.assign(o->n2(), 0.0); o->cnorm.assign(o->n2(), 0.0);
        o->gconv.assign(o->nplane() * 19, 0.0);
        o->phiconv.assign(o->nplane(), 0.0);
    }
    // derived parameters (Init_multiphase.F90:116-128; singlephase Initialization.F90:80-112)
    o->la_nui1 = 1.0 / p->la_nu1;
    o->la_nui2 = o->mp ? 1.0 / p->la_nu2 : 0.0;
    o->phi_inlet = 2.0 * p->sa_inject - 1.0;
    if (!o->mp) {
        const double omega = 1.0 / (3.0 * p->la_nu1 + 0.5);
        o->s_nu = omega;
        if (p->mrt == 1) {
            o->s_e = omega; o->s_e2 = omega; o->s_pi = omega;
            o->s_q = 8.0 * (2.0 - omega) / (8.0 - omega);
            o->s_t = o->s_q;
        } else {
            // Initialization.F90:91-112 tests `== 1` twice, so every other preset is SRT
            o->s_e = omega; o->s_e2 = omega; o->s_pi = omega; o->s_q = omega; o->s_t = omega;
        }
    }
    *out = o;
    return MFLBM_OK;
}

void orc_destroy(void *h) { delete (Orc *)h; }

const char *orc_last_error(void *h) { return h ? ((Orc *)h)->err.c_str() : g_create_err.c_str(); }

int32_t orc_set_geometry(void *h, const int8_t *walls, const mflbm_solid_bnd *s, int32_t ns, const mflbm_fluid_bnd *f,
                         int32_t nf, const double *w_in) {
    Orc *o = (Orc *)h;
    if (!walls) { o->err = "walls is NULL"; return MFLBM_EINVAL; }
    std::memcpy(o->walls.data(), walls, o->walls.size());
    o->sb.assign(s, s + (s ? ns : 0));
    o->fb.assign(f, f + (f ? nf : 0));
    if (w_in) std::memcpy(o->w_in.data(), w_in, sizeof(double) * o->nplane());
    o->geometry = true;
    return MFLBM_OK;
}

int32_t orc_upload_state(void *h, const double *const *f, const double *const *g, const double *phi, const double *fc,
                         const double *gc, const double *pc) {
    Orc *o = (Orc *)h;
    const int64_t n1 = o->n1();
    if (!f) { o->err = "f is NULL"; return MFLBM_EINVAL; }
    for (int q = 0; q < 19; ++q) std::memcpy(o->f[q].data(), f[q], sizeof(double) * n1);
    if (o->mp) {
        if (!g || !phi) { o->err = "g and phi are required for multiphase"; return MFLBM_EINVAL; }
        for (int q = 0; q < 19; ++q) std::memcpy(o->g[q].data(), g[q], sizeof(double) * n1);
        std::memcpy(o->phi.data(), phi, sizeof(double) * o->n4());
    }
    if (fc) std::memcpy(o->fconv.data(), fc, sizeof(double) * o->fconv.size());
    if (o->mp && gc) std::memcpy(o->gconv.data(), gc, sizeof(double) * o->gconv.size());
    if (o->mp && pc) std::memcpy(o->phiconv.data(), pc, sizeof(double) * o->phiconv.size());
    return MFLBM_OK;
}

int32_t orc_download_state(void *h, double *const *f, double *const *g, double *phi, double *fc, double *gc, double *pc) {
    Orc *o = (Orc *)h;
    const int64_t n1 = o->n1();
    if (f) for (int q = 0; q < 19; ++q) if (f[q]) std::memcpy(f[q], o->f[q].data(), sizeof(double) * n1);
    if (o->mp) {
        if (g) for (int q = 0; q < 19; ++q) if (g[q]) std::memcpy(g[q], o->g[q].data(), sizeof(double) * n1);
        if (phi) std::memcpy(phi, o->phi.data(), sizeof(double) * o->n4());
        if (gc) std::memcpy(gc, o->gconv.data(), sizeof(double) * o->gconv.size());
        if (pc) std::memcpy(pc, o->phiconv.data(), sizeof(double) * o->phiconv.size());
    }
    if (fc) std::memcpy(fc, o->fconv.data(), sizeof(double) * o->fconv.size());
    return MFLBM_OK;
}

// initialization_new_multi_pdf / initialization_new_pdf with u = 0, rho = 1
// (Init_multiphase.F90:357-470; singlephase Initialization.F90:240-309)
int32_t orc_init_equilibrium(void *h, const double *phi_in) {
    Orc *o = (Orc *)h;
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    if (o->mp) {
        if (!phi_in) { o->err = "phi is required for multiphase"; return MFLBM_EINVAL; }
        std::memcpy(o->phi.data(), phi_in, sizeof(double) * o->n4());
    }
    for (int k = 0; k <= nz + 1; ++k)
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                const int64_t id = o->I1(i, j, k);
                const double uu = 0.0, vv = 0.0, ww = 0.0, rr = 1.0;
                o->u[id] = uu; o->v[id] = vv; o->w[id] = ww; o->rho[id] = rr;
                const double usqrt = uu * uu + vv * vv + ww * ww;
                const double cu[19] = {0.0, uu, -uu, vv, -vv, ww, -ww, uu + vv, -uu + vv, uu - vv, -uu - vv, uu + ww, -uu + ww,
                                       uu - ww, -uu - ww, vv + ww, -vv + ww, vv - ww, -vv - ww};
                double r[2];
                int nsp = 1;
                if (o->mp) {
                    const double ph = o->PHI(i, j, k);
                    r[0] = rr * (1.0 + ph) * 0.5;
                    r[1] = rr * (1.0 - ph) * 0.5;
                    nsp = 2;
                } else {
                    r[0] = rr;
                }
                for (int s = 0; s < nsp; ++s) {
                    std::vector<double> *A = s == 0 ? o->f : o->g;
                    const double rh = r[s];
                    A[0][id] = rh * w_equ_0 + rh * w_equ_0 * (-1.5 * usqrt);
                    for (int q = 1; q < 19; ++q) {
                        const double wq = q < 7 ? w_equ_1 : w_equ_2;
                        A[q][id] = rh * wq + rh * wq * (3.0 * cu[q] + 4.5 * cu[q] * cu[q] - 1.5 * usqrt);
                    }
                }
            }
    if (o->p.outlet_bc == 1) {
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                for (int q = 0; q < 19; ++q) {
                    o->fconv[o->IC(i, j, q)] = o->f[q][o->I1(i, j, nz)];
                    if (o->mp) o->gconv[o->IC(i, j, q)] = o->g[q][o->I1(i, j, nz)];
                }
                if (o->mp) o->phiconv[o->IP(i, j)] = o->PHI(i, j, nz);
            }
    }
    return MFLBM_OK;
}

int32_t orc_step(void *h, int32_t ntime) {
    Orc *o = (Orc *)h;
    if (!o->geometry) { o->err = "set_geometry must be called before step"; return MFLBM_ESTATE; }
    step(*o, ntime);
    return MFLBM_OK;
}

int32_t orc_run(void *h, int32_t ntime0, int32_t nsteps) {
    for (int32_t t = 0; t < nsteps; ++t) {
        int rc = orc_step(h, ntime0 + t);
        if (rc) return rc;
    }
    return MFLBM_OK;
}

int32_t orc_color_gradient(void *h) {
    Orc *o = (Orc *)h;
    if (!o->mp) { o->err = "color_gradient is multiphase only"; return MFLBM_EINVAL; }
    color_gradient(*o);
    return MFLBM_OK;
}

int32_t orc_get_gradient(void *h, double *cx, double *cy, double *cz, double *cn, double *cv) {
    Orc *o = (Orc *)h;
    if (!o->mp) { o->err = "multiphase only"; return MFLBM_EINVAL; }
    const size_t b2 = sizeof(double) * o->n2();
    if (cx) std::memcpy(cx, o->cnx.data(), b2);
    if (cy) std::memcpy(cy, o->cny.data(), b2);
    if (cz) std::memcpy(cz, o->cnz.data(), b2);
    if (cn) std::memcpy(cn, o->cnorm.data(), b2);
    if (cv) std::memcpy(cv, o->curv.data(), sizeof(double) * o->n1());
    return MFLBM_OK;
}

int32_t orc_macro(void *h, double *u, double *v, double *w, double *rho, double *phi) {
    Orc *o = (Orc *)h;
    macro_vars(*o);
    const size_t b1 = sizeof(double) * o->n1();
    if (u) std::memcpy(u, o->u.data(), b1);
    if (v) std::memcpy(v, o->v.data(), b1);
    if (w) std::memcpy(w, o->w.data(), b1);
    if (rho) std::memcpy(rho, o->rho.data(), b1);
    if (phi && o->mp) std::memcpy(phi, o->phi.data(), sizeof(double) * o->n4());
    return MFLBM_OK;
}

// monitor reductions (multiphase Monitor.F90:27-85; singlephase Monitor.F90:18-59),
// summed in the reference's loop order (k slice, then j, then i)
int32_t orc_monitor(void *h, double *prof, double *scal, int32_t *status) {
    Orc *o = (Orc *)h;
    macro_vars(*o);
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    double umax = 0.0, usq1 = 0.0, usq2 = 0.0;
    bool bad = false;
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const int64_t id = o->I1(i, j, k);
                const int wi = o->WALL(i, j, k);
                double temp;
                if (o->mp) {
                    temp = (o->u[id] * o->u[id] + o->v[id] * o->v[id] + o->w[id] * o->w[id]) * (double)(1 - wi);
                } else {
                    temp = o->u[id] * o->u[id] + o->v[id] * o->v[id] + o->w[id] * o->w[id];
                }
                if (umax < temp) umax = temp;
                if (o->mp) {
                    const double ph = o->PHI(i, j, k);
                    if (ph > 0.999) usq1 = usq1 + temp;
                    else if (ph < -0.999) usq2 = usq2 + temp;
                }
            }
    for (int k = 1; k <= nz; ++k) {
        double t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, prek = 0;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const int64_t id = o->I1(i, j, k);
                const int wi = o->WALL(i, j, k);
                if (o->mp) {
                    const double m = (double)(1 - wi);
                    const double ph = o->PHI(i, j, k);
                    t3 = t3 + 0.5 * (1.0 + ph) * m;
                    t4 = t4 + 0.5 * (1.0 - ph) * m;
                    t5 = t5 + o->rho[id] * 0.5 * (1.0 + ph) * m;
                    t6 = t6 + o->rho[id] * 0.5 * (1.0 - ph) * m;
                    t1 = t1 + o->w[id] * 0.5 * (1.0 + ph) * m;
                    t2 = t2 + o->w[id] * 0.5 * (1.0 - ph) * m;
                    prek = prek + o->rho[id] * m;
                } else {
                    t1 = t1 + o->w[id];
                    prek = prek + o->rho[id];
                }
            }
        if (o->mp) {
            prof[0 * nz + k - 1] = t1; prof[1 * nz + k - 1] = t2; prof[2 * nz + k - 1] = t3; prof[3 * nz + k - 1] = t4;
            prof[4 * nz + k - 1] = t5; prof[5 * nz + k - 1] = t6; prof[6 * nz + k - 1] = prek;
            for (double x : {t1, t2, t3, t4, t5, t6, prek}) if (std::isnan(x)) bad = true;
        } else {
            prof[k - 1] = t1; prof[nz + k - 1] = prek;
            if (std::isnan(t1) || std::isnan(prek)) bad = true;
        }
    }
    scal[0] = umax; scal[1] = usq1; scal[2] = usq2;
    if (std::isnan(umax) || std::sqrt(umax) > 0.5) bad = true;
    if (status) *status = bad ? MFLBM_FAILED : MFLBM_RUNNING;
    return MFLBM_OK;
}

// The other monitors of the multiphase loop (Main_multiphase.F90:184-195), one kind per
// call, with the outputs of mflbm_steady_monitor:
//   kind 0: phi_old <- phi (the set-up of steady_state_option 2, Init_multiphase.F90:340-351)
//   kind 1: monitor_multiphase_steady_capillarypressure (Monitor.F90:370-462):
//           out = pc, pre_w, pre_nw, umax, i_w, i_nw
//   kind 2: monitor_multiphase_steady_phasefield (Monitor.F90:287-365): out = max |phi -
//           phi_old| over the fluid nodes, umax; then phi_old <- phi
//   kind 3: monitor_breakthrough (Monitor.F90:472-507): out = fluid nodes with phi > 0 in
//           the plane obs_z = nz - 1
// umax is the square root of the largest |u|^2 over the fluid nodes.  The sums run in the
// reference's loop order (k, then j, then i).
int32_t orc_steady_monitor(void *h, int32_t kind, double *out) {
    Orc *o = (Orc *)h;
    if (!o->mp) { o->err = "steady-state monitors are multiphase"; return MFLBM_EINVAL; }
    if (kind < 0 || kind > 3 || (kind > 0 && !out)) { o->err = "kind must be 0..3 and out non-NULL"; return MFLBM_EINVAL; }
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    static const double eps = 1.110223025e-16;   // Misc_module eps (Module.F90:8)
    if (kind == 0 || o->phi_old.empty()) {
        o->phi_old = o->phi;
        if (kind == 0) return MFLBM_OK;
    }
    if (kind == 3) {
        const int obs_z = nz - 1;
        int itemp = 0;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                if (o->WALL(i, j, obs_z) == 0 && o->PHI(i, j, obs_z) > 0.0) itemp = itemp + 1;
        out[0] = (double)itemp;
        return MFLBM_OK;
    }
    macro_vars(*o);
    double umax = 0.0, d_phi_max = 0.0;
    double pre_w = 0.0, pre_nw = 0.0;
    int i_w = 0, i_nw = 0;
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const int64_t id = o->I1(i, j, k), i4 = o->I4(i, j, k);
                const int wi = o->WALL(i, j, k);
                const double tmp1 = (o->u[id] * o->u[id] + o->v[id] * o->v[id] + o->w[id] * o->w[id]) * (double)(1 - wi);
                if (umax < tmp1) umax = tmp1;
                if (kind == 2) {
                    const double tmp2 = std::fabs(o->phi[i4] - o->phi_old[i4]) * (double)(1 - wi);
                    if (d_phi_max < tmp2) d_phi_max = tmp2;
                } else if (wi == 0) {
                    if (o->phi[i4] < -0.99) { pre_w = pre_w + o->rho[id]; i_w = i_w + 1; }
                    if (o->phi[i4] > 0.99) { pre_nw = pre_nw + o->rho[id]; i_nw = i_nw + 1; }
                }
            }
    if (kind == 2) {
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) o->phi_old[o->I4(i, j, k)] = o->PHI(i, j, k);
        out[0] = d_phi_max;
        out[1] = std::sqrt(umax);
        return MFLBM_OK;
    }
    const double pw = pre_w / ((double)i_w + eps), pnw = pre_nw / ((double)i_nw + eps);
    out[0] = (pnw - pw) / 3.0;
    out[1] = pw;
    out[2] = pnw;
    out[3] = std::sqrt(umax);
    out[4] = (double)i_w;
    out[5] = (double)i_nw;
    return MFLBM_OK;
}

// change_inlet_fluid_phase (multiphase_3D/0.src/Misc.F90:507-621) for one rank: every
// slot of the halo-1 box (k = 1-overlap .. nz+overlap, overlap = 1) with z = k <=
// interface_z0; cmd 1: f = f + g, g = 0; cmd 2: g = f + g, f = 0.
int32_t orc_change_inlet_fluid_phase(void *h, int32_t cmd, double interface_z0) {
    Orc *o = (Orc *)h;
    if (!o->mp) { o->err = "change_inlet_fluid_phase is multiphase only"; return MFLBM_EINVAL; }
    if (cmd < 0 || cmd > 2) { o->err = "change_inlet_fluid_phase_cmd must be 0, 1 or 2"; return MFLBM_EINVAL; }
    for (int k = 0; k <= o->nz + 1; ++k)
        for (int j = 0; j <= o->ny + 1; ++j)
            for (int i = 0; i <= o->nx + 1; ++i) {
                const int z = k;
                if (!((double)z <= interface_z0)) continue;
                const int64_t id = o->I1(i, j, k);
                for (int q = 0; q < 19; ++q) {
                    if (cmd == 1) {
                        o->f[q][id] = o->f[q][id] + o->g[q][id];
                        o->g[q][id] = 0.0;
                    } else if (cmd == 2) {
                        o->g[q][id] = o->f[q][id] + o->g[q][id];
                        o->f[q][id] = 0.0;
                    }
                }
            }
    return MFLBM_OK;
}

// cal_saturation (Monitor.F90:512-550), sequential order
int32_t orc_saturation(void *h, double *vol1, double *vol2) {
    Orc *o = (Orc *)h;
    double v1 = 0.0, v2 = 0.0;
    for (int k = 1; k <= o->nz; ++k)
        for (int j = 1; j <= o->ny; ++j)
            for (int i = 1; i <= o->nx; ++i) {
                const double m = (double)(1 - o->WALL(i, j, k));
                const double ph = o->PHI(i, j, k);
                v1 = v1 + 0.5 * (1.0 + ph) * m;
                v2 = v2 + 0.5 * (1.0 - ph) * m;
            }
    *vol1 = v1; *vol2 = v2;
    return MFLBM_OK;
}

int32_t orc_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// ------------------------------------------------------------------------------------
// Host-side setup restatements used to build oracle inputs.
// ------------------------------------------------------------------------------------

// set_walls for one rank (multiphase_3D/0.src/Misc.F90:6-210 incl. the halo transports
// of Mpi_misc.F90:337-502): walls_global (nx*ny*nz, values 0/1, channel walls not yet
// applied) -> walls with halo 2.  Returns pore_sum.
int64_t orc_set_walls(const mflbm_params *p, const int8_t *walls_global, int8_t *walls_out) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    std::vector<int8_t> wg(walls_global, walls_global + (size_t)nx * ny * nz);
    auto G = [&](int i, int j, int k) -> int8_t & { return wg[(size_t)(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1))]; };
    // channel walls on the global array (:90-109)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                if (p->wall_z_min == 1) G(i, j, 1) = 1;
                if (p->wall_z_max == 1) G(i, j, nz) = 1;
                if (p->wall_x_min == 1) G(1, j, k) = 1;
                if (p->wall_x_max == 1) G(nx, j, k) = 1;
                if (p->wall_y_min == 1) G(i, 1, k) = 1;
                if (p->wall_y_max == 1) G(i, ny, k) = 1;
            }
    const int64_t nxh = nx + 4, nyh = ny + 4;
    auto W = [&](int i, int j, int k) -> int8_t & { return walls_out[(i + 1) + nxh * ((j + 1) + nyh * (int64_t)(k + 1))]; };
    std::memset(walls_out, 0, (size_t)(nx + 4) * (ny + 4) * (nz + 4));
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) W(i, j, k) = G(i, j, k);
    // local channel walls incl. halo (:147-191)
    for (int k = -1; k <= nz + 2; ++k)
        for (int j = -1; j <= ny + 2; ++j)
            for (int i = -1; i <= nx + 2; ++i) {
                if (k <= 1 && p->wall_z_min == 1) W(i, j, k) = 1;
                if (k >= nz && p->wall_z_max == 1) W(i, j, k) = 1;
                if (i <= 1 && p->wall_x_min == 1) W(i, j, k) = 1;
                if (i >= nx && p->wall_x_max == 1) W(i, j, k) = 1;
                if (j <= 1 && p->wall_y_min == 1) W(i, j, k) = 1;
                if (j >= ny && p->wall_y_max == 1) W(i, j, k) = 1;
            }
    // ztransport_walls(0,0,2), ytransport_walls(0,2,2), xtransport_walls(2,2,2)
    if (p->kper == 1)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                for (int kk = 1; kk <= 2; ++kk) {
                    W(i, j, kk - 2) = W(i, j, nz + kk - 2);
                    W(i, j, nz + kk) = W(i, j, kk);
                }
    if (p->jper == 1)
        for (int k = -1; k <= nz + 2; ++k)
            for (int i = 1; i <= nx; ++i)
                for (int jj = 1; jj <= 2; ++jj) {
                    W(i, jj - 2, k) = W(i, ny + jj - 2, k);
                    W(i, ny + jj, k) = W(i, jj, k);
                }
    if (p->iper == 1)
        for (int k = -1; k <= nz + 2; ++k)
            for (int j = -1; j <= ny + 2; ++j)
                for (int ii = 1; ii <= 2; ++ii) {
                    W(ii - 2, j, k) = W(nx + ii - 2, j, k);
                    W(nx + ii, j, k) = W(ii, j, k);
                }
    int64_t pore = 0;
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                if (W(i, j, k) <= 0) ++pore;
    return pore;
}

// geometry_preprocessing_new for one rank (Geometry_preprocessing.F90:9-512).
// walls_channel: the global wall array after channel walls (nx*ny*nz, 0/1).
// Two-pass use: call with solid/fluid NULL to get the counts, then with buffers.
int32_t orc_geometry_preprocess(const mflbm_params *p, const int8_t *walls_channel, double theta_rad,
                                mflbm_solid_bnd *solid, int32_t *n_solid, mflbm_fluid_bnd *fluid, int32_t *n_fluid) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int gl = 6 + 4;  // ghost_layers = 6 + overlap_phi
    const int64_t sx = nx + 2 * gl, sy = ny + 2 * gl, sz = nz + 2 * gl;
    std::vector<int8_t> wt((size_t)(sx * sy * sz), 0);
    auto T = [&](int i, int j, int k) -> int8_t & { return wt[(size_t)((i - 1 + gl) + sx * ((j - 1 + gl) + sy * (int64_t)(k - 1 + gl)))]; };
    auto Wg = [&](int i, int j, int k) { return walls_channel[(size_t)(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1))]; };
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) T(i, j, k) = Wg(i, j, k);
    // ghost fill (:56-108)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
            for (int g = 1; g <= gl; ++g) {
                if (p->kper == 0) { T(i, j, 1 - g) = T(i, j, 1); T(i, j, nz + g) = T(i, j, nz); }
            }
    // periodic fills are Fortran array assignments: the right-hand side is read in
    // full before any element is stored, which matters when n < ghost_layers
    std::vector<int8_t> tmpv((size_t)2 * gl);
    if (p->kper != 0) {
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                for (int g = 0; g < gl; ++g) { tmpv[g] = T(i, j, nz - gl + 1 + g); tmpv[gl + g] = T(i, j, 1 + g); }
                for (int g = 0; g < gl; ++g) { T(i, j, 1 - gl + g) = tmpv[g]; T(i, j, nz + 1 + g) = tmpv[gl + g]; }
            }
    }
    for (int k = 1 - gl; k <= nz + gl; ++k)
        for (int i = 1; i <= nx; ++i) {
            if (p->jper == 0) {
                for (int g = 1; g <= gl; ++g) { T(i, 1 - g, k) = T(i, 1, k); T(i, ny + g, k) = T(i, ny, k); }
            } else {
                for (int g = 0; g < gl; ++g) { tmpv[g] = T(i, ny - gl + 1 + g, k); tmpv[gl + g] = T(i, 1 + g, k); }
                for (int g = 0; g < gl; ++g) { T(i, 1 - gl + g, k) = tmpv[g]; T(i, ny + 1 + g, k) = tmpv[gl + g]; }
            }
        }
    for (int k = 1 - gl; k <= nz + gl; ++k)
        for (int j = 1 - gl; j <= ny + gl; ++j) {
            if (p->iper == 0) {
                for (int g = 1; g <= gl; ++g) { T(1 - g, j, k) = T(1, j, k); T(nx + g, j, k) = T(nx, j, k); }
            } else {
                for (int g = 0; g < gl; ++g) { tmpv[g] = T(nx - gl + 1 + g, j, k); tmpv[gl + g] = T(1 + g, j, k); }
                for (int g = 0; g < gl; ++g) { T(1 - gl + g, j, k) = tmpv[g]; T(nx + 1 + g, j, k) = tmpv[gl + g]; }
            }
        }
    std::vector<double> s1((size_t)(sx * sy * sz)), s2((size_t)(sx * sy * sz));
    auto S1 = [&](int i, int j, int k) -> double & { return s1[(size_t)((i - 1 + gl) + sx * ((j - 1 + gl) + sy * (int64_t)(k - 1 + gl)))]; };
    auto S2 = [&](int i, int j, int k) -> double & { return s2[(size_t)((i - 1 + gl) + sx * ((j - 1 + gl) + sy * (int64_t)(k - 1 + gl)))]; };
    for (size_t n = 0; n < wt.size(); ++n) { s1[n] = wt[n]; s2[n] = wt[n]; }
    // classification (:121-143); the in-place update does not change any predicate
    for (int k = 2 - gl; k <= nz + gl - 1; ++k)
        for (int j = 2 - gl; j <= ny + gl - 1; ++j)
            for (int i = 2 - gl; i <= nx + gl - 1; ++i) {
                if (T(i, j, k) == 1) {
                    for (int n = 1; n <= 18; ++n)
                        if (T(i + ex[n], j + ey[n], k + ez[n]) <= 0) { T(i, j, k) = 2; break; }
                }
                if (T(i, j, k) == 0) {
                    for (int n = 1; n <= 18; ++n)
                        if (T(i + ex[n], j + ey[n], k + ez[n]) >= 1) { T(i, j, k) = -1; break; }
                }
            }
    // 27-point smoothing, 4 iterations (:145-169)
    static const int iex[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    static const int iey[27] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
    static const int iez[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1};
    const double we[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};
    for (int it = 0; it < 4; ++it) {
#pragma omp parallel for schedule(static)
        for (int k = 2 - gl; k <= nz + gl - 1; ++k)
            for (int j = 2 - gl; j <= ny + gl - 1; ++j)
                for (int i = 2 - gl; i <= nx + gl - 1; ++i) {
                    double acc = 0.0;
                    for (int n = 0; n < 27; ++n) {
                        const int m = iex[n] * iex[n] + iey[n] * iey[n] + iez[n] * iez[n];
                        acc = acc + S1(i + iex[n], j + iey[n], k + iez[n]) * we[m];
                    }
                    S2(i, j, k) = acc;
                }
#pragma omp parallel for schedule(static)
        for (int k = 2 - gl; k <= nz + gl - 1; ++k)
            for (int j = 2 - gl; j <= ny + gl - 1; ++j)
                for (int i = 2 - gl; i <= nx + gl - 1; ++i) S1(i, j, k) = S2(i, j, k);
    }
    // lists over [1-4, n+4] (:171-225), local filters (:429-507)
    int32_t cs = 0, cf = 0;
    const double ISO8[7] = {4.0 / 45.0, 1.0 / 21.0, 2.0 / 105.0, 5.0 / 504.0, 1.0 / 315.0, 1.0 / 630.0, 1.0 / 5040.0};
    for (int k = -3; k <= nz + 4; ++k)
        for (int j = -3; j <= ny + 4; ++j)
            for (int i = -3; i <= nx + 4; ++i) {
                const int8_t c = T(i, j, k);
                if (c == 2 && i >= -2 && i <= nx + 3 && j >= -2 && j <= ny + 3 && k >= -2 && k <= nz + 3) {
                    if (solid) {
                        mflbm_solid_bnd &s = solid[cs];
                        std::memset(&s, 0, sizeof(s));
                        s.ix = i; s.iy = j; s.iz = k;
                        int ncount = 0;
                        double lw = 0.0;
                        for (int n = 1; n <= 18; ++n)
                            if (T(i + ex[n], j + ey[n], k + ez[n]) <= 0) {
                                ncount = ncount + 1;
                                lw = lw + w_equ[n];
                                s.neighbor_list[ncount - 1] = n;
                            }
                        s.la_weight = lw;
                        s.i_fluid_num = ncount;
                    }
                    ++cs;
                }
                if (c == -1 && i >= -1 && i <= nx + 2 && j >= -1 && j <= ny + 2 && k >= -1 && k <= nz + 2) {
                    if (fluid) {
                        auto S = [&](int a, int b, int cc) { return S2(i + a, j + b, k + cc); };
                        const double nwx =
                            ISO8[0] * (S(1, 0, 0) - S(-1, 0, 0)) +
                            ISO8[1] * (S(1, 1, 0) - S(-1, -1, 0) + S(1, -1, 0) - S(-1, 1, 0) + S(1, 0, 1) - S(-1, 0, -1) + S(1, 0, -1) - S(-1, 0, 1)) +
                            ISO8[2] * (S(1, 1, 1) - S(-1, -1, -1) + S(1, 1, -1) - S(-1, -1, 1) + S(1, -1, 1) - S(-1, 1, -1) + S(1, -1, -1) - S(-1, 1, 1)) +
                            ISO8[3] * (S(2, 0, 0) - S(-2, 0, 0)) +
                            ISO8[4] * (S(2, 1, 0) - S(-2, -1, 0) + S(2, -1, 0) - S(-2, 1, 0) + S(2, 0, 1) - S(-2, 0, -1) + S(2, 0, -1) - S(-2, 0, 1) +
                                       S(1, 2, 0) - S(-1, -2, 0) + S(1, -2, 0) - S(-1, 2, 0) + S(1, 0, 2) - S(-1, 0, -2) + S(1, 0, -2) - S(-1, 0, 2)) +
                            ISO8[5] * (S(2, 1, 1) - S(-2, -1, -1) + S(2, 1, -1) - S(-2, -1, 1) + S(2, -1, 1) - S(-2, 1, -1) + S(2, -1, -1) - S(-2, 1, 1) +
                                       S(1, 2, 1) - S(-1, -2, -1) + S(1, 2, -1) - S(-1, -2, 1) + S(1, -2, 1) - S(-1, 2, -1) + S(1, -2, -1) - S(-1, 2, 1) +
                                       S(1, 1, 2) - S(-1, -1, -2) + S(1, 1, -2) - S(-1, -1, 2) + S(1, -1, 2) - S(-1, 1, -2) + S(1, -1, -2) - S(-1, 1, 2)) +
                            ISO8[6] * (S(2, 2, 0) - S(-2, -2, 0) + S(2, -2, 0) - S(-2, 2, 0) + S(2, 0, 2) - S(-2, 0, -2) + S(2, 0, -2) - S(-2, 0, 2));
                        const double nwy =
                            ISO8[0] * (S(0, 1, 0) - S(0, -1, 0)) +
                            ISO8[1] * (S(1, 1, 0) - S(-1, -1, 0) + S(-1, 1, 0) - S(1, -1, 0) + S(0, 1, 1) - S(0, -1, -1) + S(0, 1, -1) - S(0, -1, 1)) +
                            ISO8[2] * (S(1, 1, 1) - S(-1, -1, -1) + S(1, 1, -1) - S(-1, -1, 1) + S(-1, 1, -1) - S(1, -1, 1) + S(-1, 1, 1) - S(1, -1, -1)) +
                            ISO8[3] * (S(0, 2, 0) - S(0, -2, 0)) +
                            ISO8[4] * (S(2, 1, 0) - S(-2, -1, 0) + S(-2, 1, 0) - S(2, -1, 0) + S(0, 2, 1) - S(0, -2, -1) + S(0, 2, -1) - S(0, -2, 1) +
                                       S(1, 2, 0) - S(-1, -2, 0) + S(-1, 2, 0) - S(1, -2, 0) + S(0, 1, 2) - S(0, -1, -2) + S(0, 1, -2) - S(0, -1, 2)) +
                            ISO8[5] * (S(2, 1, 1) - S(-2, -1, -1) + S(2, 1, -1) - S(-2, -1, 1) + S(-2, 1, 1) - S(2, -1, -1) + S(-2, 1, -1) - S(2, -1, 1) +
                                       S(1, 2, 1) - S(-1, -2, -1) + S(1, 2, -1) - S(-1, -2, 1) + S(-1, 2, 1) - S(1, -2, -1) + S(-1, 2, -1) - S(1, -2, 1) +
                                       S(1, 1, 2) - S(-1, -1, -2) + S(1, 1, -2) - S(-1, -1, 2) + S(-1, 1, 2) - S(1, -1, -2) + S(-1, 1, -2) - S(1, -1, 2)) +
                            ISO8[6] * (S(2, 2, 0) - S(-2, -2, 0) + S(-2, 2, 0) - S(2, -2, 0) + S(0, 2, 2) - S(0, -2, -2) + S(0, 2, -2) - S(0, -2, 2));
                        const double nwz =
                            ISO8[0] * (S(0, 0, 1) - S(0, 0, -1)) +
                            ISO8[1] * (S(0, 1, 1) - S(0, -1, -1) + S(0, -1, 1) - S(0, 1, -1) + S(1, 0, 1) - S(-1, 0, -1) + S(-1, 0, 1) - S(1, 0, -1)) +
                            ISO8[2] * (S(1, 1, 1) - S(-1, -1, -1) + S(1, -1, 1) - S(-1, 1, -1) + S(-1, 1, 1) - S(1, -1, -1) + S(-1, -1, 1) - S(1, 1, -1)) +
                            ISO8[3] * (S(0, 0, 2) - S(0, 0, -2)) +
                            ISO8[4] * (S(0, 1, 2) - S(0, -1, -2) + S(0, -1, 2) - S(0, 1, -2) + S(2, 0, 1) - S(-2, 0, -1) + S(-2, 0, 1) - S(2, 0, -1) +
                                       S(0, 2, 1) - S(0, -2, -1) + S(0, -2, 1) - S(0, 2, -1) + S(1, 0, 2) - S(-1, 0, -2) + S(-1, 0, 2) - S(1, 0, -2)) +
                            ISO8[5] * (S(2, 1, 1) - S(-2, -1, -1) + S(2, -1, 1) - S(-2, 1, -1) + S(-2, 1, 1) - S(2, -1, -1) + S(-2, -1, 1) - S(2, 1, -1) +
                                       S(1, 2, 1) - S(-1, -2, -1) + S(1, -2, 1) - S(-1, 2, -1) + S(-1, 2, 1) - S(1, -2, -1) + S(-1, -2, 1) - S(1, 2, -1) +
                                       S(1, 1, 2) - S(-1, -1, -2) + S(1, -1, 2) - S(-1, 1, -2) + S(-1, 1, 2) - S(1, -1, -2) + S(-1, -1, 2) - S(1, 1, -2)) +
                            ISO8[6] * (S(0, 2, 2) - S(0, -2, -2) + S(0, -2, 2) - S(0, 2, -2) + S(2, 0, 2) - S(-2, 0, -2) + S(-2, 0, 2) - S(2, 0, -2));
                        const double tmp = 1.0 / (std::sqrt(nwx * nwx + nwy * nwy + nwz * nwz) + eps14);
                        mflbm_fluid_bnd &fb = fluid[cf];
                        std::memset(&fb, 0, sizeof(fb));
                        fb.ix = i; fb.iy = j; fb.iz = k;
                        fb.nwx = nwx * tmp; fb.nwy = nwy * tmp; fb.nwz = nwz * tmp;
                        fb.theta = theta_rad;
                    }
                    ++cf;
                }
            }
    if (n_solid) *n_solid = cs;
    if (n_fluid) *n_fluid = cf;
    return MFLBM_OK;
}

// inlet_vel_profile_rectangular (multiphase_3D/0.src/Misc.F90:625-665) for one rank,
// w_in is (0:nx+1, 0:ny+1); la_x = nx-2, la_y = ny-2 (Init_multiphase.F90:71-74).
// The Fortran `n**5` and `n**3` are default-integer powers; n**5 wraps for n >= 75
// in 32-bit two's complement, which is restated here so the series is the same.
void orc_inlet_profile(int32_t nx, int32_t ny, double vel_avg, int32_t num_terms, double *w_in) {
    const double pi = 3.14159265358979323846;
    const double la_x = (double)nx - 1.0 - 0.5 - 0.5;
    const double la_y = (double)ny - 1.0 - 0.5 - 0.5;
    const double a = 0.5 * la_x, b = 0.5 * la_y;
    auto ipow = [](int32_t n, int e) -> int32_t {
        uint32_t r = 1;
        for (int t = 0; t < e; ++t) r = r * (uint32_t)n;
        return (int32_t)r;
    };
    double tmp1 = 0.0;
    for (int n = 1; n <= num_terms; n += 2) tmp1 = tmp1 + (std::tanh(0.5 * (double)n * pi * b / a)) / (double)ipow(n, 5);
    // pi**5 as an integer power: binary powering, (pi^2)^2 * pi
    const double pi2 = pi * pi;
    const double pi5 = (pi2 * pi2) * pi;
    double tmp2 = 1.0 - 192.0 / pi5 * (a / b) * tmp1;
    tmp2 = -3.0 * vel_avg / (tmp2 * (a * a));
    for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i) w_in[i + (int64_t)(nx + 2) * j] = 0.0;
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const int x = i, y = j;
            if (x > 1 && x < nx && y > 1 && y < ny) {
                const double xx = x - 1.5 - a;
                const double yy = y - 1.5 - b;
                double tmp3 = 0.0;
                for (int n = 1; n <= num_terms; n += 2) {
                    tmp3 = tmp3 + std::pow(-1.0, 0.5 * (double)(n - 1)) * std::cos(0.5 * n * pi * xx / a) / (double)ipow(n, 3) *
                                      (1.0 - (std::exp(0.5 * n * pi * (yy - b) / a) + std::exp(0.5 * n * pi * (-yy - b) / a)) /
                                                 (1.0 + std::exp(0.5 * n * pi * (-b - b) / a)));
                }
                w_in[i + (int64_t)(nx + 2) * j] = tmp3 * (-16.0 * tmp2 * (a * a) * (1.0 / (pi * pi * pi)));
            }
        }
}

}  // extern "C"
