// common.cuh -- device-side data layout shared by the kernels and the C-ABI layer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include "ffloat.cuh"

namespace mflbm {

// D3Q19 lattice, multiphase_3D/0.src/Module.F90:111-114.  Used with compile-time q
// (fully unrolled loops), so every call folds to a constant.
__host__ __device__ constexpr int EX(int q) {
    return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int EY(int q) {
    return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int EZ(int q) {
    return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
         : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
// opposite direction (opc, Module.F90:114)
__host__ __device__ constexpr int OPP(int q) {
    return q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 4 : q == 4 ? 3 : q == 5 ? 6 : q == 6 ? 5
         : q == 7 ? 10 : q == 8 ? 9 : q == 9 ? 8 : q == 10 ? 7
         : q == 11 ? 14 : q == 12 ? 13 : q == 13 ? 12 : q == 14 ? 11
         : q == 15 ? 18 : q == 16 ? 17 : q == 17 ? 16 : q == 18 ? 15 : 0;
}
static_assert(OPP(9) == 8 && OPP(17) == 16 && OPP(0) == 0, "opposite table");
static_assert(EX(OPP(13)) == -EX(13) && EZ(OPP(13)) == -EZ(13), "opposite table");

// Device layout of the PDF arrays.
// Each direction q is one SoA plane over the halo-1 box i,j,k in [0, n+1].  Rows are
// padded so that interior node i=1 starts on a 32-byte boundary for every storage type:
//   element(q,i,j,k) = q*qs + (i + xo) + pitch*j + pz*k,   pz = pitch*(ny+2)
struct Layout {
    int nx, ny, nz;
    int xo;          // element offset of i=0 inside a row
    int64_t pitch;   // row pitch in elements
    int64_t pz;      // plane pitch in elements
    int64_t qs;      // direction stride in elements
    // Fortran-layout strides of the auxiliary arrays
    int64_t h1x, h1xy;   // halo 1:  (nx+2), (nx+2)(ny+2)
    int64_t h2x, h2xy;   // halo 2:  (nx+4), (nx+4)(ny+4)
    int64_t h4x, h4xy;   // halo 4:  (nx+8), (nx+8)(ny+8)

    __host__ __device__ __forceinline__ int64_t cell(int i, int j, int k) const {
        return (int64_t)(i + xo) + pitch * j + pz * k;
    }
    __host__ __device__ __forceinline__ int64_t i1(int i, int j, int k) const { return (int64_t)i + h1x * j + h1xy * k; }
    __host__ __device__ __forceinline__ int64_t i2(int i, int j, int k) const {
        return (int64_t)(i + 1) + h2x * (j + 1) + h2xy * (k + 1);
    }
    __host__ __device__ __forceinline__ int64_t i4(int i, int j, int k) const {
        return (int64_t)(i + 3) + h4x * (j + 3) + h4xy * (k + 3);
    }
    __host__ __device__ __forceinline__ int64_t ip(int i, int j) const { return (int64_t)i + h1x * j; }
    __host__ __device__ __forceinline__ int64_t ic(int i, int j, int q) const { return (int64_t)i + h1x * j + h1xy * q; }
};

// Where population q of the halo-1 cell (i, j, k) is stored, for the kernels that address
// PDFs by cell (boundary conditions, monitor, initialisation): the dense planes (map ==
// nullptr, qs = Layout::qs) or the multiphase fluid list (map: slot of every halo-1 cell,
// >= 0 owned, <= -2 the periodic image's slot -m-2, -1 none; qs = the list stride).
struct PdfAt {
    int64_t qs;
    const int32_t *map;
    int64_t spare;     // list: the slot of cells that have none (never read for a value)
    __host__ __device__ __forceinline__ int64_t slot(const Layout &L, int i, int j, int k) const {
        if (!map) return L.cell(i, j, k);
        const int32_t m = map[L.i1(i, j, k)];
        return m >= 0 ? (int64_t)m : (m <= -2 ? (int64_t)(-m - 2) : spare);
    }
    // the cell owns its slot (dense: every cell)
    __host__ __device__ __forceinline__ bool owned(const Layout &L, int i, int j, int k) const {
        return !map || map[L.i1(i, j, k)] >= 0;
    }
    __host__ __device__ __forceinline__ int64_t operator()(const Layout &L, int q, int i, int j, int k) const {
        return (int64_t)q * qs + slot(L, i, j, k);
    }
};

// Parameters read by the per-step kernels.
struct StepParams {
    double force_z;
    double gamma, beta;
    double la_nui1, la_nui2;
    double sa_inject, phi_inlet;
    double uin_avg, rho_in, rho_out, relaxation;
    double s_e, s_e2, s_q, s_nu, s_pi, s_t;  // singlephase MRT rates
    int mrt;                                 // multiphase `mrt` switch
    int porous_plate_cmd, z_porous_plate;
    int iper, jper, kper;
};

// One fluid-boundary node on the device: the host evaluates cos/sin of the local
// contact angle once, so every step reuses them.
struct FluidBnd {
    int ix, iy, iz, pad;
    double nwx, nwy, nwz, cos_t, sin_t;
};

// The colour-gradient normal of one halo-2 cell (the reference's cn_x, cn_y, cn_z, c_norm
// arrays, Phase_gradient.F90:33-79) as one record: unit normal (x, y, z) and |grad phi| (n).
// A stencil gathers a neighbour with one 16-byte load (FP32; two in FP64) instead of three
// or four scalar loads from separate arrays.
template <class T>
struct alignas(4 * sizeof(T)) Nrm {
    T x, y, z, n;
};

struct SolidBnd {  // identical to mflbm_solid_bnd (96 bytes)
    int ix, iy, iz, i_fluid_num;
    int nbr[18];
    double la_weight;
};

// A cell of the halo-2 neighbourhood [-2, 2045] x [-2, 2045] x [-2, 1021] packed in 32 bits
// (device lists of the multiphase colour-gradient kernels)
__host__ __device__ constexpr uint32_t pack_cell(int i, int j, int k) {
    return (uint32_t)(i + 2) | ((uint32_t)(j + 2) << 11) | ((uint32_t)(k + 2) << 22);
}
__host__ __device__ __forceinline__ void unpack_cell(uint32_t c, int &i, int &j, int &k) {
    i = (int)(c & 0x7ffu) - 2;
    j = (int)((c >> 11) & 0x7ffu) - 2;
    k = (int)(c >> 22) - 2;
}
__host__ __device__ constexpr bool cell_packable(int nx, int ny, int nz) {
    return nx + 5 <= 2047 && ny + 5 <= 2047 && nz + 5 <= 1023;
}

// run constants of the double-word multiphase collision, split once on the host
struct MpConstFF {
    ff half_gamma;   // 0.5 * gamma
    ff force_z;
    ff nui1, nui2;   // 1 / la_nu1, 1 / la_nu2
    ff beta;
    ff w1_tmp_scale; // w_equ_1 (the recolouring weight of the axis directions)
    ff rkw2;         // 1 / sqrt(2) / 36 (the diagonal directions)
};

// compact solid-boundary record: packed cell, bit (d-1) set for every fluid-neighbour
// direction d, and the record's la_weight (16 bytes)
struct SolidBndC {
    uint32_t ijk;
    uint32_t mask;
    double la_weight;
};

// Folded MRT coefficients (see mrt_collide_pairs in kernels.cuh): every post-collision
// moment, already divided by its back-transform norm, is a linear combination of the
// pre-collision moment, its equilibrium term and its forcing term.
template <class R> struct MrtFold {
    R e_m, e_den, e_u2, e_f;   // e'   (/2394)
    R e2_m, e2_u2, e2_f;       // e2'  (/252)
    R q_m, q_u, q_f;           // q'   (/40)
    R x3_m, x3_eq, x3_f;       // 3pxx'  (/36)
    R xi_m, xi_f;              // 3pixx' (/72)
    R w_m, w_eq, w_f;          // pww'   (/12)
    R wi_m, wi_f;              // piww'  (/24)
    R o_m, o_eq, o_f;          // pxy', pyz', pzx' (/4)
    R t_m;                     // t'     (/8)
    R fz;                      // body force along z (singlephase)
};

// the fold's non-conserved even-order moment coefficients all vanish (s_e = s_e2 =
// s_pi = s_nu = 1), so the collision may skip those moments
template <class R> inline bool fold_is_unit(const MrtFold<R> &c) {
    return c.e_m == R(0) && c.e2_m == R(0) && c.x3_m == R(0) && c.xi_m == R(0) && c.w_m == R(0) && c.wi_m == R(0) &&
           c.o_m == R(0);
}

template <class R>
__host__ __device__ __forceinline__ MrtFold<R> fold_rates(double s_e, double s_e2, double s_q, double s_nu, double s_pi,
                                                          double s_t) {
    MrtFold<R> c;
    c.e_m = R((1.0 - s_e) / 2394.0);
    c.e_den = R(-11.0 * s_e / 2394.0);
    c.e_u2 = R(19.0 * s_e / 2394.0);
    c.e_f = R((38.0 - 19.0 * s_e) / 2394.0);
    c.e2_m = R((1.0 - s_e2) / 252.0);
    c.e2_u2 = R(s_e2 * (-475.0 / 63.0) / 252.0);
    c.e2_f = R((-11.0 + 5.5 * s_e2) / 252.0);
    c.q_m = R((1.0 - s_q) / 40.0);
    c.q_u = R(s_q * (-2.0 / 3.0) / 40.0);
    c.q_f = R((-2.0 / 3.0 + s_q / 3.0) / 40.0);
    c.x3_m = R((1.0 - s_nu) / 36.0);
    c.x3_eq = R(s_nu / 36.0);
    c.x3_f = R((2.0 - s_nu) / 36.0);
    c.xi_m = R((1.0 - s_pi) / 72.0);
    c.xi_f = R((1.0 - 0.5 * s_pi) / 72.0);
    c.w_m = R((1.0 - s_nu) / 12.0);
    c.w_eq = R(s_nu / 12.0);
    c.w_f = R((2.0 - s_nu) / 12.0);
    c.wi_m = R((1.0 - s_pi) / 24.0);
    c.wi_f = R((1.0 - 0.5 * s_pi) / 24.0);
    c.o_m = R((1.0 - s_nu) / 4.0);
    c.o_eq = R(s_nu / 4.0);
    c.o_f = R((1.0 - 0.5 * s_nu) / 4.0);
    c.t_m = R((1.0 - s_t) / 8.0);
    c.fz = R(0.0);
    return c;
}

// an FP64 fold as double words (host)
inline MrtFold<ff> fold_to_ff(const MrtFold<double> &d) {
    MrtFold<ff> c;
    c.e_m = ff(d.e_m); c.e_den = ff(d.e_den); c.e_u2 = ff(d.e_u2); c.e_f = ff(d.e_f);
    c.e2_m = ff(d.e2_m); c.e2_u2 = ff(d.e2_u2); c.e2_f = ff(d.e2_f);
    c.q_m = ff(d.q_m); c.q_u = ff(d.q_u); c.q_f = ff(d.q_f);
    c.x3_m = ff(d.x3_m); c.x3_eq = ff(d.x3_eq); c.x3_f = ff(d.x3_f);
    c.xi_m = ff(d.xi_m); c.xi_f = ff(d.xi_f);
    c.w_m = ff(d.w_m); c.w_eq = ff(d.w_eq); c.w_f = ff(d.w_f);
    c.wi_m = ff(d.wi_m); c.wi_f = ff(d.wi_f);
    c.o_m = ff(d.o_m); c.o_eq = ff(d.o_eq); c.o_f = ff(d.o_f);
    c.t_m = ff(d.t_m);
    c.fz = ff(d.fz);
    return c;
}

// The same fold evaluated in the arithmetic type R, for the per-node rates of the
// multiphase collision (omega depends on phi).  Divisions by the constant norms are
// multiplications by their reciprocals (default build only; a division costs about ten
// FP64 instructions), and a caller passing literal rates gets them constant-folded.
template <class R>
__device__ __forceinline__ MrtFold<R> fold_rates_dev(R s_e, R s_e2, R s_q, R s_nu, R s_pi, R s_t) {
    MrtFold<R> c;
    const R n_e = R(1.0 / 2394.0), n_e2 = R(1.0 / 252.0), n_q = R(1.0 / 40.0), n_x3 = R(1.0 / 36.0);
    const R n_xi = R(1.0 / 72.0), n_w = R(1.0 / 12.0), n_wi = R(1.0 / 24.0), n_o = R(0.25), n_t = R(0.125);
    c.e_m = (R(1.0) - s_e) * n_e;
    c.e_den = R(-11.0) * s_e * n_e;
    c.e_u2 = R(19.0) * s_e * n_e;
    c.e_f = (R(38.0) - R(19.0) * s_e) * n_e;
    c.e2_m = (R(1.0) - s_e2) * n_e2;
    c.e2_u2 = s_e2 * R(-475.0 / 63.0) * n_e2;
    c.e2_f = (R(-11.0) + R(5.5) * s_e2) * n_e2;
    c.q_m = (R(1.0) - s_q) * n_q;
    c.q_u = s_q * R(-2.0 / 3.0) * n_q;
    c.q_f = (R(-2.0 / 3.0) + s_q * R(1.0 / 3.0)) * n_q;
    c.x3_m = (R(1.0) - s_nu) * n_x3;
    c.x3_eq = s_nu * n_x3;
    c.x3_f = (R(2.0) - s_nu) * n_x3;
    c.xi_m = (R(1.0) - s_pi) * n_xi;
    c.xi_f = (R(1.0) - R(0.5) * s_pi) * n_xi;
    c.w_m = (R(1.0) - s_nu) * n_w;
    c.w_eq = s_nu * n_w;
    c.w_f = (R(2.0) - s_nu) * n_w;
    c.wi_m = (R(1.0) - s_pi) * n_wi;
    c.wi_f = (R(1.0) - R(0.5) * s_pi) * n_wi;
    c.o_m = (R(1.0) - s_nu) * n_o;
    c.o_eq = s_nu * n_o;
    c.o_f = (R(1.0) - R(0.5) * s_nu) * n_o;
    c.t_m = (R(1.0) - s_t) * n_t;
    c.fz = R(0.0);
    return c;
}

// Ensemble launch arguments (kernels.cuh, k_ens_step / k_ens_persistent)
struct EnsTile { int32_t start; int32_t count; };

struct EnsArgs {
    void *A;
    int64_t stride;
    const int32_t *nb;
    int64_t nf;              // fluid nodes of the whole arena (neighbour-table row length)
    const EnsTile *tiles;
    const int32_t *ntiles;   // device scalar
    StepParams P;
    MrtFold<double> fold;
    MrtFold<float> fold32;
    MrtFold<ff> foldff;
    float scale;
    int32_t ntime0;          // ntime of the first step of the launch
    int32_t nsteps;          // steps per persistent launch
    unsigned int *bar;       // [2] arrival count, generation
    int32_t *err;            // set when a barrier wait gives up
    int32_t unit;            // 1: the unit-rate collision (tau = 1, MRT preset 1) applies
    long long spin_limit;    // polls of one grid-barrier wait before it gives up
    uint32_t bar_extra;      // arrivals a barrier waits for beyond the grid (0; >0 only in
                             // the timeout test: the barrier can then never open)
};
// default poll limit of the persistent ensemble kernel's grid barrier (100 ns sleeps:
// several seconds, far beyond any step)
constexpr long long kBarrierSpinsDefault = 1ll << 26;

// FP16 deviation storage: value = w_q * ref + half_value * scale, ref = the rest
// density of the species.
template <class S> struct StoreTraits;
template <> struct StoreTraits<double> { static constexpr int bytes = 8; };
template <> struct StoreTraits<float> { static constexpr int bytes = 4; };
template <> struct StoreTraits<__half> { static constexpr int bytes = 2; };

}  // namespace mflbm
