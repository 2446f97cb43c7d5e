// launch.cuh -- host launchers of one kernel flavour; included after kernels.cuh.
#pragma once
#include "kernels.cuh"
#include "../../include/mflbm.h"

namespace mflbm {
namespace MFLBM_NS {

inline dim3 row_block(int nx) {
    int bx = nx >= 128 ? 128 : ((nx + 31) / 32) * 32;
    return dim3(bx, 128 / bx, 1);
}

template <class S> inline S *fs(const DevState &st) { return reinterpret_cast<S *>(st.f); }
template <class T> inline Nrm<T> *nrm(const DevState &st) { return reinterpret_cast<Nrm<T> *>(st.cn); }
template <class S> inline S *gs(const DevState &st) { return reinterpret_cast<S *>(st.g); }
// field arrays (phi, gradient) of the compute type T
template <class T> inline T *fld(void *p) { return reinterpret_cast<T *>(p); }

// storage type of the multiphase forms: FP64, or FP32 for the mixed form
inline bool mp_fp32(const DevState &st) { return st.multiphase && st.prec == MFLBM_FP32; }
// the multiphase double-word forms (FP64 storage or double-word storage): FP64 fields, the
// normal and curvature stencils in double-word arithmetic
inline bool dw_grad(const DevState &st) {
    return st.multiphase && (st.prec == MFLBM_FP64FF || st.prec == MFLBM_FF);
}
// the FP32 multiphase collision computes each node's curvature from the normal records
// (default build, fluid-cell gradient lists): the colour-gradient pass skips the curvature
// kernel, which then runs only before a reader of the curv field (monitor, get_gradient)
inline bool fused_curvature(const DevState &st) {
#ifdef MFLBM_STRICT
    (void)st;
    return false;
#else
    return mp_fp32(st) && st.glist && !st.gtile && !st.gsplit && st.n_gcell_c > 0;
#endif
}

// where the cell-addressed kernels find a population: dense planes, or a fluid list with
// boundary-plane slots (multiphase; singlephase with an inlet or outlet) through its slot map
inline PdfAt pdf_at(const DevState &st) {
    PdfAt a;
    a.qs = st.pmap ? st.lstride : st.L.qs;
    a.map = st.pmap;
    a.spare = st.pspare;
    return a;
}

template <class R> const MrtFold<R> &fold_of(const DevState &st);
template <> inline const MrtFold<double> &fold_of<double>(const DevState &st) { return st.fold; }
template <> inline const MrtFold<float> &fold_of<float>(const DevState &st) { return st.fold32; }
template <> inline const MrtFold<ff> &fold_of<ff>(const DevState &st) { return st.foldff; }

// The launchers are split over three translation units per flavour so that they compile
// in parallel: MFLBM_PART 1 the collision sweeps, 2 the ensembles and the velocity
// initialisation, 3 the rest and the launch table (which names the other two parts' entries).
#ifndef MFLBM_PART
#define MFLBM_PART 3
#endif
int collide(const DevState &st, bool odd, cudaStream_t s);
int ens_run(const EnsArgs &a, int prec, int persistent, int grid, int block, cudaStream_t s);
int ens_monitor(const EnsArgs &a, int prec, const int32_t *seg0, const int32_t *seg1, int nseg, double *out,
                cudaStream_t s);
int ens_init(const EnsArgs &a, int prec, cudaStream_t s);
int ens_max_grid(int prec, int block);
int init_velocity(const DevState &st, const double *rho, int rest_base, cudaStream_t s);

#if MFLBM_PART == 1
// The TMA even step: a persistent grid of as many blocks as fit on the device at once
// (blocks per SM from the occupancy calculator, cached per device), at most one per tile.
template <class S, bool UNIT>
int even_tma(const DevState &st, cudaStream_t s) {
    // whole tiles through the copies; the last block also takes the nfl % 128 nodes after them
    const int ntiles = st.nfl / kTmaNodes;
    if (ntiles == 0) return -1;   // fewer than 128 fluid nodes: the plain sweep
    const int smem = TmaTile<S>::stages * TmaTile<S>::bytes + 1024;
    static int max_grid[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    if (max_grid[dev] == 0) {
        int per = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sp_list_even_tma<S, UNIT>, kTmaNodes + 32, smem) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || per < 1)
            return -1;
        max_grid[dev] = per * sms;
    }
    const int grid = ntiles < max_grid[dev] ? ntiles : max_grid[dev];
    k_sp_list_even_tma<S, UNIT><<<grid, kTmaNodes + 32, smem, s>>>(st.tmap, fs<S>(st), st.lstride, st.nfl, st.P,
                                                                   fold_of<typename Store<S>::RS>(st), st.scale, st.err);
    return 1;
}

template <class S>
int collide_list(const DevState &st, bool odd, cudaStream_t s) {
    // the TMA even step for the double-word and FP16 storage (faster than the plain even
    // step on the 256^3 packing: 0.229 against 0.242 ms per sweep averaged with the odd
    // step, FP16 0.087 against 0.092); the FP32 deviation form moves only 135 bytes per node
    // and runs as fast plain, FP64 is bound by its arithmetic, and FP64 storage with the
    // double-word collision is issue-bound and faster at the plain sweep's occupancy
    if (!odd && st.tma && (std::is_same<S, ffs>::value || std::is_same<S, __half>::value)) {
        const int r = st.unit ? even_tma<S, true>(st, s) : even_tma<S, false>(st, s);
        if (r >= 0) return r;
    }
    const unsigned nb = (unsigned)((st.nfl + 127) / 128);
    const auto &cf = fold_of<typename Store<S>::RS>(st);
    if (st.unit) {
        if (odd) k_sp_list<S, true, true><<<nb, 128, 0, s>>>(fs<S>(st), st.lstride, st.nb, st.nfl, st.P, cf, st.scale);
        else k_sp_list<S, false, true><<<nb, 128, 0, s>>>(fs<S>(st), st.lstride, st.nb, st.nfl, st.P, cf, st.scale);
    } else {
        if (odd) k_sp_list<S, true, false><<<nb, 128, 0, s>>>(fs<S>(st), st.lstride, st.nb, st.nfl, st.P, cf, st.scale);
        else k_sp_list<S, false, false><<<nb, 128, 0, s>>>(fs<S>(st), st.lstride, st.nb, st.nfl, st.P, cf, st.scale);
    }
    return 1;
}

template <class S>
int collide_t(const DevState &st, bool odd, cudaStream_t s) {
    if (st.list) return collide_list<S>(st, odd, s);
    if (st.ncell == 0) return 0;
    const unsigned nb = (unsigned)((st.ncell + 127) / 128);
    const auto &cf = fold_of<typename Store<S>::RS>(st);
    if (st.unit) {
        if (odd) k_sp_step<S, true, true><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
        else k_sp_step<S, false, true><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
    } else {
        if (odd) k_sp_step<S, true, false><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
        else k_sp_step<S, false, false><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
    }
    return 1;
}

template <class T>
int collide_mp(const DevState &st, bool odd, cudaStream_t s) {
    if (st.mplist) {
        const unsigned nb = (unsigned)((st.nfl + 127) / 128);
        T *f = fs<T>(st), *gg = gs<T>(st);
        auto *phi = fld<T>(st.phi);
        auto *cn = nrm<T>(st);
        auto *curv = fld<T>(st.curv);
        if (fused_curvature(st)) {
            if (odd)
                k_mp_step<T, true, true, true><<<nb, 128, 0, s>>>(f, gg, phi, cn, curv, st.cell1, st.nfl, st.L, st.P,
                                                                  st.rk_weight2, st.nb, st.lstride);
            else
                k_mp_step<T, false, true, true><<<nb, 128, 0, s>>>(f, gg, phi, cn, curv, st.cell1, st.nfl, st.L, st.P,
                                                                   st.rk_weight2, st.nb, st.lstride);
            return 1;
        }
        if (odd)
            k_mp_step<T, true, true><<<nb, 128, 0, s>>>(f, gg, phi, cn, curv, st.cell1, st.nfl, st.L, st.P,
                                                        st.rk_weight2, st.nb, st.lstride);
        else
            k_mp_step<T, false, true><<<nb, 128, 0, s>>>(f, gg, phi, cn, curv, st.cell1, st.nfl, st.L, st.P,
                                                         st.rk_weight2, st.nb, st.lstride);
        return 1;
    }
    if (st.ncell == 0) return 0;
    const unsigned nb = (unsigned)((st.ncell + 127) / 128);
    T *f = fs<T>(st), *gg = gs<T>(st);
    if (fused_curvature(st)) {
        if (odd)
            k_mp_step<T, true, false, true><<<nb, 128, 0, s>>>(f, gg, fld<T>(st.phi), nrm<T>(st), fld<T>(st.curv),
                                                               st.cells, st.ncell, st.L, st.P, st.rk_weight2);
        else
            k_mp_step<T, false, false, true><<<nb, 128, 0, s>>>(f, gg, fld<T>(st.phi), nrm<T>(st), fld<T>(st.curv),
                                                                st.cells, st.ncell, st.L, st.P, st.rk_weight2);
        return 1;
    }
    if (odd)
        k_mp_step<T, true><<<nb, 128, 0, s>>>(f, gg, fld<T>(st.phi), nrm<T>(st), fld<T>(st.curv), st.cells, st.ncell, st.L, st.P,
                                              st.rk_weight2);
    else
        k_mp_step<T, false><<<nb, 128, 0, s>>>(f, gg, fld<T>(st.phi), nrm<T>(st), fld<T>(st.curv), st.cells, st.ncell, st.L, st.P,
                                               st.rk_weight2);
    return 1;
}

template <class S>
int collide_mp_ff(const DevState &st, bool odd, cudaStream_t s) {
    if (st.mplist) {
        const unsigned nb = (unsigned)((st.nfl + 127) / 128);
        S *f = fs<S>(st), *gg = gs<S>(st);
        if (odd)
            k_mp_step_ff<true, S, true><<<nb, 128, 0, s>>>(f, gg, fld<double>(st.phi), nrm<double>(st),
                                                           fld<double>(st.curv), st.cell1, st.nfl, st.L, st.mpff, st.P.mrt,
                                                           st.nb, st.lstride);
        else
            k_mp_step_ff<false, S, true><<<nb, 128, 0, s>>>(f, gg, fld<double>(st.phi), nrm<double>(st),
                                                            fld<double>(st.curv), st.cell1, st.nfl,
                                                            st.L, st.mpff, st.P.mrt, st.nb, st.lstride);
        return 1;
    }
    if (st.ncell == 0) return 0;
    const unsigned nb = (unsigned)((st.ncell + 127) / 128);
    S *f = fs<S>(st), *gg = gs<S>(st);
    if (odd)
        k_mp_step_ff<true, S><<<nb, 128, 0, s>>>(f, gg, fld<double>(st.phi), nrm<double>(st), fld<double>(st.curv), st.cells,
                                             st.ncell, st.L, st.mpff, st.P.mrt);
    else
        k_mp_step_ff<false, S><<<nb, 128, 0, s>>>(f, gg, fld<double>(st.phi), nrm<double>(st), fld<double>(st.curv), st.cells,
                                              st.ncell, st.L, st.mpff, st.P.mrt);
    return 1;
}

int collide(const DevState &st, bool odd, cudaStream_t s) {
    if (st.multiphase) {
        if (st.prec == MFLBM_FP64FF) return collide_mp_ff<double>(st, odd, s);
        if (st.prec == MFLBM_FF) return collide_mp_ff<ffs>(st, odd, s);
        return mp_fp32(st) ? collide_mp<float>(st, odd, s) : collide_mp<double>(st, odd, s);
    }
    switch (st.prec) {
        case MFLBM_FP32: return collide_t<dfloat>(st, odd, s);
        case MFLBM_FP16: return collide_t<__half>(st, odd, s);
        case MFLBM_FP64FF: return collide_t<f64ff>(st, odd, s);
        case MFLBM_FF: return collide_t<ffs>(st, odd, s);
        default: return collide_t<double>(st, odd, s);
    }
}

#endif  // MFLBM_PART == 1

#if MFLBM_PART == 3
template <class S>
int wrap_t(const DevState &st, bool pull, cudaStream_t s) {
    int n_launch = 0;
    const Layout &L = st.L;
    const int nsp = st.multiphase ? 2 : 1;
    S *f = fs<S>(st);
    // faces in the reference's order z, y (then the x extension), edges last
    const int per[3] = {st.P.iper, st.P.jper, st.P.kper};
    const int order[3] = {2, 1, 0};
    for (int d : order) {
        if (!per[d]) continue;
        const int64_t n1 = d == 0 ? L.ny : L.nx;
        const int64_t n2 = d == 2 ? L.ny : L.nz;
        const int64_t n = n1 * n2 * nsp;
        k_wrap_faces<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f, nsp, L, d, pull ? 1 : 0);
        ++n_launch;
    }
    // edge along axis a exists when the two other axes are periodic
    for (int a = 0; a < 3; ++a) {
        const int o1 = (a + 1) % 3, o2 = (a + 2) % 3;
        if (!(per[o1] && per[o2])) continue;
        const int len = a == 0 ? L.nx : (a == 1 ? L.ny : L.nz);
        const int64_t n = (int64_t)len * nsp;
        k_wrap_edges<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f, nsp, L, a, pull ? 1 : 0);
        ++n_launch;
    }
    return n_launch;
}

int wrap(const DevState &st, bool pull, cudaStream_t s) {
    // the fluid-list neighbour table already wraps periodic directions (phi, dense in every
    // layout, is wrapped below)
    if ((st.list && !st.mplist) || !(st.P.iper || st.P.jper || st.P.kper)) return 0;
    int n_launch = 0;
    if (!st.mplist) switch (st.prec) {
        case MFLBM_FP32: n_launch = st.multiphase ? wrap_t<float>(st, pull, s) : wrap_t<dfloat>(st, pull, s); break;
        case MFLBM_FP16: n_launch = wrap_t<__half>(st, pull, s); break;
        case MFLBM_FF: n_launch = wrap_t<ffs>(st, pull, s); break;
        default: n_launch = wrap_t<double>(st, pull, s); break;
    }
    if (st.mplist && st.nwrap > 0) {
        const unsigned nb = (unsigned)((2 * st.nwrap + 255) / 256);
        const int pl = pull ? 1 : 0;
        // plain copies: moved as 4- or 8-byte words whatever the storage type
        if (mp_fp32(st))
            k_mp_wrap_ghosts<uint32_t><<<nb, 256, 0, s>>>(fs<uint32_t>(st), gs<uint32_t>(st), st.lstride, st.pwrap,
                                                          st.nwrap, pl);
        else
            k_mp_wrap_ghosts<uint64_t><<<nb, 256, 0, s>>>(fs<uint64_t>(st), gs<uint64_t>(st), st.lstride, st.pwrap,
                                                          st.nwrap, pl);
        ++n_launch;
    }
    if (st.multiphase && (st.P.jper || st.P.kper)) {
        const Layout &L = st.L;
        const int64_t n = (st.P.kper ? (int64_t)4 * L.nx * L.ny : 0) + (st.P.jper ? (int64_t)4 * L.nx * L.nz : 0) +
                          ((st.P.jper && st.P.kper) ? (int64_t)16 * L.nx : 0);
        if (mp_fp32(st))
            k_wrap_phi<float><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fld<float>(st.phi), L, st.P.jper, st.P.kper);
        else
            k_wrap_phi<double><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fld<double>(st.phi), L, st.P.jper, st.P.kper);
        ++n_launch;
    }
    return n_launch;
}

template <class S>
int boundary_t(const DevState &st, bool before_odd, int inlet_bc, int outlet_bc, bool open_z, cudaStream_t s) {
    int n_launch = 0;
    const Layout &L = st.L;
    const int bx = L.nx >= 128 ? 128 : ((L.nx + 31) / 32) * 32;
    const dim3 b(bx), g((L.nx + bx - 1) / bx, L.ny);
    S *f = fs<S>(st), *gg = st.multiphase ? gs<S>(st) : nullptr;
    using FT = typename Store<S>::R;
    FT *phi = st.multiphase ? fld<FT>(st.phi) : nullptr;
    const int bo = before_odd ? 1 : 0;
    if (open_z) {
        if (inlet_bc == 1)
            k_inlet_velocity<S><<<g, b, 0, s>>>(f, gg, phi, st.walls, st.w_in, L, pdf_at(st), st.P, bo, st.multiphase,
                                                st.ref, st.scale);
        else if (inlet_bc == 2)
            k_inlet_zouhe<S><<<g, b, 0, s>>>(f, gg, phi, st.walls, L, pdf_at(st), st.P, bo, st.multiphase, st.ref,
                                             st.scale);
        if (outlet_bc == 1)
            k_outlet_convective<S><<<g, b, 0, s>>>(f, gg, phi, st.fconv, st.gconv, st.phiconv, st.walls, L, pdf_at(st),
                                                   st.P, bo, st.multiphase, st.ref, st.scale);
        else if (outlet_bc == 2)
            k_outlet_zouhe<S><<<g, b, 0, s>>>(f, gg, phi, st.walls, L, pdf_at(st), st.P, bo, st.multiphase, st.ref,
                                              st.scale);
        n_launch += (inlet_bc == 1 || inlet_bc == 2) + (outlet_bc == 1 || outlet_bc == 2);
    }
    return n_launch;
}

int boundary(const DevState &st, bool before_odd, int inlet_bc, int outlet_bc, bool open_z, cudaStream_t s) {
    int n_launch;
    switch (st.prec) {
        case MFLBM_FP32:
            n_launch = st.multiphase ? boundary_t<float>(st, before_odd, inlet_bc, outlet_bc, open_z, s)
                                     : boundary_t<dfloat>(st, before_odd, inlet_bc, outlet_bc, open_z, s);
            break;
        case MFLBM_FP16: n_launch = boundary_t<__half>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
        case MFLBM_FF: n_launch = boundary_t<ffs>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
        default: n_launch = boundary_t<double>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
    }
    if (st.multiphase && st.P.porous_plate_cmd != 0 && st.P.z_porous_plate >= 1 && st.P.z_porous_plate <= st.L.nz) {
        const Layout &L = st.L;
        const int bx = L.nx >= 128 ? 128 : ((L.nx + 31) / 32) * 32;
        void *blocked = st.P.porous_plate_cmd == 1 ? st.f : st.g;
        void *passing = st.P.porous_plate_cmd == 1 ? st.g : st.f;
        const dim3 gp((L.nx + bx - 1) / bx, L.ny);
        if (mp_fp32(st))
            k_porous_plate<float><<<gp, bx, 0, s>>>(fld<float>(blocked), fld<float>(passing), L, pdf_at(st),
                                                    st.P.z_porous_plate, before_odd ? 1 : 0);
        else
            k_porous_plate<double><<<gp, bx, 0, s>>>(fld<double>(blocked), fld<double>(passing), L, pdf_at(st),
                                                     st.P.z_porous_plate, before_odd ? 1 : 0);
        ++n_launch;
    }
    return n_launch;
}

template <class T>
int color_gradient_t(const DevState &st, cudaStream_t s) {
    const Layout &L = st.L;
    T *phi = fld<T>(st.phi), *curv = fld<T>(st.curv);
    Nrm<T> *cn = nrm<T>(st);
    int n_launch = 2 + (st.ns > 0 ? 2 : 0) + (st.nf > 0 ? 1 : 0);
    const T min_one_m = sizeof(T) == 4 ? T(1e-6) : (dw_grad(st) ? T(1e-12) : T(0.0));
    bool wet_done = false;   // the normals kernel applied the wetting
    if (st.ns > 0) {
        if (st.sbc) k_extrap_phi_c<T><<<(st.ns + 127) / 128, 128, 0, s>>>(phi, st.sbc, st.ns, L);
        else k_extrap_phi<T><<<(st.ns + 127) / 128, 128, 0, s>>>(phi, st.sb, st.ns, L);
    }
#ifndef MFLBM_STRICT
    if (st.gtile && !dw_grad(st)) {
        const dim3 b(GRAD_TX, GRAD_TY);
        const dim3 g((L.nx + 4 + GRAD_TX - 1) / GRAD_TX, (L.ny + 4 + GRAD_TY - 1) / GRAD_TY,
                     (L.nz + 4 + GRAD_KCH - 1) / GRAD_KCH);
        k_normals_tile<T><<<g, b, 0, s>>>(phi, st.walls, cn, L);
    } else if (st.glist) {
        if (st.n_gcell_n > 0) {
            bool done = false;
            if constexpr (std::is_same<T, double>::value) {
                if (dw_grad(st)) {
                    k_normals_list_ff<<<(st.n_gcell_n + 255) / 256, 256, 0, s>>>(phi, st.gcell_n, st.n_gcell_n, cn, L);
                    done = true;
                }
            }
            if (!done && st.gwet) {
                k_normals_list<T, true><<<(st.n_gcell_n + 255) / 256, 256, 0, s>>>(phi, st.gcell_n, st.n_gcell_n, cn, L,
                                                                                   st.fb, st.nf, min_one_m);
                done = wet_done = true;
            }
            if (!done)
                k_normals_list<T><<<(st.n_gcell_n + 255) / 256, 256, 0, s>>>(phi, st.gcell_n, st.n_gcell_n, cn, L);
        }
    } else
#endif
    {
        const int nxh = L.nx + 4;
        const int bx = nxh >= 128 ? 128 : ((nxh + 31) / 32) * 32;
        const dim3 b(bx, 256 / bx > 0 ? (unsigned)(256 / bx) : 1u);
        const dim3 g((nxh + b.x - 1) / b.x, (L.ny + 4 + b.y - 1) / b.y, L.nz + 4);
        k_normals<T><<<g, b, 0, s>>>(phi, st.walls, cn, L);
    }
    if (st.nf > 0 && !wet_done) k_wetting<T><<<(st.nf + 127) / 128, 128, 0, s>>>(cn, st.fb, st.nf, L, min_one_m);
    if (wet_done) --n_launch;
    if (st.ns > 0) {
        if (st.sbc) k_extrap_normals_c<T><<<(st.ns + 127) / 128, 128, 0, s>>>(cn, st.sbc, st.ns, L);
        else k_extrap_normals<T><<<(st.ns + 127) / 128, 128, 0, s>>>(cn, st.sb, st.ns, L);
    }
#ifndef MFLBM_STRICT
    if (st.gtile && !dw_grad(st)) {
        const dim3 b(GRAD_TX, GRAD_TY);
        const dim3 g((L.nx + GRAD_TX - 1) / GRAD_TX, (L.ny + GRAD_TY - 1) / GRAD_TY, (L.nz + GRAD_KCH - 1) / GRAD_KCH);
        k_curvature_tile<T><<<g, b, 0, s>>>(cn, curv, st.walls, L);
    } else if (st.glist) {
        if (st.n_gcell_c > 0) {
            bool done = false;
            if constexpr (std::is_same<T, double>::value) {
                if (dw_grad(st)) {
                    k_curvature_list_ff<<<(st.n_gcell_c + 255) / 256, 256, 0, s>>>(cn, curv, st.gcell_c,
                                                                                  st.n_gcell_c, L);
                    done = true;
                }
            }
            if (!done && fused_curvature(st)) {
                done = true;   // each node's curvature is computed by the next collision
                --n_launch;
            }
            if (!done)
                k_curvature_list<T><<<(st.n_gcell_c + 255) / 256, 256, 0, s>>>(cn, curv, st.gcell_c,
                                                                               st.n_gcell_c, L);
        }
    } else
#endif
    {
        const int bx = L.nx >= 128 ? 128 : ((L.nx + 31) / 32) * 32;
        const dim3 b(bx, 256 / bx);
        const dim3 g((L.nx + b.x - 1) / b.x, (L.ny + b.y - 1) / b.y, L.nz);
        k_curvature<T><<<g, b, 0, s>>>(cn, curv, st.walls, L);
    }
    return n_launch;
}

// the curv field for a reader other than the collision, when the collision computes the
// curvature itself (the colour-gradient pass then leaves curv unwritten)
int curvature_field(const DevState &st, cudaStream_t s) {
    if (!fused_curvature(st)) return 0;
    k_curvature_list<float><<<(st.n_gcell_c + 255) / 256, 256, 0, s>>>(nrm<float>(st), fld<float>(st.curv), st.gcell_c,
                                                                       st.n_gcell_c, st.L);
    return 1;
}

int color_gradient(const DevState &st, cudaStream_t s) {
    if (!st.multiphase) return 0;
    return mp_fp32(st) ? color_gradient_t<float>(st, s) : color_gradient_t<double>(st, s);
}

template <class S>
int monitor_t(const DevState &st, cudaStream_t s) {
    using FT = typename Store<S>::R;
    if (st.list && !st.mplist) {
        const size_t b1 = sizeof(double) * (size_t)(st.L.nx + 2) * (st.L.ny + 2) * (st.L.nz + 2);
        cudaMemsetAsync(st.u, 0, b1, s);
        cudaMemsetAsync(st.v, 0, b1, s);
        cudaMemsetAsync(st.w, 0, b1, s);
        cudaMemsetAsync(st.rho, 0, b1, s);
        cudaMemsetAsync(st.mon, 0, sizeof(double) * kMonNQ * st.L.nz, s);
        k_list_monitor<S><<<st.L.nz, MON_THREADS, 0, s>>>(fs<S>(st), st.lstride, st.lseg, st.lseg + 1, st.L.nz, st.cell1, st.u, st.v,
                                                          st.w, st.rho, st.mon, st.P, 1, st.scale);
        return 1;
    }
    const int nc = st.multiphase ? curvature_field(st, s) : 0;
    k_monitor<S><<<st.L.nz, MON_THREADS, 0, s>>>(fs<S>(st), st.multiphase ? gs<S>(st) : nullptr, fld<FT>(st.phi), st.walls,
                                                 nrm<FT>(st),
                                                 fld<FT>(st.curv), st.u, st.v, st.w, st.rho, st.mon, st.L, pdf_at(st),
                                                 st.P, st.multiphase, 1, st.ref, st.scale);
    return 1 + nc;
}

int monitor(const DevState &st, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return st.multiphase ? monitor_t<float>(st, s) : monitor_t<dfloat>(st, s);
        case MFLBM_FP16: return monitor_t<__half>(st, s);
        case MFLBM_FF: return monitor_t<ffs>(st, s);
        default: return monitor_t<double>(st, s);
    }
}

int saturation(const DevState &st, cudaStream_t s) {
    if (!st.multiphase) return 0;
    if (mp_fp32(st))
        k_saturation<float><<<st.L.nz, MON_THREADS, 0, s>>>(fld<float>(st.phi), st.walls, st.mon, st.L);
    else
        k_saturation<double><<<st.L.nz, MON_THREADS, 0, s>>>(fld<double>(st.phi), st.walls, st.mon, st.L);
    return 1;
}

template <class S>
int init_t(const DevState &st, bool convec, cudaStream_t s) {
    const Layout &L = st.L;
    if (st.list && !st.mplist) {
        // the rest equilibrium in every slot (fluid nodes, boundary-plane cells, links)
        const int64_t n = 19 * st.lstride;
        k_list_init<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fs<S>(st), st.lstride, st.scale);
        const size_t b1 = sizeof(double) * (size_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        cudaMemsetAsync(st.u, 0, b1, s);
        cudaMemsetAsync(st.v, 0, b1, s);
        cudaMemsetAsync(st.w, 0, b1, s);
        const int64_t nb1 = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        k_list_plane_fill<<<(unsigned)((nb1 + 255) / 256), 256, 0, s>>>(st.rho, nb1, 1.0);
        if (!convec) return 2;
        const int64_t np = (int64_t)(L.nx + 2) * (L.ny + 2);
        k_init_convec<S><<<(unsigned)((np + 255) / 256), 256, 0, s>>>(fs<S>(st), nullptr, nullptr, st.fconv, nullptr,
                                                                      nullptr, L, pdf_at(st), 0, st.ref, st.scale);
        return 3;
    }
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    S *g = st.multiphase ? gs<S>(st) : nullptr;
    using FT = typename Store<S>::R;
    k_init_eq<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(fs<S>(st), g, fld<FT>(st.phi), st.u, st.v, st.w, st.rho, L,
                                                              pdf_at(st), st.multiphase, st.ref, st.scale);
    int n = 1;
    if (st.mplist && st.nlink > 0) {
        k_mp_init_links<S><<<(unsigned)((st.nlink + 255) / 256), 256, 0, s>>>(fs<S>(st), g, fld<FT>(st.phi), st.lstride,
                                                                              st.link, st.nlink, L);
        ++n;
    }
    if (convec) {
        const int64_t np = (int64_t)(L.nx + 2) * (L.ny + 2);
        k_init_convec<S><<<(unsigned)((np + 255) / 256), 256, 0, s>>>(fs<S>(st), g, fld<FT>(st.phi), st.fconv, st.gconv, st.phiconv,
                                                                      L, pdf_at(st), st.multiphase, st.ref, st.scale);
        ++n;
    }
    return n;
}

int init_equilibrium(const DevState &st, bool convec, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return st.multiphase ? init_t<float>(st, convec, s) : init_t<dfloat>(st, convec, s);
        case MFLBM_FP16: return init_t<__half>(st, convec, s);
        case MFLBM_FF: return init_t<ffs>(st, convec, s);
        default: return init_t<double>(st, convec, s);
    }
}

template <class S>
int convert_in_t(const DevState &st, int sp, int q, cudaStream_t s) {
    const Layout &L = st.L;
    if (st.list) {
        S *A = sp == 0 ? fs<S>(st) : gs<S>(st);
        const int64_t n = st.nfl + st.nlink;
        k_list_in<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, st.lstride, q, st.cell1, st.nfl, st.link, st.nlink,
                                                                 st.stage, st.scale);
        if (!st.pmap) return 1;
        const int64_t n1 = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        k_mp_planes_in<S><<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(A, st.lstride, q, st.pmap, st.nfl, n1, st.stage,
                                                                       st.scale);
        return 2;
    }
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    S *base = (sp == 0 ? fs<S>(st) : gs<S>(st)) + (int64_t)q * L.qs;
    k_convert_in<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(base, st.stage, L, q, st.ref, st.scale);
    return 1;
}

template <class S>
int convert_out_t(const DevState &st, int sp, int q, cudaStream_t s) {
    const Layout &L = st.L;
    if (st.list) {
        // fluid nodes, link slots, periodic ghosts as their images, boundary-plane slots; the
        // cells that no update reads keep the rest weight
        const S *A = sp == 0 ? fs<S>(st) : gs<S>(st);
        const int64_t n1 = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        const int64_t n = st.nfl + st.nlink;
        k_list_plane_fill<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(st.stage, n1, WEQ(q));
        k_list_out<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, st.lstride, q, st.cell1, st.nfl, st.link, st.nlink,
                                                                  st.stage, st.scale);
        k_list_ghosts<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(st.stage, L, st.P.iper, st.P.jper, st.P.kper);
        if (!st.pmap) return 3;
        k_mp_planes_out<S><<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(A, st.lstride, q, st.pmap, st.nfl, n1, st.stage,
                                                                        st.scale);
        return 4;
    }
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const S *base = (sp == 0 ? fs<S>(st) : gs<S>(st)) + (int64_t)q * L.qs;
    k_convert_out<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(st.stage, base, L, q, st.ref, st.scale);
    return 1;
}

int convert_in(const DevState &st, int sp, int q, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return st.multiphase ? convert_in_t<float>(st, sp, q, s) : convert_in_t<dfloat>(st, sp, q, s);
        case MFLBM_FP16: return convert_in_t<__half>(st, sp, q, s);
        case MFLBM_FF: return convert_in_t<ffs>(st, sp, q, s);
        default: return convert_in_t<double>(st, sp, q, s);
    }
}

int convert_out(const DevState &st, int sp, int q, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return st.multiphase ? convert_out_t<float>(st, sp, q, s) : convert_out_t<dfloat>(st, sp, q, s);
        case MFLBM_FP16: return convert_out_t<__half>(st, sp, q, s);
        case MFLBM_FF: return convert_out_t<ffs>(st, sp, q, s);
        default: return convert_out_t<double>(st, sp, q, s);
    }
}

int field_in(const DevState &st, void *dst, int64_t n, cudaStream_t s) {
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (st.felt == 4) k_field_in<float><<<nb, 256, 0, s>>>(fld<float>(dst), st.stage, n);
    else k_field_in<double><<<nb, 256, 0, s>>>(fld<double>(dst), st.stage, n);
    return 1;
}

int field_out(const DevState &st, const void *src, int64_t n, int stride, cudaStream_t s) {
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (st.felt == 4) k_field_out<float><<<nb, 256, 0, s>>>(st.stage, reinterpret_cast<const float *>(src), n, stride);
    else k_field_out<double><<<nb, 256, 0, s>>>(st.stage, reinterpret_cast<const double *>(src), n, stride);
    return 1;
}

#endif  // MFLBM_PART == 3

#if MFLBM_PART == 2
// ---- ensembles --------------------------------------------------------------------
template <class S>
int ens_run_t(const EnsArgs &a, int persistent, int grid, int block, cudaStream_t s) {
    if (persistent) {
        void *args[] = {const_cast<EnsArgs *>(&a)};
        const void *fn = a.unit ? (const void *)k_ens_persistent<S, true> : (const void *)k_ens_persistent<S, false>;
        cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, 0, s);
        return e == cudaSuccess ? 1 : -1;
    }
    for (int t = 0; t < a.nsteps; ++t) {
        const bool odd = ((a.ntime0 + t) & 1) != 0;
        if (a.unit) {
            if (odd) k_ens_step<S, true, true><<<grid, block, 0, s>>>(a);
            else k_ens_step<S, false, true><<<grid, block, 0, s>>>(a);
        } else {
            if (odd) k_ens_step<S, true, false><<<grid, block, 0, s>>>(a);
            else k_ens_step<S, false, false><<<grid, block, 0, s>>>(a);
        }
    }
    return cudaPeekAtLastError() == cudaSuccess ? a.nsteps : -1;
}

int ens_run(const EnsArgs &a, int prec, int persistent, int grid, int block, cudaStream_t s) {
    switch (prec) {
        case MFLBM_FP32: return ens_run_t<dfloat>(a, persistent, grid, block, s);
        case MFLBM_FP16: return ens_run_t<__half>(a, persistent, grid, block, s);
        case MFLBM_FP64FF: return ens_run_t<f64ff>(a, persistent, grid, block, s);
        case MFLBM_FF: return ens_run_t<ffs>(a, persistent, grid, block, s);
        default: return ens_run_t<double>(a, persistent, grid, block, s);
    }
}

template <class S>
int ens_monitor_t(const EnsArgs &a, const int32_t *seg0, const int32_t *seg1, int nseg, double *out, cudaStream_t s) {
    k_list_monitor<S><<<nseg, MON_THREADS, 0, s>>>(reinterpret_cast<const S *>(a.A), a.stride, seg0, seg1, nseg, nullptr,
                                                   nullptr, nullptr, nullptr, nullptr, out, a.P, 0, a.scale);
    return 1;
}

int ens_monitor(const EnsArgs &a, int prec, const int32_t *seg0, const int32_t *seg1, int nseg, double *out,
                cudaStream_t s) {
    switch (prec) {
        case MFLBM_FP32: return ens_monitor_t<dfloat>(a, seg0, seg1, nseg, out, s);
        case MFLBM_FP16: return ens_monitor_t<__half>(a, seg0, seg1, nseg, out, s);
        case MFLBM_FF: return ens_monitor_t<ffs>(a, seg0, seg1, nseg, out, s);
        default: return ens_monitor_t<double>(a, seg0, seg1, nseg, out, s);
    }
}

int ens_init(const EnsArgs &a, int prec, cudaStream_t s) {
    const int64_t n = 19 * a.stride;
    const unsigned nb = (unsigned)((n + 255) / 256);
    switch (prec) {
        case MFLBM_FP32: k_list_init<dfloat><<<nb, 256, 0, s>>>(reinterpret_cast<dfloat *>(a.A), a.stride, a.scale); break;
        case MFLBM_FP16: k_list_init<__half><<<nb, 256, 0, s>>>(reinterpret_cast<__half *>(a.A), a.stride, a.scale); break;
        case MFLBM_FF: k_list_init<ffs><<<nb, 256, 0, s>>>(reinterpret_cast<ffs *>(a.A), a.stride, a.scale); break;
        default: k_list_init<double><<<nb, 256, 0, s>>>(reinterpret_cast<double *>(a.A), a.stride, a.scale); break;
    }
    return 1;
}

int ens_max_grid(int prec, int block) {
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    cudaError_t e;
    switch (prec) {
        case MFLBM_FP32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ens_persistent<dfloat, false>, block, 0); break;
        case MFLBM_FP16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ens_persistent<__half, false>, block, 0); break;
        case MFLBM_FP64FF: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ens_persistent<f64ff, false>, block, 0); break;
        case MFLBM_FF: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ens_persistent<ffs, false>, block, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ens_persistent<double, false>, block, 0); break;
    }
    return e == cudaSuccess ? per * nsm : 0;
}

template <class S>
int init_velocity_t(const DevState &st, const double *rho, int rest_base, cudaStream_t s) {
    if (st.list) {
        k_init_vel_list<S><<<(unsigned)((st.lstride + 255) / 256), 256, 0, s>>>(fs<S>(st), st.lstride, st.cell1, st.nfl,
                                                                                 rho, st.u, st.v, st.w, rest_base,
                                                                                 st.scale);
        k_init_vel_links<S><<<(unsigned)((st.nfl + 255) / 256), 256, 0, s>>>(fs<S>(st), st.lstride, st.nb, st.cell1,
                                                                             st.nfl, rho, st.u, st.v, st.w, rest_base,
                                                                             st.scale);
        if (!st.pmap) return 2;
        // the boundary-plane cells last, as the dense kernel writes them
        const Layout &L = st.L;
        const int64_t n1 = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        k_init_vel_planes<S><<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(fs<S>(st), pdf_at(st), st.nfl, rho, st.u,
                                                                          st.v, st.w, st.walls, L, rest_base, st.scale);
        return 3;
    }
    const Layout &L = st.L;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    k_init_vel_dense<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(fs<S>(st), rho, st.u, st.v, st.w, st.walls, L,
                                                                     rest_base, st.scale);
    return 1;
}

int init_velocity(const DevState &st, const double *rho, int rest_base, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return init_velocity_t<dfloat>(st, rho, rest_base, s);
        case MFLBM_FP16: return init_velocity_t<__half>(st, rho, rest_base, s);
        case MFLBM_FF: return init_velocity_t<ffs>(st, rho, rest_base, s);
        default: return init_velocity_t<double>(st, rho, rest_base, s);
    }
}

#endif  // MFLBM_PART == 2

#if MFLBM_PART == 3
int steady(const DevState &st, void *phi_old, double *out, int obs_z, int copy_old, cudaStream_t s) {
    if (mp_fp32(st))
        k_steady<float><<<st.L.nz, MON_THREADS, 0, s>>>(fld<float>(st.phi), fld<float>(phi_old), st.rho, st.u, st.v,
                                                        st.w, st.walls, out, st.L, obs_z, copy_old);
    else
        k_steady<double><<<st.L.nz, MON_THREADS, 0, s>>>(fld<double>(st.phi), fld<double>(phi_old), st.rho, st.u, st.v,
                                                         st.w, st.walls, out, st.L, obs_z, copy_old);
    return 1;
}

int change_inlet_phase(const DevState &st, int cmd, int kmax, cudaStream_t s) {
    if (kmax < 0 || (cmd != 1 && cmd != 2)) return 0;
    const Layout &L = st.L;
    const int64_t n = (int64_t)19 * (L.nx + 2) * (L.ny + 2) * (kmax + 1);
    const unsigned nb = (unsigned)((n + 255) / 256);
    const PdfAt pa = pdf_at(st);
    const unsigned nl = (unsigned)((st.nlink + 255) / 256);
    const bool links = st.mplist && st.nlink > 0;
    if (mp_fp32(st)) {
        k_change_inlet_phase<float><<<nb, 256, 0, s>>>(fs<float>(st), gs<float>(st), L, pa, kmax, cmd == 1);
        if (links) k_change_inlet_links<float><<<nl, 256, 0, s>>>(fs<float>(st), gs<float>(st), st.lstride, st.link,
                                                                  st.nlink, L, kmax, cmd == 1);
        return links ? 2 : 1;
    }
    if (st.prec == MFLBM_FF) {
        k_change_inlet_phase<ffs><<<nb, 256, 0, s>>>(fs<ffs>(st), gs<ffs>(st), L, pa, kmax, cmd == 1);
        if (links) k_change_inlet_links<ffs><<<nl, 256, 0, s>>>(fs<ffs>(st), gs<ffs>(st), st.lstride, st.link, st.nlink,
                                                                L, kmax, cmd == 1);
        return links ? 2 : 1;
    }
    if (links) k_change_inlet_links<double><<<nl, 256, 0, s>>>(fs<double>(st), gs<double>(st), st.lstride, st.link,
                                                               st.nlink, L, kmax, cmd == 1);
    k_change_inlet_phase<double><<<nb, 256, 0, s>>>(fs<double>(st), gs<double>(st), L, pa, kmax, cmd == 1);
    return links ? 2 : 1;
}

const KernelTable table = {collide,          wrap,        boundary,   color_gradient, monitor, saturation,
                           init_equilibrium, convert_in,  convert_out, field_in,      field_out,
                           ens_run,          ens_monitor, ens_init,   ens_max_grid,   init_velocity,
                           steady,           change_inlet_phase, curvature_field};

#endif  // MFLBM_PART == 3

}  // namespace MFLBM_NS
}  // namespace mflbm
