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

template <class S> S *fs(const DevState &st) { return reinterpret_cast<S *>(st.f); }
template <class S> S *gs(const DevState &st) { return reinterpret_cast<S *>(st.g); }

template <class R> const MrtFold<R> &fold_of(const DevState &st);
template <> const MrtFold<double> &fold_of<double>(const DevState &st) { return st.fold; }
template <> const MrtFold<float> &fold_of<float>(const DevState &st) { return st.fold32; }

template <class S>
int collide_t(const DevState &st, bool odd, cudaStream_t s) {
    if (st.ncell == 0) return 0;
    const unsigned nb = (unsigned)((st.ncell + 127) / 128);
    const auto &cf = fold_of<typename Store<S>::R>(st);
    if (odd)
        k_sp_step<S, true><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
    else
        k_sp_step<S, false><<<nb, 128, 0, s>>>(fs<S>(st), st.cells, st.ncell, st.L, st.P, cf, st.scale);
    return 1;
}

int collide(const DevState &st, bool odd, cudaStream_t s) {
    if (st.multiphase) {
        if (st.ncell == 0) return 0;
        const unsigned nb = (unsigned)((st.ncell + 127) / 128);
        double *f = fs<double>(st), *gg = gs<double>(st);
        if (odd)
            k_mp_step<true><<<nb, 128, 0, s>>>(f, gg, st.phi, st.cnx, st.cny, st.cnz, st.cnorm, st.curv, st.cells, st.ncell,
                                               st.L, st.P, st.rk_weight2);
        else
            k_mp_step<false><<<nb, 128, 0, s>>>(f, gg, st.phi, st.cnx, st.cny, st.cnz, st.cnorm, st.curv, st.cells,
                                                st.ncell, st.L, st.P, st.rk_weight2);
        return 1;
    }
    switch (st.prec) {
        case MFLBM_FP32: return collide_t<float>(st, odd, s);
        case MFLBM_FP16: return collide_t<__half>(st, odd, s);
        default: return collide_t<double>(st, odd, s);
    }
}

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
    if (!(st.P.iper || st.P.jper || st.P.kper)) return 0;
    int n_launch;
    switch (st.multiphase ? MFLBM_FP64 : st.prec) {
        case MFLBM_FP32: n_launch = wrap_t<float>(st, pull, s); break;
        case MFLBM_FP16: n_launch = wrap_t<__half>(st, pull, s); break;
        default: n_launch = wrap_t<double>(st, pull, s); break;
    }
    if (st.multiphase && (st.P.jper || st.P.kper)) {
        const Layout &L = st.L;
        const int64_t n = (st.P.kper ? (int64_t)4 * L.nx * L.ny : 0) + (st.P.jper ? (int64_t)4 * L.nx * L.nz : 0) +
                          ((st.P.jper && st.P.kper) ? (int64_t)16 * L.nx : 0);
        k_wrap_phi<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st.phi, L, st.P.jper, st.P.kper);
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
    const int bo = before_odd ? 1 : 0;
    if (open_z) {
        if (inlet_bc == 1)
            k_inlet_velocity<S><<<g, b, 0, s>>>(f, gg, st.phi, st.walls, st.w_in, L, st.P, bo, st.multiphase, st.ref, st.scale);
        else if (inlet_bc == 2)
            k_inlet_zouhe<S><<<g, b, 0, s>>>(f, gg, st.phi, st.walls, L, st.P, bo, st.multiphase, st.ref, st.scale);
        if (outlet_bc == 1)
            k_outlet_convective<S><<<g, b, 0, s>>>(f, gg, st.phi, st.fconv, st.gconv, st.phiconv, st.walls, L, st.P, bo,
                                                   st.multiphase, st.ref, st.scale);
        else if (outlet_bc == 2)
            k_outlet_zouhe<S><<<g, b, 0, s>>>(f, gg, st.phi, st.walls, L, st.P, bo, st.multiphase, st.ref, st.scale);
        n_launch += (inlet_bc == 1 || inlet_bc == 2) + (outlet_bc == 1 || outlet_bc == 2);
    }
    return n_launch;
}

int boundary(const DevState &st, bool before_odd, int inlet_bc, int outlet_bc, bool open_z, cudaStream_t s) {
    int n_launch;
    switch (st.multiphase ? MFLBM_FP64 : st.prec) {
        case MFLBM_FP32: n_launch = boundary_t<float>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
        case MFLBM_FP16: n_launch = boundary_t<__half>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
        default: n_launch = boundary_t<double>(st, before_odd, inlet_bc, outlet_bc, open_z, s); break;
    }
    if (st.multiphase && st.P.porous_plate_cmd != 0 && st.P.z_porous_plate >= 1 && st.P.z_porous_plate <= st.L.nz) {
        const Layout &L = st.L;
        const int bx = L.nx >= 128 ? 128 : ((L.nx + 31) / 32) * 32;
        double *f = fs<double>(st), *gg = gs<double>(st);
        double *blocked = st.P.porous_plate_cmd == 1 ? f : gg;
        double *passing = st.P.porous_plate_cmd == 1 ? gg : f;
        k_porous_plate<<<dim3((L.nx + bx - 1) / bx, L.ny), bx, 0, s>>>(blocked, passing, L, st.P.z_porous_plate,
                                                                        before_odd ? 1 : 0);
        ++n_launch;
    }
    return n_launch;
}

int color_gradient(const DevState &st, cudaStream_t s) {
    if (!st.multiphase) return 0;
    const Layout &L = st.L;
    int n_launch = 2 + (st.ns > 0 ? 2 : 0) + (st.nf > 0 ? 1 : 0);
    if (st.ns > 0) k_extrap_phi<<<(st.ns + 127) / 128, 128, 0, s>>>(st.phi, st.sb, st.ns, L);
    {
        const int nxh = L.nx + 4;
        const int bx = nxh >= 128 ? 128 : ((nxh + 31) / 32) * 32;
        const dim3 b(bx, 256 / bx > 0 ? (unsigned)(256 / bx) : 1u);
        const dim3 g((nxh + b.x - 1) / b.x, (L.ny + 4 + b.y - 1) / b.y, L.nz + 4);
        k_normals<<<g, b, 0, s>>>(st.phi, st.walls, st.cnx, st.cny, st.cnz, st.cnorm, L);
    }
    if (st.nf > 0) k_wetting<<<(st.nf + 127) / 128, 128, 0, s>>>(st.cnx, st.cny, st.cnz, st.cnorm, st.fb, st.nf, L);
    if (st.ns > 0) k_extrap_normals<<<(st.ns + 127) / 128, 128, 0, s>>>(st.cnx, st.cny, st.cnz, st.sb, st.ns, L);
    {
        const int bx = L.nx >= 128 ? 128 : ((L.nx + 31) / 32) * 32;
        const dim3 b(bx, 256 / bx);
        const dim3 g((L.nx + b.x - 1) / b.x, (L.ny + b.y - 1) / b.y, L.nz);
        k_curvature<<<g, b, 0, s>>>(st.cnx, st.cny, st.cnz, st.curv, st.walls, L);
    }
    return n_launch;
}

template <class S>
int monitor_t(const DevState &st, cudaStream_t s) {
    k_monitor<S><<<st.L.nz, MON_THREADS, 0, s>>>(fs<S>(st), st.multiphase ? gs<S>(st) : nullptr, st.phi, st.walls, st.cnx,
                                                 st.cny, st.cnz, st.cnorm, st.curv, st.u, st.v, st.w, st.rho, st.mon, st.L,
                                                 st.P, st.multiphase, 1, st.ref, st.scale);
    return 1;
}

int monitor(const DevState &st, cudaStream_t s) {
    switch (st.multiphase ? MFLBM_FP64 : st.prec) {
        case MFLBM_FP32: return monitor_t<float>(st, s);
        case MFLBM_FP16: return monitor_t<__half>(st, s);
        default: return monitor_t<double>(st, s);
    }
}

int saturation(const DevState &st, cudaStream_t s) {
    if (!st.multiphase) return 0;
    k_saturation<<<st.L.nz, MON_THREADS, 0, s>>>(st.phi, st.walls, st.mon, st.L);
    return 1;
}

template <class S>
int init_t(const DevState &st, bool convec, cudaStream_t s) {
    const Layout &L = st.L;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    S *g = st.multiphase ? gs<S>(st) : nullptr;
    k_init_eq<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(fs<S>(st), g, st.phi, st.u, st.v, st.w, st.rho, L,
                                                              st.multiphase, st.ref, st.scale);
    if (convec) {
        const int64_t np = (int64_t)(L.nx + 2) * (L.ny + 2);
        k_init_convec<S><<<(unsigned)((np + 255) / 256), 256, 0, s>>>(fs<S>(st), g, st.phi, st.fconv, st.gconv, st.phiconv,
                                                                      L, st.multiphase, st.ref, st.scale);
        return 2;
    }
    return 1;
}

int init_equilibrium(const DevState &st, bool convec, cudaStream_t s) {
    switch (st.multiphase ? MFLBM_FP64 : st.prec) {
        case MFLBM_FP32: return init_t<float>(st, convec, s);
        case MFLBM_FP16: return init_t<__half>(st, convec, s);
        default: return init_t<double>(st, convec, s);
    }
}

template <class S>
int convert_in_t(const DevState &st, int sp, int q, cudaStream_t s) {
    const Layout &L = st.L;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    S *base = (sp == 0 ? fs<S>(st) : gs<S>(st)) + (int64_t)q * L.qs;
    k_convert_in<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(base, st.stage, L, q, st.ref, st.scale);
    return 1;
}

template <class S>
int convert_out_t(const DevState &st, int sp, int q, cudaStream_t s) {
    const Layout &L = st.L;
    const int64_t nb = (int64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const S *base = (sp == 0 ? fs<S>(st) : gs<S>(st)) + (int64_t)q * L.qs;
    k_convert_out<S><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(st.stage, base, L, q, st.ref, st.scale);
    return 1;
}

int convert_in(const DevState &st, int sp, int q, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return convert_in_t<float>(st, sp, q, s);
        case MFLBM_FP16: return convert_in_t<__half>(st, sp, q, s);
        default: return convert_in_t<double>(st, sp, q, s);
    }
}

int convert_out(const DevState &st, int sp, int q, cudaStream_t s) {
    switch (st.prec) {
        case MFLBM_FP32: return convert_out_t<float>(st, sp, q, s);
        case MFLBM_FP16: return convert_out_t<__half>(st, sp, q, s);
        default: return convert_out_t<double>(st, sp, q, s);
    }
}

const KernelTable table = {collide, wrap, boundary, color_gradient, monitor, saturation, init_equilibrium, convert_in, convert_out};

}  // namespace MFLBM_NS
}  // namespace mflbm
