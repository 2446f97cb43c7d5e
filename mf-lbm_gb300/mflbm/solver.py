"""Python host mirror of the per-step interface (the calls a Fortran host makes).

``Solver`` owns one libmflbm context.  Its methods map one-to-one onto the C ABI
(include/mflbm.h) and take numpy arrays in the reference's halo'd layouts:

  f, g      float64 (19, nz+2, ny+2, nx+2)   f0..f18 / g0..g18, halo 1
  phi       float64 (nz+8, ny+8, nx+8)       halo 4
  walls     int8    (nz+4, ny+4, nx+4)       halo 2
  w_in      float64 (ny+2, nx+2)
  convec    float64 (19, ny+2, nx+2), phi_convec (ny+2, nx+2)
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import MFLBM_ABI_VERSION, Params


def make_params(**kw):
    """mflbm_params with the reference's template defaults, overridden by kw.

    precision: MFLBM_FP64 (0, the drop-in), MFLBM_FP32 (1), MFLBM_FP16 (2, singlephase),
    MFLBM_FP64FF (3, FP64 storage with the double-word collision), MFLBM_FF (4,
    double-word storage); layout: 0 auto, 1 dense, 2 fluid list (singlephase)."""
    p = Params()
    p.abi_version = MFLBM_ABI_VERSION
    defaults = dict(multiphase=0, nx=16, ny=16, nz=16, iper=0, jper=0, kper=0, wall_x_min=1, wall_x_max=1,
                    wall_y_min=1, wall_y_max=1, wall_z_min=0, wall_z_max=0, inlet_bc=0, outlet_bc=0, mrt=2,
                    porous_plate_cmd=0, z_porous_plate=0, precision=0, strict_fp=0, device=0, la_nu1=1.0 / 6.0,
                    la_nu2=1.0 / 6.0, gamma=0.01, beta=0.95, sa_inject=1.0, force_z=0.0, uin_avg=0.0, rho_in=1.0,
                    rho_out=1.0, relaxation=1.0)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _ptr_array(arr):
    """19 plane pointers of a (19, ...) contiguous array as a void*[19]."""
    if arr is None:
        return None, None
    arr = np.ascontiguousarray(arr)
    ptrs = (C.c_void_p * 19)(*[arr[q].ctypes.data for q in range(19)])
    return ptrs, arr


class Solver:
    def __init__(self, params, lib=None):
        self.lib = lib or _capi.load()
        self.p = params
        self.nx, self.ny, self.nz = params.nx, params.ny, params.nz
        self.multiphase = bool(params.multiphase)
        h = C.c_void_p()
        rc = self.lib.mflbm_create(C.byref(params), C.byref(h))
        _capi.check(self.lib, None, rc)
        self.ctx = h

    @property
    def layout(self):
        """LAYOUT_DENSE or LAYOUT_LIST once the geometry is set (LAYOUT_AUTO before)."""
        return self.lib.mflbm_layout(self.ctx)

    # --- shapes -------------------------------------------------------------------
    def shape1(self):
        return (self.nz + 2, self.ny + 2, self.nx + 2)

    def shape2(self):
        return (self.nz + 4, self.ny + 4, self.nx + 4)

    def shape4(self):
        return (self.nz + 8, self.ny + 8, self.nx + 8)

    def _check(self, rc):
        return _capi.check(self.lib, self.ctx, rc)

    # --- setup --------------------------------------------------------------------
    def set_geometry(self, walls, solid=None, fluid=None, w_in=None):
        walls = np.ascontiguousarray(walls, dtype=np.int8)
        assert walls.shape == self.shape2()
        ns = 0 if solid is None else int(solid.size)
        nf = 0 if fluid is None else int(fluid.size)
        solid = None if solid is None else np.ascontiguousarray(solid)
        fluid = None if fluid is None else np.ascontiguousarray(fluid)
        if w_in is not None:
            w_in = np.ascontiguousarray(w_in, dtype=np.float64)
            assert w_in.shape == (self.ny + 2, self.nx + 2)
        self._check(self.lib.mflbm_set_geometry(self.ctx, _ptr(walls), _ptr(solid) if ns else None, ns,
                                                _ptr(fluid) if nf else None, nf, _ptr(w_in)))

    def init_equilibrium(self, phi=None):
        if phi is not None:
            phi = np.ascontiguousarray(phi, dtype=np.float64)
            assert phi.shape == self.shape4()
        self._check(self.lib.mflbm_init_equilibrium(self.ctx, _ptr(phi)))

    def init_velocity(self, u=None, v=None, w=None, rho=None, rest_base=True):
        """State from density and velocity fields: interior arrays (nz, ny, nx) or halo-1
        arrays; the ghost layer of interior arrays is filled periodically."""
        arrs = []
        for a in (rho, u, v, w):
            if a is None:
                arrs.append(None)
                continue
            a = np.asarray(a, dtype=np.float64)
            if a.shape == (self.nz, self.ny, self.nx):
                a = np.pad(a, 1, mode="wrap")
            assert a.shape == self.shape1()
            arrs.append(np.ascontiguousarray(a))
        self._check(self.lib.mflbm_init_velocity(self.ctx, *[_ptr(a) for a in arrs], int(bool(rest_base))))

    def upload_state(self, f, g=None, phi=None, f_convec=None, g_convec=None, phi_convec=None):
        fp, f = _ptr_array(f)
        gp, g = _ptr_array(g)
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (phi, f_convec, g_convec, phi_convec)]
        self._check(self.lib.mflbm_upload_state(self.ctx, fp, gp, *[_ptr(a) for a in arrs]))

    def download_state(self):
        f = np.empty((19,) + self.shape1())
        fp, _ = _ptr_array(f)
        g = gp = phi = gc = pc = None
        if self.multiphase:
            g = np.empty((19,) + self.shape1())
            gp, _ = _ptr_array(g)
            phi = np.empty(self.shape4())
            gc = np.empty((19, self.ny + 2, self.nx + 2))
            pc = np.empty((self.ny + 2, self.nx + 2))
        fc = np.empty((19, self.ny + 2, self.nx + 2))
        self._check(self.lib.mflbm_download_state(self.ctx, fp, gp, _ptr(phi), _ptr(fc), _ptr(gc), _ptr(pc)))
        out = {"f": f, "f_convec": fc}
        if self.multiphase:
            out.update(g=g, phi=phi, g_convec=gc, phi_convec=pc)
        return out

    # --- time stepping ------------------------------------------------------------
    def step(self, ntime):
        self._check(self.lib.mflbm_step(self.ctx, ntime))

    def run(self, ntime0, nsteps):
        self._check(self.lib.mflbm_run(self.ctx, ntime0, nsteps))

    def synchronize(self):
        self._check(self.lib.mflbm_synchronize(self.ctx))

    def color_gradient(self):
        self._check(self.lib.mflbm_color_gradient(self.ctx))

    def get_gradient(self):
        s2, s1 = self.shape2(), self.shape1()
        cx, cy, cz, cn = (np.empty(s2) for _ in range(4))
        cv = np.empty(s1)
        self._check(self.lib.mflbm_get_gradient(self.ctx, _ptr(cx), _ptr(cy), _ptr(cz), _ptr(cn), _ptr(cv)))
        return {"cn_x": cx, "cn_y": cy, "cn_z": cz, "c_norm": cn, "curv": cv}

    # --- diagnostics --------------------------------------------------------------
    def macro(self):
        s1 = self.shape1()
        u, v, w, rho = (np.empty(s1) for _ in range(4))
        phi = np.empty(self.shape4()) if self.multiphase else None
        self._check(self.lib.mflbm_macro(self.ctx, _ptr(u), _ptr(v), _ptr(w), _ptr(rho), _ptr(phi)))
        out = {"u": u, "v": v, "w": w, "rho": rho}
        if self.multiphase:
            out["phi"] = phi
        return out

    def monitor(self):
        nq = 7 if self.multiphase else 2
        prof = np.empty(nq * self.nz)
        scal = np.empty(3)
        st = C.c_int32()
        self._check(self.lib.mflbm_monitor(self.ctx, _ptr(prof), _ptr(scal), C.byref(st)))
        return prof.reshape(nq, self.nz), scal, st.value

    def steady_monitor(self, kind):
        """mflbm_steady_monitor: 0 snapshot phi_old, 1 capillary pressure (pc, pre_w, pre_nw,
        umax, count_w, count_nw), 2 phase-field change (d_phi_max, umax), 3 breakthrough
        count at z = nz - 1."""
        out = np.zeros(6)
        self._check(self.lib.mflbm_steady_monitor(self.ctx, kind, _ptr(out)))
        return out[:{0: 0, 1: 6, 2: 2, 3: 1}[kind]]

    def change_inlet_fluid_phase(self, cmd, interface_z0):
        """change_inlet_fluid_phase: cmd 1 moves species 2 into species 1 for z <= interface_z0,
        cmd 2 the reverse (0 does nothing)."""
        self._check(self.lib.mflbm_change_inlet_fluid_phase(self.ctx, int(cmd), float(interface_z0)))

    def saturation(self):
        a, b = C.c_double(), C.c_double()
        self._check(self.lib.mflbm_saturation(self.ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_profiling(self, enable):
        self._check(self.lib.mflbm_set_profiling(self.ctx, 1 if enable else 0))

    def get_profile(self):
        rg, ms, n, k = C.c_double(), C.c_double(), C.c_int64(), C.c_int64()
        self._check(self.lib.mflbm_get_profile(self.ctx, C.byref(rg), C.byref(ms), C.byref(n), C.byref(k)))
        return {"region_ms": rg.value, "collide_ms": ms.value, "collide_launches": n.value, "kernel_launches": k.value}

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.mflbm_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
