"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Mirrors mflbm.Solver method for method, so a test can drive the GPU library and the
oracle with the same calls and compare every array.  Only tests/, the smoke check and
bench.py's CPU-baseline leg import this module.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mflbm_oracle_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_build = _load_build()

_libs = {}


def load(variant="strict"):
    name = f"liborc_{variant}.so"
    if name in _libs:
        return _libs[name]
    path = _build.lib_path(name)
    if not os.path.exists(path):
        _build.build()
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "orc_create": (C.c_int32, [P, C.POINTER(C.c_void_p)]),
        "orc_destroy": (None, [P]),
        "orc_last_error": (C.c_char_p, [P]),
        "orc_set_geometry": (C.c_int32, [P, P, P, C.c_int32, P, C.c_int32, P]),
        "orc_upload_state": (C.c_int32, [P, P, P, P, P, P, P]),
        "orc_download_state": (C.c_int32, [P, P, P, P, P, P, P]),
        "orc_init_equilibrium": (C.c_int32, [P, P]),
        "orc_step": (C.c_int32, [P, C.c_int32]),
        "orc_run": (C.c_int32, [P, C.c_int32, C.c_int32]),
        "orc_color_gradient": (C.c_int32, [P]),
        "orc_get_gradient": (C.c_int32, [P, P, P, P, P, P]),
        "orc_macro": (C.c_int32, [P, P, P, P, P, P]),
        "orc_monitor": (C.c_int32, [P, P, P, P]),
        "orc_saturation": (C.c_int32, [P, P, P]),
        "orc_steady_monitor": (C.c_int32, [P, C.c_int32, P]),
        "orc_change_inlet_fluid_phase": (C.c_int32, [P, C.c_int32, C.c_double]),
        "orc_set_threads": (C.c_int32, [C.c_int32]),
        "orc_set_walls": (C.c_int64, [P, P, P]),
        "orc_geometry_preprocess": (C.c_int32, [P, P, C.c_double, P, P, P, P]),
        "orc_inlet_profile": (None, [C.c_int32, C.c_int32, C.c_double, C.c_int32, P]),
    }
    for k, (r, a) in sig.items():
        fn = getattr(lib, k)
        fn.restype = r
        fn.argtypes = a
    _libs[name] = lib
    return lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _ptrs(arr):
    if arr is None:
        return None
    return (C.c_void_p * 19)(*[arr[q].ctypes.data for q in range(19)])


class OracleError(RuntimeError):
    pass


class Oracle:
    """Same interface as mflbm.Solver, computed by the C++ restatement."""

    def __init__(self, params, variant="strict", threads=0):
        self.lib = load(variant)
        if threads:
            self.lib.orc_set_threads(threads)
        self.p = params
        self.nx, self.ny, self.nz = params.nx, params.ny, params.nz
        self.multiphase = bool(params.multiphase)
        h = C.c_void_p()
        rc = self.lib.orc_create(C.cast(C.pointer(params), C.c_void_p), C.byref(h))
        if rc:
            raise OracleError(f"{rc}: {self.lib.orc_last_error(None).decode()}")
        self.h = h

    def _check(self, rc):
        if rc:
            raise OracleError(f"{rc}: {self.lib.orc_last_error(self.h).decode()}")

    def shape1(self):
        return (self.nz + 2, self.ny + 2, self.nx + 2)

    def shape2(self):
        return (self.nz + 4, self.ny + 4, self.nx + 4)

    def shape4(self):
        return (self.nz + 8, self.ny + 8, self.nx + 8)

    def set_geometry(self, walls, solid=None, fluid=None, w_in=None):
        walls = np.ascontiguousarray(walls, dtype=np.int8)
        ns = 0 if solid is None else int(solid.size)
        nf = 0 if fluid is None else int(fluid.size)
        solid = None if solid is None else np.ascontiguousarray(solid)
        fluid = None if fluid is None else np.ascontiguousarray(fluid)
        w_in = None if w_in is None else np.ascontiguousarray(w_in, dtype=np.float64)
        self._check(self.lib.orc_set_geometry(self.h, _ptr(walls), _ptr(solid) if ns else None, ns,
                                              _ptr(fluid) if nf else None, nf, _ptr(w_in)))

    def init_equilibrium(self, phi=None):
        phi = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        self._check(self.lib.orc_init_equilibrium(self.h, _ptr(phi)))

    def upload_state(self, f, g=None, phi=None, f_convec=None, g_convec=None, phi_convec=None):
        f = np.ascontiguousarray(f)
        g = None if g is None else np.ascontiguousarray(g)
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (phi, f_convec, g_convec, phi_convec)]
        self._check(self.lib.orc_upload_state(self.h, _ptrs(f), _ptrs(g), *[_ptr(a) for a in arrs]))

    def download_state(self):
        f = np.empty((19,) + self.shape1())
        fc = np.empty((19, self.ny + 2, self.nx + 2))
        g = phi = gc = pc = None
        if self.multiphase:
            g = np.empty((19,) + self.shape1())
            phi = np.empty(self.shape4())
            gc = np.empty((19, self.ny + 2, self.nx + 2))
            pc = np.empty((self.ny + 2, self.nx + 2))
        self._check(self.lib.orc_download_state(self.h, _ptrs(f), _ptrs(g), _ptr(phi), _ptr(fc), _ptr(gc), _ptr(pc)))
        out = {"f": f, "f_convec": fc}
        if self.multiphase:
            out.update(g=g, phi=phi, g_convec=gc, phi_convec=pc)
        return out

    def step(self, ntime):
        self._check(self.lib.orc_step(self.h, ntime))

    def run(self, ntime0, nsteps):
        self._check(self.lib.orc_run(self.h, ntime0, nsteps))

    def synchronize(self):
        pass

    def color_gradient(self):
        self._check(self.lib.orc_color_gradient(self.h))

    def get_gradient(self):
        s2, s1 = self.shape2(), self.shape1()
        cx, cy, cz, cn = (np.empty(s2) for _ in range(4))
        cv = np.empty(s1)
        self._check(self.lib.orc_get_gradient(self.h, _ptr(cx), _ptr(cy), _ptr(cz), _ptr(cn), _ptr(cv)))
        return {"cn_x": cx, "cn_y": cy, "cn_z": cz, "c_norm": cn, "curv": cv}

    def macro(self):
        s1 = self.shape1()
        u, v, w, rho = (np.empty(s1) for _ in range(4))
        phi = np.empty(self.shape4()) if self.multiphase else None
        self._check(self.lib.orc_macro(self.h, _ptr(u), _ptr(v), _ptr(w), _ptr(rho), _ptr(phi)))
        out = {"u": u, "v": v, "w": w, "rho": rho}
        if self.multiphase:
            out["phi"] = phi
        return out

    def monitor(self):
        nq = 7 if self.multiphase else 2
        prof = np.empty(nq * self.nz)
        scal = np.empty(3)
        st = C.c_int32()
        self._check(self.lib.orc_monitor(self.h, _ptr(prof), _ptr(scal), C.byref(st)))
        return prof.reshape(nq, self.nz), scal, st.value

    def saturation(self):
        a, b = C.c_double(), C.c_double()
        self._check(self.lib.orc_saturation(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def change_inlet_fluid_phase(self, cmd, interface_z0):
        self._check(self.lib.orc_change_inlet_fluid_phase(self.h, int(cmd), float(interface_z0)))

    def steady_monitor(self, kind):
        n = {0: 0, 1: 6, 2: 2, 3: 1}[kind]
        out = np.zeros(max(n, 1))
        self._check(self.lib.orc_steady_monitor(self.h, kind, _ptr(out)))
        return out[:n]

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# host-side setup restatements
def set_walls(params, walls_global):
    lib = load()
    wg = np.ascontiguousarray(walls_global, dtype=np.int8)
    out = np.zeros((params.nz + 4, params.ny + 4, params.nx + 4), dtype=np.int8)
    pore = lib.orc_set_walls(C.cast(C.pointer(params), C.c_void_p), _ptr(wg), _ptr(out))
    return out, int(pore)


def geometry_preprocess(params, walls_channel, theta_rad):
    sys.path.insert(0, os.path.join(HERE, "..", "mf-lbm_gb300"))
    from mflbm._capi import FLUID_DTYPE, SOLID_DTYPE
    lib = load()
    wc = np.ascontiguousarray(walls_channel, dtype=np.int8)
    ns, nf = C.c_int32(), C.c_int32()
    pp = C.cast(C.pointer(params), C.c_void_p)
    lib.orc_geometry_preprocess(pp, _ptr(wc), theta_rad, None, C.byref(ns), None, C.byref(nf))
    solid = np.zeros(ns.value, dtype=SOLID_DTYPE)
    fluid = np.zeros(nf.value, dtype=FLUID_DTYPE)
    lib.orc_geometry_preprocess(pp, _ptr(wc), theta_rad, _ptr(solid), C.byref(ns), _ptr(fluid), C.byref(nf))
    return solid, fluid


def inlet_profile(nx, ny, vel_avg, num_terms=1000):
    w = np.zeros((ny + 2, nx + 2))
    load().orc_inlet_profile(nx, ny, vel_avg, num_terms, _ptr(w))
    return w
