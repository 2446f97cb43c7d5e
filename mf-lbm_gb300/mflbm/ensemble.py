"""Ensembles of singlephase samples through the C ABI (mflbm_ensemble_*).

All samples of an Ensemble advance together in one fluid-list arena on one GPU; a
sample whose permeability has converged leaves the sweep.  The permeability of a sample
is k = nu * u_mean / F_z with u_mean = sum of w over its nx*ny*nz nodes / (nx*ny*nz),
as in mflbm.permeability.
"""
import ctypes as C
import dataclasses
import json
import os
import time

import numpy as np

from . import _capi

P = C.c_void_p


class Ensemble:
    """samples: list of (nx, ny, nz, walls_halo2) with walls as (nz+4, ny+4, nx+4) int8."""

    def __init__(self, params, samples, lib=None):
        self.lib = lib or _capi.load()
        self.p = params
        self.n = len(samples)
        self.dims = np.array([[s[0], s[1], s[2]] for s in samples], dtype=np.int32)
        self._walls = [np.ascontiguousarray(s[3], dtype=np.int8) for s in samples]
        for (nx, ny, nz), w in zip(self.dims, self._walls):
            assert w.shape == (nz + 4, ny + 4, nx + 4)
        ptrs = (C.c_void_p * self.n)(*[w.ctypes.data for w in self._walls])
        h = C.c_void_p()
        rc = self.lib.mflbm_ensemble_create(C.byref(params), self.n, self.dims.ctypes.data, ptrs, C.byref(h))
        if rc:
            raise _capi.MflbmError(rc, self.lib.mflbm_ensemble_last_error(None).decode())
        self.h = h
        self.volume = self.dims.prod(axis=1).astype(np.float64)

    def _check(self, rc):
        if rc:
            raise _capi.MflbmError(rc, self.lib.mflbm_ensemble_last_error(self.h).decode())

    def init(self):
        self._check(self.lib.mflbm_ensemble_init(self.h))

    def set_active(self, active):
        a = np.ascontiguousarray(active, dtype=np.int32)
        self._check(self.lib.mflbm_ensemble_set_active(self.h, a.ctypes.data))

    def run(self, ntime0, nsteps):
        self._check(self.lib.mflbm_ensemble_run(self.h, ntime0, nsteps))

    def flux(self):
        w = np.empty(self.n)
        um = np.empty(self.n)
        st = C.c_int32()
        self._check(self.lib.mflbm_ensemble_flux(self.h, w.ctypes.data, um.ctypes.data, C.byref(st)))
        return w, um, st.value

    def configure(self, block, persistent):
        self._check(self.lib.mflbm_ensemble_configure(self.h, block, int(bool(persistent))))

    def set_wait(self, spin_limit=0, unreachable=False):
        """Grid-barrier poll limit (0: default) and the unreachable-barrier hook of the
        timeout test; clears the barrier state."""
        self._check(self.lib.mflbm_ensemble_set_wait(self.h, int(spin_limit), int(bool(unreachable))))

    def tune(self, steps=10):
        buf = C.create_string_buffer(8192)
        self._check(self.lib.mflbm_ensemble_tune(self.h, steps, buf, len(buf)))
        return json.loads(buf.value.decode())

    def info(self):
        n = C.c_int64()
        b, pers, g = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.mflbm_ensemble_info(self.h, C.byref(n), C.byref(b), C.byref(pers), C.byref(g)))
        return {"active_nodes": n.value, "block": b.value, "persistent": pers.value, "grid": g.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.mflbm_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def tune_cached(ens, cache_path=None, steps=10):
    """Autotune once per (precision, arena size class) and reuse the choice from a JSON
    cache file; without cache_path the tuner simply runs."""
    key = f"prec{ens.p.precision}_nodes2^{int(np.log2(max(1, ens.info()['active_nodes'])))}"
    if cache_path and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
            if key in cache:
                ens.configure(cache[key]["block"], cache[key]["persistent"])
                return {"cached": True, "chosen": cache[key]}
        except (OSError, ValueError, KeyError):
            pass
    rep = ens.tune(steps)
    if cache_path:
        cache = {}
        if os.path.exists(cache_path):
            try:
                cache = json.load(open(cache_path))
            except (OSError, ValueError):
                cache = {}
        cache[key] = rep["chosen"]
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        with open(cache_path, "w") as fh:
            json.dump(cache, fh, indent=1)
    return rep


@dataclasses.dataclass
class EnsembleResult:
    k: np.ndarray            # permeability per sample
    steps: np.ndarray        # steps to convergence per sample
    converged: np.ndarray
    seconds: float           # wall time of the whole loop
    status: int
    fluid_updates: int       # fluid-node updates performed (sum over samples of nf * steps)


def run_to_steady(ens, nf, check_every=100, tol=1e-7, max_steps=200000, clock=time.perf_counter):
    """Run every sample until |du|/u < tol between checks, dropping converged samples.

    nf: fluid nodes per sample (for the update count)."""
    if check_every % 2:
        raise ValueError("check_every must be even")
    n = ens.n
    active = np.ones(n, dtype=np.int32)
    prev = np.full(n, np.nan)
    u = np.zeros(n)
    steps = np.zeros(n, dtype=np.int64)
    conv = np.zeros(n, dtype=bool)
    updates = 0
    status = 0
    t0 = clock()
    done = 0
    ens.set_active(active)
    while done < max_steps and active.any():
        ens.run(1 + done, check_every)
        done += check_every
        updates += int(np.sum(np.asarray(nf)[active.astype(bool)])) * check_every
        w, _, status = ens.flux()
        if status != 0:
            break
        cur = w / ens.volume
        left = False
        for s in np.nonzero(active)[0]:
            u[s] = cur[s]
            steps[s] = done
            if np.isfinite(prev[s]) and cur[s] != 0.0 and abs(cur[s] - prev[s]) / abs(cur[s]) < tol:
                conv[s] = True
                active[s] = 0
                left = True
            prev[s] = cur[s]
        if left:   # the device's tile table changes only when a sample has left it
            ens.set_active(active)
    secs = clock() - t0
    k = ens.p.la_nu1 * u / ens.p.force_z
    return EnsembleResult(k=k, steps=steps, converged=conv, seconds=secs, status=status, fluid_updates=updates)
