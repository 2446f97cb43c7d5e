"""Steady-state permeability of a body-force-driven singlephase run.

The reference stops a singlephase run once the relative change of the flow rate between
two monitor calls falls below ``convergence_criteria`` (singlephase_3D/0.src/
Monitor.F90:145-156), the flow rate being the slice sums of w averaged over z
(:30-43, 110-117).  It never computes a permeability.  Here

    u_mean = sum over all nx*ny*nz nodes of w / (nx*ny*nz)   (solid nodes contribute 0)
    k      = nu * u_mean / F_z                               (lattice units)

which is Darcy's law for a periodic sample driven by the body force F_z.  The slice sums
come from the device monitor reduction, which accumulates in FP64 in every storage
precision; u_mean and k are FP64 host sums of those slices.

``run_to_steady`` works with any object that has ``run(ntime0, nsteps)`` and
``monitor()`` (the GPU Solver or the CPU oracle).
"""
import dataclasses
import time

import numpy as np


@dataclasses.dataclass
class SteadyResult:
    k: float                  # permeability, lattice units
    u_mean: float             # mean z velocity over the whole lattice
    steps: int                # time steps taken
    seconds: float            # wall time of the loop (run + monitor), host clock
    converged: bool
    status: int               # monitor status of the last check (3 = NaN / unstable)
    history: list             # (steps, u_mean) at every check


def mean_velocity(sim, nx, ny, nz):
    """u_mean from the monitor's per-slice flow sums (valid after even steps)."""
    prof, _, status = sim.monitor()
    fl = np.asarray(prof[0], dtype=np.float64)
    return float(fl.sum()) / float(nx * ny * nz), int(status)


def permeability(u_mean, nu, force_z):
    return nu * u_mean / force_z


def run_to_steady(sim, params, check_every=100, tol=1e-7, max_steps=200000, ntime0=1, clock=time.perf_counter):
    """Run until |u_mean(t) - u_mean(t - check_every)| / |u_mean(t)| < tol.

    check_every must be even so that every check follows an even step, where the
    reference's compute_macro_vars is valid (multiphase_3D/0.src/Misc.F90:416-421).
    ntime0 is the ntime of the first step (odd for a state produced by an even step or
    by init_equilibrium)."""
    if check_every % 2:
        raise ValueError("check_every must be even")
    nx, ny, nz = params.nx, params.ny, params.nz
    hist = []
    prev = None
    steps = 0
    status = 0
    converged = False
    u = 0.0
    t0 = clock()
    while steps < max_steps:
        sim.run(ntime0 + steps, check_every)
        steps += check_every
        u, status = mean_velocity(sim, nx, ny, nz)
        hist.append((steps, u))
        if status != 0 or not np.isfinite(u):
            break
        if prev is not None and u != 0.0 and abs(u - prev) / abs(u) < tol:
            converged = True
            break
        prev = u
    dt = clock() - t0
    return SteadyResult(k=permeability(u, params.la_nu1, params.force_z), u_mean=u, steps=steps, seconds=dt,
                        converged=converged, status=status, history=hist)
