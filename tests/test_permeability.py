"""Steady-state permeability (CPU, oracle): plane Poiseuille channel, analytic k."""
import numpy as np
import pytest

from mflbm import geometry
from mflbm.permeability import permeability, run_to_steady
from mflbm.solver import make_params
from pyoracle import Oracle


def test_channel_permeability_is_analytic():
    # solid planes at x=1 and x=nx in an otherwise periodic box; halfway bounce-back puts
    # the walls at x=1.5 and x=nx-0.5, so h = nx-2.  The node values of the parabola
    # F/(2 nu) (x-1.5)(nx-0.5-x) summed over the h fluid columns give F/(2 nu) (h^3/6 + h/12),
    # hence k = (h^3 + h/2) / (12 nx).  tau=1 with s_q = 8(2-s)/(8-s) makes the wall
    # location exact, so the lattice solution is the parabola to rounding.
    nx, ny, nz = 10, 3, 4
    nu, fz = 1.0 / 6.0, 1e-6
    p = make_params(multiphase=0, nx=nx, ny=ny, nz=nz, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                    wall_y_min=0, wall_y_max=0, mrt=1, la_nu1=nu, force_z=fz)
    wg = np.zeros((nz, ny, nx), np.int8)
    wg[:, :, 0] = 1
    wg[:, :, -1] = 1
    walls, pore, _ = geometry.set_walls(p, wg)
    o = Oracle(p, variant="fast")
    o.set_geometry(walls)
    o.init_equilibrium()
    res = run_to_steady(o, p, check_every=200, tol=1e-12, max_steps=40000)
    o.close()
    assert res.converged and res.status == 0
    h = nx - 2
    np.testing.assert_allclose(res.k, (h ** 3 + 0.5 * h) / (12.0 * nx), rtol=1e-8)
    assert res.history[-1][1] == res.u_mean
    assert permeability(res.u_mean, nu, fz) == res.k


def test_check_interval_must_be_even():
    with pytest.raises(ValueError):
        run_to_steady(None, make_params(multiphase=0), check_every=101)


class _FakeSim:
    """run() advances a scripted mean velocity; monitor() reports it as one slice sum."""

    def __init__(self, us, status_at=None, nx=2, ny=2, nz=1):
        self.us, self.i, self.status_at, self.n = list(us), 0, status_at, nx * ny * nz
        self.calls = []

    def run(self, ntime0, nsteps):
        self.calls.append((ntime0, nsteps))
        self.i += 1

    def monitor(self):
        u = self.us[min(self.i, len(self.us)) - 1]
        st = 3 if self.status_at is not None and self.i >= self.status_at else 0
        return np.array([[u * self.n], [0.0]]), np.zeros(3), st


def test_stopping_rule_and_failure_paths():
    p = make_params(multiphase=0, nx=2, ny=2, nz=1, la_nu1=1.0 / 6.0, force_z=1e-6)
    # relative change below tol between two checks: stops at the third check
    sim = _FakeSim([1.0, 1.1, 1.1 + 1e-9, 9.0])
    r = run_to_steady(sim, p, check_every=100, tol=1e-7, max_steps=10000)
    assert r.converged and r.steps == 300 and r.status == 0
    assert sim.calls == [(1, 100), (101, 100), (201, 100)]
    assert r.k == permeability(1.1 + 1e-9, 1.0 / 6.0, 1e-6)
    # the instability status of the monitor (NaN or |u| > 0.5) ends the run unconverged
    r = run_to_steady(_FakeSim([1.0, 2.0, 3.0], status_at=2), p, check_every=100, tol=1e-7, max_steps=10000)
    assert not r.converged and r.status == 3 and r.steps == 200
    # a NaN mean velocity ends it too
    r = run_to_steady(_FakeSim([1.0, float("nan")]), p, check_every=100, tol=1e-7, max_steps=10000)
    assert not r.converged and r.steps == 200
    # the step cap
    r = run_to_steady(_FakeSim([1.0, 2.0, 4.0, 8.0, 16.0]), p, check_every=100, tol=1e-7, max_steps=400)
    assert not r.converged and r.steps == 400 and len(r.history) == 4
