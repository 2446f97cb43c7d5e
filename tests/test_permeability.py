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
