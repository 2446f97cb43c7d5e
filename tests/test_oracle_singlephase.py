"""Known-answer checks that pin the CPU oracle's singlephase path.

The reference ships no golden vectors, so the oracle is pinned by physics its own
decks rely on: a rest state stays at rest, mass is conserved in a periodic box, and
body-force-driven channel flow between bounce-back walls reaches the parabolic
profile with the wall halfway between the last fluid and the first solid node
(exact for the MRT "bounce-back optimised" rates, Initialization.F90:91-97).
"""
import numpy as np
import pytest

from cases import W, sp_case
from mflbm import geometry
from mflbm.solver import make_params
from pyoracle import Oracle


def _run(case, steps):
    o = Oracle(case["params"])
    o.set_geometry(case["walls"], None, None, case["w_in"])
    o.upload_state(case["f"], f_convec=case["f_convec"])
    o.run(1, steps)
    return o


# Rest state of the reference MRT.  Its equilibrium energy-square moment is
# mrt_e2_coef1*rho = 0 (Module.F90:120), so the rest distribution is not the BGK
# weights: back-transforming (rho=1, e=-11, all else 0) gives 4/21, 13/126, 1/63.
W_MRT = np.array([4.0 / 21.0] + [13.0 / 126.0] * 6 + [1.0 / 63.0] * 12)


def test_rest_state_stays_at_rest():
    case = sp_case(nx=8, ny=9, nz=10, per=(1, 1, 1), force=0.0, spheres=2)
    shape1 = case["f"].shape[1:]
    case["f"] = np.broadcast_to(W_MRT[:, None, None, None], (19,) + shape1).copy()
    o = _run(case, 10)  # ends after step 10 (even): natural order
    f = o.download_state()["f"]
    fluid = case["walls"][1:-1, 1:-1, 1:-1] == 0
    for q in range(19):
        np.testing.assert_allclose(f[q][fluid], W_MRT[q], rtol=1e-14)


def test_bgk_weights_relax_to_mrt_rest_state():
    # the reference initialises with the BGK equilibrium (Initialization.F90:255-273);
    # the MRT then drives it to its own rest state
    case = sp_case(nx=6, ny=6, nz=6, per=(1, 1, 1), force=0.0, spheres=0)
    shape1 = case["f"].shape[1:]
    case["f"] = np.broadcast_to(W[:, None, None, None], (19,) + shape1).copy()
    o = _run(case, 200)
    f = o.download_state()["f"]
    for q in range(19):
        np.testing.assert_allclose(f[q][1:-1, 1:-1, 1:-1], W_MRT[q], rtol=1e-12)


OPC = [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]
EXYZ = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (-1, 1, 0),
        (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1), (-1, 0, -1), (0, 1, 1), (0, -1, 1), (0, 1, -1),
        (0, -1, -1)]


def total_mass_even(f, walls, n):
    """Mass after an even step: every fluid node's own slots plus, for every fluid->solid
    link, the population emitted into the solid node at the previous odd step (AA-pattern
    full-way bounce-back keeps it in the solid node's opposite slot for one step).
    Periodic links are followed through the halo, whose values the push copied back."""
    nx, ny, nz = n
    wi = walls[1:-1, 1:-1, 1:-1]        # halo-1 box view of the halo-2 walls
    fl = wi[1:-1, 1:-1, 1:-1] == 0      # interior fluid
    m = sum(f[q][1:-1, 1:-1, 1:-1][fl].sum() for q in range(19))
    ks, js, is_ = np.nonzero(fl)
    for q in range(1, 19):
        ex, ey, ez = EXYZ[q]
        # neighbour in halo-1 array coordinates, wrapped onto the interior image
        kk = (ks + ez) % nz + 1
        jj = (js + ey) % ny + 1
        ii = (is_ + ex) % nx + 1
        solid = wi[ks + 1 + ez, js + 1 + ey, is_ + 1 + ex] != 0
        m += f[OPC[q]][kk[solid], jj[solid], ii[solid]].sum()
    return m


def test_mass_conserved_fully_periodic():
    case = sp_case(nx=10, ny=9, nz=11, per=(1, 1, 1), force=1e-4, spheres=3, seed=5)
    o = Oracle(case["params"])
    o.set_geometry(case["walls"])
    o.upload_state(case["f"])
    m0 = None
    for n in range(1, 15):
        o.step(n)
        if n % 2 == 0:
            m = total_mass_even(o.download_state()["f"], case["walls"], (10, 9, 11))
            if m0 is None:
                m0 = m
            assert abs(m - m0) <= 1e-13 * m0


def test_poiseuille_channel_profile():
    # walls at x=1 and x=nx (fluid 2..nx-1), periodic y, z; body force along z
    nx, ny, nz = 10, 3, 3
    nu, fz = 1.0 / 6.0, 1e-6
    p = make_params(multiphase=0, nx=nx, ny=ny, nz=nz, iper=0, jper=1, kper=1, wall_y_min=0, wall_y_max=0,
                    mrt=1, la_nu1=nu, force_z=fz, strict_fp=1)
    walls, pore, _ = geometry.set_walls(p, np.zeros((nz, ny, nx), np.int8))
    o = Oracle(p)
    o.set_geometry(walls)
    o.init_equilibrium()
    o.run(1, 4000)
    w = o.macro()["w"][1:-1, 1:-1, 1:-1]  # (nz, ny, nx) interior
    x = np.arange(1, nx + 1, dtype=float)
    x0, x1 = 1.5, nx - 0.5
    exact = fz / (2.0 * nu) * (x - x0) * (x1 - x)
    prof = w[1, 1, 1:-1]
    np.testing.assert_allclose(prof, exact[1:-1], rtol=1e-8)


def test_duct_inlet_profile_matches_oracle_restatement():
    from pyoracle import inlet_profile
    for nx, ny in [(12, 12), (16, 10), (64, 64)]:
        a = geometry.inlet_profile(nx, ny, 1e-4)
        b = inlet_profile(nx, ny, 1e-4)
        np.testing.assert_allclose(a, b, rtol=2e-14, atol=1e-22)
        # mean over the open cross-section equals the prescribed average velocity
        inner = a[2:ny, 2:nx]
        assert abs(inner.sum() / ((nx - 2) * (ny - 2)) - 1e-4) < 2e-6


def test_velocity_inlet_convective_outlet_runs_stable():
    case = sp_case(nx=12, ny=12, nz=16, per=(0, 0, 0), inlet=1, outlet=1, force=0.0, spheres=2, uin=1e-3)
    o = _run(case, 40)
    prof, scal, status = o.monitor()
    assert status == 0
    assert np.isfinite(prof).all()
    # the inlet drives +z flow through every slice
    assert (prof[0][2:-2] > 0).all()
