"""The singlephase fluid-list layout with an open z direction (inlet and outlet conditions):
the fluid nodes plus private slots for the cells of the planes the conditions address
(z = 0, 1, 2, nz-1, nz, nz+1), found through a slot map, against the dense planes and the
oracle.

The update is the dense layout's slot for slot, so in every storage form the fluid nodes'
populations and the convective-outlet memory are bit-identical to the dense layout after
1, 2, 3 and 8 steps (velocity and pressure inlets, convective and pressure outlets, walled
and periodic y, an open z without conditions); the monitor sums equal the dense layout's to
rtol 1e-12; the strict build equals the oracle; equilibrium and velocity initialisation
write the same fluid and boundary-plane values as the dense kernels.
"""
import copy

import numpy as np
import pytest

from cases import load_case, periodic_ghosts, sp_case
from mflbm import Solver
from mflbm._capi import LAYOUT_DENSE, LAYOUT_LIST
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "velocity_inlet_convective_outlet": dict(per=(0, 0, 0), inlet=1, outlet=1, force=0.0),
    "velocity_inlet_convective_periodic_y": dict(per=(0, 1, 0), inlet=1, outlet=1, force=0.0),
    "pressure_inlet_pressure_outlet": dict(per=(0, 0, 0), inlet=2, outlet=2, force=0.0),
    "pressure_bcs_periodic_y": dict(per=(0, 1, 0), inlet=2, outlet=2, force=0.0),
    "velocity_inlet_pressure_outlet": dict(per=(0, 1, 0), inlet=1, outlet=2, force=0.0),
    "open_z_without_conditions": dict(per=(0, 1, 0), force=1e-5),
    "ragged_velocity_inlet": dict(nx=9, ny=7, nz=11, per=(0, 1, 0), inlet=1, outlet=1, force=0.0, spheres=1),
}


def _case(name, strict=0, precision=0):
    kw = dict(CASES[name])
    c = sp_case(rest="mrt", strict=strict, precision=precision, **kw)
    # the list reads the periodic images where the dense step reads the uploaded ghosts
    c["f"] = periodic_ghosts(c["f"], kw["per"])
    return c


def _fluid(case):
    return case["walls"][2:-2, 2:-2, 2:-2] == 0


def _run(case, layout, steps):
    p = copy.copy(case["params"])
    p.layout = layout
    with Solver(p) as sim:
        load_case(sim, case)
        assert sim.layout == layout
        for n in range(1, steps + 1):
            sim.step(n)
        st = sim.download_state()
        mon = sim.monitor() if steps % 2 == 0 else None
    return st, mon


@pytest.mark.parametrize("precision", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("steps", [1, 2, 3, 8])
def test_list_equals_dense(name, steps, precision):
    case = _case(name, precision=precision)
    fl = _fluid(case)
    a = _run(case, LAYOUT_LIST, steps)
    b = _run(case, LAYOUT_DENSE, steps)
    x, y = a[0]["f"][:, 1:-1, 1:-1, 1:-1][:, fl], b[0]["f"][:, 1:-1, 1:-1, 1:-1][:, fl]
    assert np.array_equal(x, y), np.abs(x - y).max()
    assert np.array_equal(a[0]["f_convec"], b[0]["f_convec"])
    if a[1] is not None:
        np.testing.assert_allclose(a[1][0], b[1][0], rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(a[1][1], b[1][1], rtol=1e-12, atol=1e-300)
        assert a[1][2] == b[1][2]


@pytest.mark.parametrize("name", ["velocity_inlet_convective_outlet", "pressure_bcs_periodic_y",
                                  "velocity_inlet_pressure_outlet"])
def test_strict_list_equals_oracle(name):
    case = _case(name, strict=1)
    fl = _fluid(case)
    a, _ = _run(case, LAYOUT_LIST, 6)
    orc = Oracle(case["params"])
    load_case(orc, case)
    orc.run(1, 6)
    b = orc.download_state()
    orc.close()
    assert np.array_equal(a["f"][:, 1:-1, 1:-1, 1:-1][:, fl], b["f"][:, 1:-1, 1:-1, 1:-1][:, fl])
    assert np.array_equal(a["f_convec"], b["f_convec"])


@pytest.mark.parametrize("precision", [0, 1])
def test_initialisation_equals_dense(precision):
    """init_equilibrium (rest, convective memory from the outlet plane) and init_velocity
    (fluid nodes from their velocity, solid and boundary-plane cells as the dense kernel
    writes them) give the dense layout's fluid nodes and convective memory, before and
    after 4 steps."""
    case = _case("velocity_inlet_convective_periodic_y", precision=precision)
    fl = _fluid(case)
    nz, ny, nx = case["walls"].shape[0] - 4, case["walls"].shape[1] - 4, case["walls"].shape[2] - 4
    rng = np.random.default_rng(4)
    fields = [periodic_ghosts(a, (0, 1, 0)) for a in
              (1.0 + 1e-3 * rng.standard_normal((nz + 2, ny + 2, nx + 2)),
               *(1e-3 * rng.standard_normal((nz + 2, ny + 2, nx + 2)) for _ in range(3)))]
    out = {}
    for layout in (LAYOUT_LIST, LAYOUT_DENSE):
        p = copy.copy(case["params"])
        p.layout = layout
        with Solver(p) as sim:
            sim.set_geometry(case["walls"], w_in=case["w_in"])
            sim.init_equilibrium()
            s0 = sim.download_state()
            sim.init_velocity(u=fields[1], v=fields[2], w=fields[3], rho=fields[0])
            s1 = sim.download_state()
            sim.run(1, 4)
            s2 = sim.download_state()
        out[layout] = (s0, s1, s2)
    for a, b in zip(out[LAYOUT_LIST], out[LAYOUT_DENSE]):
        assert np.array_equal(a["f"][:, 1:-1, 1:-1, 1:-1][:, fl], b["f"][:, 1:-1, 1:-1, 1:-1][:, fl])
        assert np.array_equal(a["f_convec"], b["f_convec"])
