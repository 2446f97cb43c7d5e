"""The multiphase fluid-list layout (f and g over the fluid nodes, the boundary planes'
private slots and the bounce-back link slots; MFLBM_LAYOUT_LIST) against the dense planes
and the oracle.

The update is the dense layout's slot for slot, so in every storage form the fluid nodes'
populations, phi, the gradient fields and the convective-outlet memory are bit-identical to
the dense layout after 1, 2, 3 and 8 steps, for every boundary family of the dense tests
(periodic y and z, velocity and pressure inlets, convective and Zou-He outlets, porous
plates, MRT variants, a viscosity ratio); the strict build equals the oracle; the monitor
sums equal the dense layout's to rtol 1e-12, and change_inlet_fluid_phase and a checkpoint
round trip behave as on the dense layout.
"""
import copy

import numpy as np
import pytest

from cases import load_case, mp_case, periodic_ghosts
from mflbm import Solver
from mflbm._capi import LAYOUT_DENSE, LAYOUT_LIST
from pyoracle import Oracle
from test_gpu_multiphase import MP_CASES

pytestmark = pytest.mark.gpu


def _case(name, strict):
    """The dense step pulls from the ghost layers as uploaded and wraps after the collision;
    the list reads the periodic images directly, so the uploaded ghosts hold those images."""
    kw = MP_CASES[name]
    case = mp_case(strict=strict, **kw)
    per = kw.get("per", (0, 1, 1))
    for k in ("f", "g"):
        case[k] = periodic_ghosts(case[k], per)
    return case


def _fluid(case):
    return case["walls"][2:-2, 2:-2, 2:-2] == 0


def _run(case, layout, precision, steps, strict):
    p = copy.copy(case["params"])
    p.layout = layout
    p.precision = precision
    p.strict_fp = strict
    with Solver(p) as sim:
        load_case(sim, case)
        assert sim.layout == layout
        for n in range(1, steps + 1):
            sim.step(n)
        st = sim.download_state()
        gr = sim.get_gradient()
        mon = sim.monitor() if steps % 2 == 0 else None
    return st, gr, mon


def _compare(a, b, fl, case):
    for k in ("f", "g"):
        x, y = a[0][k][:, 1:-1, 1:-1, 1:-1][:, fl], b[0][k][:, 1:-1, 1:-1, 1:-1][:, fl]
        assert np.array_equal(x, y), (k, np.abs(x - y).max())
    for k in ("phi", "f_convec", "g_convec", "phi_convec"):
        if k in a[0]:
            assert np.array_equal(a[0][k], b[0][k]), (k, np.abs(a[0][k] - b[0][k]).max())
    for k in a[1]:
        assert np.array_equal(a[1][k], b[1][k]), k
    if a[2] is not None:
        np.testing.assert_allclose(a[2][0], b[2][0], rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(a[2][1], b[2][1], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("precision", [0, 1, 3, 4])
@pytest.mark.parametrize("name", list(MP_CASES))
@pytest.mark.parametrize("steps", [1, 2, 3, 8])
def test_list_equals_dense(name, steps, precision):
    case = _case(name, 0)
    fl = _fluid(case)
    a = _run(case, LAYOUT_LIST, precision, steps, 0)
    b = _run(case, LAYOUT_DENSE, precision, steps, 0)
    _compare(a, b, fl, case)


@pytest.mark.parametrize("name", ["walled_velocity_inlet_convective", "walled_pressure_bcs", "periodic_yz",
                                  "porous_plate_blocks_fluid1", "periodic_y_velocity_inlet_convective"])
def test_strict_list_equals_oracle(name):
    case = _case(name, 1)
    fl = _fluid(case)
    a = _run(case, LAYOUT_LIST, 0, 6, 1)
    orc = Oracle(case["params"])
    load_case(orc, case)
    orc.run(1, 6)
    b = orc.download_state()
    for k in ("f", "g"):
        assert np.array_equal(a[0][k][:, 1:-1, 1:-1, 1:-1][:, fl], b[k][:, 1:-1, 1:-1, 1:-1][:, fl]), k
    for k in ("phi", "f_convec", "g_convec", "phi_convec"):
        assert np.array_equal(a[0][k], b[k]), k
    orc.close()


def test_change_inlet_and_checkpoint_round_trip():
    case = _case("walled_velocity_inlet_convective", 0)
    fl = _fluid(case)
    out = []
    for layout in (LAYOUT_LIST, LAYOUT_DENSE):
        p = copy.copy(case["params"])
        p.layout = layout
        with Solver(p) as sim:
            load_case(sim, case)
            sim.run(1, 4)
            sim.change_inlet_fluid_phase(2, 5.5)
            sim.color_gradient()
            sim.run(5, 4)
            st = sim.download_state()
            sim.upload_state(st["f"], st["g"], st["phi"], st["f_convec"], st["g_convec"], st["phi_convec"])
            sim.color_gradient()
            sim.run(9, 4)
            out.append(sim.download_state())
    for k in ("f", "g"):
        assert np.array_equal(out[0][k][:, 1:-1, 1:-1, 1:-1][:, fl], out[1][k][:, 1:-1, 1:-1, 1:-1][:, fl]), k
    assert np.array_equal(out[0]["phi"], out[1]["phi"])


def test_plate_on_the_first_plane_with_periodic_y_falls_back_to_dense():
    """The porous plate's lower plane would be the z = 0 ghost plane, whose periodic-y ghosts
    the list cannot give private slots: AUTO takes the dense planes, an explicit list request
    is refused when the geometry is set."""
    from mflbm import MflbmError
    from mflbm._capi import LAYOUT_AUTO
    case = mp_case(strict=0, per=(0, 1, 0), inlet=1, outlet=1, plate=1, zplate=1, layout=LAYOUT_AUTO)
    with Solver(case["params"]) as sim:
        load_case(sim, case)
        assert sim.layout == LAYOUT_DENSE
    p = copy.copy(case["params"])
    p.layout = LAYOUT_LIST
    with Solver(p) as sim:
        with pytest.raises(MflbmError):
            sim.set_geometry(case["walls"], case["solid"], case["fluid"], case["w_in"])


def test_auto_takes_the_list():
    from mflbm._capi import LAYOUT_AUTO
    for name in ("periodic_yz", "porous_plate_blocks_fluid1", "walled_pressure_bcs"):
        case = mp_case(strict=0, layout=LAYOUT_AUTO, **MP_CASES[name])
        with Solver(case["params"]) as sim:
            load_case(sim, case)
            assert sim.layout == LAYOUT_LIST, name
