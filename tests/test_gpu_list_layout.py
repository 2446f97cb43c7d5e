"""Fluid-list layout (singlephase, periodic or walled samples) against the oracle and the
dense layout.

strict build: fluid-node PDFs bit-identical to the oracle after 1, 2, 3, 8 steps.
default build, every precision: bit-identical to the dense layout (same arithmetic).
Monitor sums agree to rtol 1e-12 (summation order differs); macro fields bit-identical.
"""
import numpy as np
import pytest

from cases import load_case, periodic_ghosts, sp_case
from mflbm import Solver
from mflbm._capi import LAYOUT_DENSE, LAYOUT_LIST, MflbmError
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "periodic_xyz_spheres": dict(per=(1, 1, 1), spheres=4, force=1e-5),
    "walled_x_periodic_yz": dict(per=(0, 1, 1), spheres=3, force=1e-5),
    "walled_xy_periodic_z": dict(per=(0, 0, 1), spheres=2, force=1e-5),
    "periodic_xyz_mrt_srt": dict(per=(1, 1, 1), spheres=3, mrt=2, nu=0.05, force=2e-5),
    "thin_periodic_y": dict(per=(1, 1, 1), ny=3, spheres=1, force=1e-5),
}


def _case(kw, **extra):
    c = sp_case(rest="mrt", **kw, **extra)
    c["f"] = periodic_ghosts(c["f"], kw["per"])
    return c


def _fluid(case):
    return case["walls"][2:-2, 2:-2, 2:-2] == 0     # interior (nz, ny, nx)


def _inner(a):
    return a[:, 1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("steps", [1, 2, 3, 8])
def test_strict_list_bit_identical_to_oracle(name, steps):
    case = _case(CASES[name], strict=1)
    gpu = Solver(case["params"])
    load_case(gpu, case)
    assert gpu.layout == LAYOUT_LIST
    orc = Oracle(case["params"])
    load_case(orc, case)
    gpu.run(1, steps)
    orc.run(1, steps)
    fl = _fluid(case)
    a, b = _inner(gpu.download_state()["f"]), _inner(orc.download_state()["f"])
    assert np.array_equal(a[:, fl], b[:, fl]), np.abs(a[:, fl] - b[:, fl]).max()
    if steps % 2 == 0:
        ma, mb = gpu.macro(), orc.macro()
        for k in ("u", "v", "w", "rho"):
            assert np.array_equal(ma[k][1:-1, 1:-1, 1:-1], mb[k][1:-1, 1:-1, 1:-1]), k
        pa, sa, _ = gpu.monitor()
        pb, sb, _ = orc.monitor()
        np.testing.assert_allclose(pa, pb, rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(sa, sb, rtol=1e-12)
    gpu.close()
    orc.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_list_equals_dense_default_build(precision):
    kw = CASES["periodic_xyz_spheres"]
    out = []
    for layout in (LAYOUT_DENSE, LAYOUT_LIST):
        case = _case(kw, strict=0, precision=precision)
        case["params"].layout = layout
        with Solver(case["params"]) as gpu:
            load_case(gpu, case)
            assert gpu.layout == layout
            gpu.run(1, 20)
            out.append((_inner(gpu.download_state()["f"]), gpu.monitor()[0]))
    fl = _fluid(case)
    assert np.array_equal(out[0][0][:, fl], out[1][0][:, fl])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-300)


def test_graph_run_equals_steps_and_init():
    kw = CASES["walled_x_periodic_yz"]
    case = _case(kw, strict=0)
    a, b = Solver(case["params"]), Solver(case["params"])
    for s in (a, b):
        s.set_geometry(case["walls"])
        s.init_equilibrium()
    for n in range(1, 38):
        a.step(n)
    b.run(1, 37)
    assert np.array_equal(a.download_state()["f"], b.download_state()["f"])
    # the rest state after init_equilibrium downloads as the BGK weights everywhere
    c = Solver(case["params"])
    c.set_geometry(case["walls"])
    c.init_equilibrium()
    f = c.download_state()["f"]
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    assert np.array_equal(f, np.broadcast_to(w[:, None, None, None], f.shape))
    for s in (a, b, c):
        s.close()


def test_layout_choice_with_open_z():
    """An open z direction (inlet / outlet conditions, or neither) takes the fluid list with
    boundary-plane slots when x is walled; with x periodic it falls back to the dense planes
    under AUTO, and an explicit list request is refused when the context is created."""
    case = sp_case(nx=10, ny=8, nz=12, per=(0, 0, 0), inlet=1, outlet=1, force=0.0, spheres=1)
    with Solver(case["params"]) as s:
        s.set_geometry(case["walls"], w_in=case["w_in"])
        assert s.layout == LAYOUT_LIST
    case = sp_case(nx=10, ny=8, nz=12, per=(0, 1, 0), spheres=1)
    with Solver(case["params"]) as s:
        s.set_geometry(case["walls"])
        assert s.layout == LAYOUT_LIST
    case = sp_case(nx=10, ny=8, nz=12, per=(1, 1, 0), inlet=1, outlet=1, force=0.0, spheres=1)
    with Solver(case["params"]) as s:
        s.set_geometry(case["walls"], w_in=case["w_in"])
        assert s.layout == LAYOUT_DENSE
    case["params"].layout = LAYOUT_LIST
    with pytest.raises(MflbmError):
        Solver(case["params"])


def test_unit_rate_collision_matches_oracle():
    # tau = 1 with MRT preset 1 takes the unit-rate collision (zero-coefficient moments skipped)
    kw = dict(per=(1, 1, 1), spheres=3, force=1e-5, nu=1.0 / 6.0)
    case = _case(kw, strict=0)
    gpu = Solver(case["params"])
    load_case(gpu, case)
    orc = Oracle(case["params"], variant="fast")
    load_case(orc, case)
    gpu.run(1, 20)
    orc.run(1, 20)
    fl = _fluid(case)
    a, b = _inner(gpu.download_state()["f"]), _inner(orc.download_state()["f"])
    assert np.abs(a[:, fl] - b[:, fl]).max() <= 1e-14
    gpu.close()
    orc.close()
