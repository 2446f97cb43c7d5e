"""GPU parity of the singlephase path against the CPU oracle, through the C ABI.

strict_fp=1 builds compile without FMA contraction and must be bit-identical to the
oracle on every slot of the halo'd state.  The default build (FMA) is held to a stated
FP64 tolerance.  FP32 / FP16-deviation storage are held to the precision of their
storage format against the FP64 oracle.
"""
import numpy as np
import pytest

from cases import load_case
from cases import sp_case as _sp_case


def sp_case(**kw):
    """The cases of this module exercise the dense layout (the reference's array layout,
    including ghost and solid slots); the fluid-list layout has its own tests."""
    return _sp_case(layout=1, **kw)
from mflbm import MFLBM_FP16, MFLBM_FP32, Solver
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

# max |delta f| allowed for the FMA build after the steps below (f ~ 0.05)
FMA_ATOL = 1e-14

SP_CASES = {
    "periodic_xyz": dict(per=(1, 1, 1), force=1e-5),
    "periodic_yz_xwalls": dict(per=(0, 1, 1), force=1e-5),
    "periodic_z_duct": dict(per=(0, 0, 1), force=1e-5, mrt=1),
    "srt_preset": dict(per=(0, 1, 1), force=1e-5, mrt=0),
    "velocity_inlet_convective_outlet": dict(per=(0, 0, 0), inlet=1, outlet=1, force=0.0),
    "velocity_inlet_periodic_y": dict(per=(0, 1, 0), inlet=1, outlet=1, force=0.0),
    "pressure_inlet_pressure_outlet": dict(per=(0, 0, 0), inlet=2, outlet=2, force=0.0),
    "velocity_inlet_pressure_outlet": dict(per=(0, 1, 0), inlet=1, outlet=2, force=0.0),
    "ragged_odd_sizes": dict(nx=7, ny=5, nz=9, per=(0, 1, 1), force=2e-5, spheres=1),
    "wide_rows": dict(nx=150, ny=6, nz=5, per=(1, 1, 1), force=1e-5, spheres=4),
}


def _pair(kw, strict=1, precision=0):
    case = sp_case(strict=strict, precision=precision, **kw)
    gpu = Solver(case["params"])
    orc = Oracle(case["params"])
    load_case(gpu, case)
    load_case(orc, case)
    return case, gpu, orc


@pytest.mark.parametrize("name", list(SP_CASES))
@pytest.mark.parametrize("steps", [1, 2, 3, 8])
def test_strict_bit_identical(name, steps):
    case, gpu, orc = _pair(SP_CASES[name], strict=1)
    for n in range(1, steps + 1):
        gpu.step(n)
        orc.step(n)
    a, b = gpu.download_state(), orc.download_state()
    assert np.array_equal(a["f"], b["f"]), np.abs(a["f"] - b["f"]).max()
    assert np.array_equal(a["f_convec"], b["f_convec"])


@pytest.mark.parametrize("name", list(SP_CASES))
def test_fma_build_within_tolerance(name):
    case, gpu, orc = _pair(SP_CASES[name], strict=0)
    gpu.run(1, 20)
    orc.run(1, 20)
    a, b = gpu.download_state(), orc.download_state()
    assert np.abs(a["f"] - b["f"]).max() <= FMA_ATOL


def test_graph_run_equals_single_steps():
    kw = SP_CASES["velocity_inlet_convective_outlet"]
    case, g1, _ = _pair(kw, strict=1)
    _, g2, _ = _pair(kw, strict=1)
    for n in range(3, 3 + 37):
        g1.step(n)
    g2.run(3, 37)         # odd start, 8-pair graph blocks, pair graphs, tail step
    a, b = g1.download_state(), g2.download_state()
    assert np.array_equal(a["f"], b["f"])


def test_monitor_and_macro_against_oracle():
    kw = dict(per=(0, 1, 1), force=1e-4, spheres=3)
    case, gpu, orc = _pair(kw, strict=1)
    gpu.run(1, 30)
    orc.run(1, 30)
    pa, sa, st_a = gpu.monitor()
    pb, sb, st_b = orc.monitor()
    assert st_a == st_b == 0
    np.testing.assert_allclose(pa, pb, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(sa, sb, rtol=1e-12, atol=0)
    ma, mb = gpu.macro(), orc.macro()
    for k in ("u", "v", "w", "rho"):
        assert np.array_equal(ma[k][1:-1, 1:-1, 1:-1], mb[k][1:-1, 1:-1, 1:-1]), k


def test_init_equilibrium_matches_oracle():
    case = sp_case(per=(0, 0, 0), inlet=1, outlet=1, force=0.0)
    gpu, orc = Solver(case["params"]), Oracle(case["params"])
    for s in (gpu, orc):
        s.set_geometry(case["walls"], None, None, case["w_in"])
        s.init_equilibrium()
    a, b = gpu.download_state(), orc.download_state()
    assert np.array_equal(a["f"], b["f"]) and np.array_equal(a["f_convec"], b["f_convec"])


def test_nan_reported_as_failed_status():
    case = sp_case(per=(1, 1, 1), force=1e-5)
    case["f"][3, 5, 5, 5] = np.nan
    gpu = Solver(case["params"])
    load_case(gpu, case)
    gpu.run(1, 4)
    _, _, status = gpu.monitor()
    assert status == 3


@pytest.mark.parametrize("precision,atol", [(MFLBM_FP32, 1e-6), (MFLBM_FP16, 1e-5)])
def test_reduced_precision_storage_tracks_fp64(precision, atol):
    # start near the MRT rest state, the regime a body-force run lives in
    kw = dict(per=(0, 1, 1), force=1e-5, spheres=3, rest="mrt")
    case = sp_case(precision=precision, strict=0, **kw)
    gpu = Solver(case["params"])
    load_case(gpu, case)
    ref = Oracle(case["params"])
    load_case(ref, case)
    gpu.run(1, 40)
    ref.run(1, 40)
    ua, ub = gpu.macro(), ref.macro()
    for k in ("u", "v", "w"):
        assert np.abs(ua[k] - ub[k]).max() <= atol, k
    assert np.abs(ua["rho"] - ub["rho"]).max() <= 50 * atol


def test_errors_are_reported():
    case = sp_case(per=(1, 1, 1))
    gpu = Solver(case["params"])
    from mflbm import MflbmError
    with pytest.raises(MflbmError):
        gpu.step(1)            # before set_geometry: MFLBM_ESTATE
    bad = case["walls"][:-1]
    with pytest.raises(AssertionError):
        gpu.set_geometry(bad)
