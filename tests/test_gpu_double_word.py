"""The double-word forms against the FP64 oracle: FP64 storage with the double-word
collision (MFLBM_FP64FF) and double-word storage with it (MFLBM_FF, a hi + lo FP32 pair
per population; the upload splits the FP64 state, the download joins it).

The sweep computes in two-FP32 arithmetic (about 48 significant bits; a split keeps 47
bits of an FP64 value), so after n steps the PDFs differ from the oracle's FP64 ones by
rounding noise only: |df| <= 2e-14 (n + 1) on every fluid node, for populations of
order 0.1 perturbed by 1e-3 and forces of 1e-5 (a wrong coefficient or sign shows up at
1e-8 or above).  Cases: fluid-list and dense layouts, unit rates (tau = 1, MRT preset 1)
and general rates, the SRT preset, walls, and open z with inlet/outlet conditions.
The strict (--fmad=false) and default builds are bit-identical in this form (every
operation of the sweep is an explicit rounding intrinsic).
"""
import numpy as np
import pytest

from cases import load_case, periodic_ghosts, sp_case
from mflbm import MFLBM_FF, MFLBM_FP64FF, Solver
from mflbm._capi import LAYOUT_DENSE, LAYOUT_LIST
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "list_unit_rates": dict(per=(1, 1, 1), spheres=4, nu=1.0 / 6.0, force=1e-5, layout=LAYOUT_LIST),
    "list_general_rates": dict(per=(1, 1, 1), spheres=3, nu=0.1, force=2e-5, layout=LAYOUT_LIST),
    "list_walled_x": dict(per=(0, 1, 1), spheres=3, nu=0.1, force=1e-5, layout=LAYOUT_LIST),
    "dense_unit_rates": dict(per=(0, 1, 1), spheres=3, nu=1.0 / 6.0, force=1e-5, layout=LAYOUT_DENSE),
    "dense_srt": dict(per=(0, 1, 1), spheres=2, mrt=2, nu=0.05, force=1e-5, layout=LAYOUT_DENSE),
    "velocity_inlet_convective_outlet": dict(per=(0, 1, 0), inlet=1, outlet=1, force=0.0, layout=LAYOUT_DENSE),
    "pressure_inlet_pressure_outlet": dict(per=(0, 0, 0), inlet=2, outlet=2, force=0.0, layout=LAYOUT_DENSE),
}


def _case(kw, strict=0, precision=MFLBM_FP64FF):
    kw = dict(kw)
    layout = kw.pop("layout")
    c = sp_case(rest="mrt", precision=precision, strict=strict, layout=layout, **kw)
    c["f"] = periodic_ghosts(c["f"], kw["per"])
    return c


def _fluid(case):
    return case["walls"][2:-2, 2:-2, 2:-2] == 0


def _inner(a):
    return a[:, 1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("precision", [MFLBM_FP64FF, MFLBM_FF])
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("steps", [1, 2, 9, 40])
def test_double_word_collision_tracks_fp64_oracle(name, steps, precision):
    case = _case(CASES[name], precision=precision)
    with Solver(case["params"]) as gpu:
        load_case(gpu, case)
        assert gpu.layout == CASES[name]["layout"]
        gpu.run(1, steps)
        a = _inner(gpu.download_state()["f"])
        pa, _, _ = gpu.monitor()
    orc = Oracle(case["params"])
    load_case(orc, case)
    orc.run(1, steps)
    b = _inner(orc.download_state()["f"])
    pb, _, _ = orc.monitor()
    orc.close()
    fl = _fluid(case)
    err = np.abs(a[:, fl] - b[:, fl]).max()
    print(f"precision {precision} {name} steps {steps}: max |df| {err:.3e}")
    assert err <= 2e-14 * (steps + 1)
    # per-slice flow rates (sums over ~100 nodes of the momentum, values ~1e-5): the
    # rounding noise of the populations summed, far below a coefficient error (>= 1e-8)
    np.testing.assert_allclose(pa, pb, rtol=0, atol=1e-11)


@pytest.mark.parametrize("precision", [MFLBM_FP64FF, MFLBM_FF])
@pytest.mark.parametrize("name", ["list_unit_rates", "dense_srt"])
def test_strict_and_default_builds_identical(name, precision):
    out = []
    for strict in (0, 1):
        case = _case(CASES[name], strict=strict, precision=precision)
        with Solver(case["params"]) as gpu:
            load_case(gpu, case)
            gpu.run(1, 12)
            out.append(_inner(gpu.download_state()["f"]))
    fl = _fluid(case)
    assert np.array_equal(out[0][:, fl], out[1][:, fl])


@pytest.mark.parametrize("name", ["list_unit_rates", "dense_unit_rates"])
def test_fp64_storage_split_of_zero_and_tiny_populations(name):
    """FP64 storage with the double-word collision splits a node's 19 loads with the
    select-free split of the range [2^-103, 2^128) and reads them again through the general
    split when one lies outside it.  Nodes holding an exact zero, a value below 2^-103 and
    one below the FP32 range take that second path; every node must still track the FP64
    oracle to rounding noise after one and two steps."""
    kw = dict(CASES[name])
    layout = kw.pop("layout")
    case = sp_case(rest="mrt", precision=MFLBM_FP64FF, strict=0, layout=layout, **kw)
    fl = _fluid(case)
    k, j, i = np.nonzero(fl)
    f = case["f"].copy()
    for n, (q, v) in enumerate([(3, 0.0), (7, 1e-35), (12, -1e-40), (0, 0.0), (18, 3e-33), (5, -0.0)]):
        f[q, k[5 * n] + 1, j[5 * n] + 1, i[5 * n] + 1] = v
    case["f"] = periodic_ghosts(f, kw["per"])
    for steps in (1, 2):
        with Solver(case["params"]) as gpu:
            load_case(gpu, case)
            gpu.run(1, steps)
            a = _inner(gpu.download_state()["f"])
        orc = Oracle(case["params"])
        load_case(orc, case)
        orc.run(1, steps)
        b = _inner(orc.download_state()["f"])
        orc.close()
        err = np.abs(a[:, fl] - b[:, fl]).max()
        print(f"{name} steps {steps}: max |df| {err:.3e}")
        assert np.isfinite(a[:, fl]).all()
        assert err <= 2e-14 * (steps + 1)


def test_double_word_storage_round_trip():
    """Upload then download without a step: every population back within 2^-46 relative
    (split to 47 bits, joined by one FP64 add)."""
    case = _case(CASES["list_walled_x"], precision=MFLBM_FF)
    with Solver(case["params"]) as gpu:
        load_case(gpu, case)
        a = _inner(gpu.download_state()["f"])
    b = _inner(case["f"])
    fl = _fluid(case)
    assert np.all(np.abs(a[:, fl] - b[:, fl]) <= 2.0 ** -46 * np.abs(b[:, fl]))


MP_CASES = {
    "mp_periodic_yz": dict(per=(0, 1, 1)),
    "mp_velocity_inlet_convective": dict(per=(0, 0, 0), inlet=1, outlet=1, theta_deg=30.0),
    "mp_pressure_bcs": dict(per=(0, 0, 0), inlet=2, outlet=2, sa_inject=0.0),
    "mp_viscosity_ratio_mrt1": dict(per=(0, 1, 1), nu1=0.02, nu2=0.2, mrt=1),
    "mp_mrt2_fixed_rates": dict(per=(0, 1, 1), mrt=2),
    "mp_mrt3": dict(per=(0, 1, 1), mrt=3, theta_deg=120.0),
    "mp_mrt4": dict(per=(0, 1, 1), mrt=4, beta=0.7),
    "mp_body_force": dict(per=(0, 0, 1), force=1e-5),
}


@pytest.mark.parametrize("precision", [MFLBM_FP64FF, MFLBM_FF])
@pytest.mark.parametrize("name", list(MP_CASES))
@pytest.mark.parametrize("steps", [1, 9, 40])
def test_multiphase_double_word_collision_tracks_fp64_oracle(name, steps, precision):
    """Multiphase, the double-word collision and colour-gradient stencils on FP64 storage
    (MFLBM_FP64FF) or on double-word storage (MFLBM_FF, f and g kept as FP32 pairs), against
    the FP64 oracle after n = 1, 9, 40 steps (populations of order 0.1; a wrong term shows
    at 1e-6 and above): f, g, phi and |grad phi| within 1e-10, the gradient n |grad phi|
    within 1e-10 away from the wetting nodes and 1e-8 at them, kappa |grad phi| at fluid
    nodes within 1e-8.  Measured (FP64 storage): f within 3e-11, phi within 2e-12."""
    from cases import mp_case
    case = mp_case(strict=0, precision=precision, **MP_CASES[name])
    with Solver(case["params"]) as gpu:
        load_case(gpu, case)
        for n in range(1, steps + 1):
            gpu.step(n)
        a = gpu.download_state()
        ga = gpu.get_gradient()
    orc = Oracle(case["params"])
    load_case(orc, case)
    for n in range(1, steps + 1):
        orc.step(n)
    b = orc.download_state()
    gb = orc.get_gradient()
    orc.close()
    df = max(np.abs(a[k] - b[k]).max() for k in ("f", "g"))
    dphi = np.abs(a["phi"] - b["phi"]).max()
    # The gradient enters the collision as n |grad phi| and kappa |grad phi| (CSF force,
    # recolouring), so those products are compared, not the unit normal (which amplifies the
    # ~1e-14 gradient error by 1/|grad phi| where the gradient is just above the 1e-6 cut-off).
    # At the fluid-boundary nodes the reference's wetting step replaces the normal through
    # 1/sqrt(1 - (n_w . n)^2), which amplifies the incoming error by up to ~1e4 where the phase
    # normal is nearly parallel to the wall normal (the FP64 build sees the same factor on a
    # 2^-53 base): those nodes get their own, looser gate.
    wet = np.zeros(case["walls"].shape, dtype=bool)
    fb = case["fluid"]
    wet[fb["iz"] + 1, fb["iy"] + 1, fb["ix"] + 1] = True
    # cells within rounding of the reference's |grad phi| < 1e-6 cut-off may fall on either
    # side in the two forms (the product n |grad phi| then jumps by ~1e-6): left out, with
    # the curvature stencil's neighbours
    band = ((ga["c_norm"] > 5e-7) & (ga["c_norm"] < 2e-6)) | ((gb["c_norm"] > 5e-7) & (gb["c_norm"] < 2e-6))
    near = np.zeros_like(band)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                near |= np.roll(band, (dz, dy, dx), axis=(0, 1, 2))
    dg = np.max([np.abs(ga[k] * ga["c_norm"] - gb[k] * gb["c_norm"]) for k in ("cn_x", "cn_y", "cn_z")], axis=0)
    dgrad, dgrad_wet = dg[~wet & ~band].max(), dg[wet & ~band].max()
    dnorm = np.abs(ga["c_norm"] - gb["c_norm"]).max()
    fl = (case["walls"][2:-2, 2:-2, 2:-2] == 0) & ~near[2:-2, 2:-2, 2:-2]
    ka = (ga["curv"] * ga["c_norm"][1:-1, 1:-1, 1:-1])[1:-1, 1:-1, 1:-1][fl]
    kb = (gb["curv"] * gb["c_norm"][1:-1, 1:-1, 1:-1])[1:-1, 1:-1, 1:-1][fl]
    dforce = np.abs(ka - kb).max()
    print(f"precision {precision} {name} steps {steps}: max |df| {df:.3e} |dphi| {dphi:.3e} |d(n|g|)| {dgrad:.3e} (wetting nodes "
          f"{dgrad_wet:.3e}) |d|g|| {dnorm:.3e} |d(kappa|g|)| {dforce:.3e}")
    assert df <= 1e-10
    assert dphi <= 1e-10
    assert dnorm <= 1e-10
    assert dgrad <= 1e-10
    assert dgrad_wet <= 1e-8
    assert dforce <= 1e-8


@pytest.mark.parametrize("precision", [1, MFLBM_FP64FF, MFLBM_FF])
def test_wetting_with_wall_parallel_phase_normals_stays_finite(precision):
    """A flat phase slab across a channel walled in x (uniform in y and z, exact rest states):
    every phase normal is parallel to the wall normal, where the reference's wetting factor
    1/sqrt(1 - (nw.n)^2) has no value once rounding puts |nw.n| at or above 1.  The FP32 and
    double-word forms bound 1 - (nw.n)^2 below (1e-6, 1e-12) and stay finite over 200 steps;
    the FP64 drop-in keeps the reference's formula."""
    from cases import W, mp_case
    case = mp_case(nx=12, ny=6, nz=8, per=(0, 1, 1), spheres=0, strict=0, precision=precision, theta_deg=30.0)
    p = case["params"]
    nx, ny, nz = p.nx, p.ny, p.nz
    x = np.arange(-3, nx + 5, dtype=np.float64)
    phi = np.broadcast_to(np.tanh((x - 0.5 * nx) / 1.5), (nz + 8, ny + 8, nx + 8)).copy()
    ph1 = phi[3:nz + 5, 3:ny + 5, 3:nx + 5]
    case["phi"] = phi
    case["f"] = W[:, None, None, None] * (0.5 * (1.0 + ph1))[None]
    case["g"] = W[:, None, None, None] * (0.5 * (1.0 - ph1))[None]
    with Solver(p) as gpu:
        load_case(gpu, case)
        gpu.run(1, 200)
        st = gpu.download_state()
        grad = gpu.get_gradient()
        v1, v2 = gpu.saturation()
    assert np.isfinite(st["f"]).all() and np.isfinite(st["g"]).all() and np.isfinite(st["phi"]).all()
    assert np.isfinite(grad["cn_x"]).all() and np.isfinite(v1) and np.isfinite(v2)
