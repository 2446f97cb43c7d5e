"""GPU parity of the multiphase colour-gradient path against the CPU oracle (C ABI).

strict_fp=1: bit-identical PDFs, phi, normals, curvature on every slot after 1-3 and
several steps (both AA parities, all boundary families).  Default (FMA) build: stated
FP64 tolerances.  Monitor reductions: FP64 sums in a different order, rtol 1e-12.
"""
import numpy as np
import pytest

from cases import load_case, mp_case
from mflbm import Solver
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

MP_CASES = {
    "periodic_yz": dict(per=(0, 1, 1)),
    "periodic_y_velocity_inlet_convective": dict(per=(0, 1, 0), inlet=1, outlet=1),
    "walled_velocity_inlet_convective": dict(per=(0, 0, 0), inlet=1, outlet=1, theta_deg=30.0),
    "walled_pressure_bcs": dict(per=(0, 0, 0), inlet=2, outlet=2, sa_inject=0.0),
    "velocity_inlet_pressure_outlet": dict(per=(0, 0, 0), inlet=1, outlet=2),
    "periodic_z_only": dict(per=(0, 0, 1), force=1e-5),
    "viscosity_ratio_mrt1": dict(per=(0, 1, 1), nu1=0.02, nu2=0.2, mrt=1),
    "mrt3": dict(per=(0, 1, 1), mrt=3, theta_deg=120.0),
    "mrt4": dict(per=(0, 1, 1), mrt=4, beta=0.7),
    "porous_plate_blocks_fluid1": dict(per=(0, 1, 0), inlet=1, outlet=1, plate=1, zplate=8),
    "porous_plate_blocks_fluid2": dict(per=(0, 1, 0), inlet=1, outlet=1, plate=2, zplate=6),
    "ragged_sizes": dict(nx=9, ny=7, nz=11, per=(0, 1, 1), spheres=1),
}

FIELDS = ("f", "g", "phi", "f_convec", "g_convec", "phi_convec")


def _pair(kw, strict=1):
    case = mp_case(strict=strict, **kw)
    gpu = Solver(case["params"])
    orc = Oracle(case["params"])
    load_case(gpu, case)
    load_case(orc, case)
    return case, gpu, orc


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_initial_color_gradient_bit_identical():
    case, gpu, orc = _pair(MP_CASES["walled_velocity_inlet_convective"])
    ga, gb = gpu.get_gradient(), orc.get_gradient()
    for k in ga:
        assert _same(ga[k], gb[k]), k


@pytest.mark.parametrize("name", list(MP_CASES))
@pytest.mark.parametrize("steps", [1, 2, 3, 6])
def test_strict_bit_identical(name, steps):
    case, gpu, orc = _pair(MP_CASES[name])
    for n in range(1, steps + 1):
        gpu.step(n)
        orc.step(n)
    a, b = gpu.download_state(), orc.download_state()
    for k in FIELDS:
        if k in a:
            assert _same(a[k], b[k]), (k, np.nanmax(np.abs(a[k] - b[k])))
    ga, gb = gpu.get_gradient(), orc.get_gradient()
    for k in ga:
        assert _same(ga[k], gb[k]), k


@pytest.mark.parametrize("name", ["periodic_yz", "walled_velocity_inlet_convective", "viscosity_ratio_mrt1"])
def test_fma_build_within_tolerance(name):
    case, gpu, orc = _pair(MP_CASES[name], strict=0)
    gpu.run(1, 40)
    orc.run(1, 40)
    a, b = gpu.download_state(), orc.download_state()
    assert np.abs(a["f"] - b["f"]).max() <= 1e-12
    assert np.abs(a["g"] - b["g"]).max() <= 1e-12
    assert np.abs(a["phi"] - b["phi"]).max() <= 1e-10


def test_graph_run_equals_steps():
    kw = MP_CASES["periodic_y_velocity_inlet_convective"]
    _, g1, _ = _pair(kw)
    _, g2, _ = _pair(kw)
    for n in range(1, 1 + 21):
        g1.step(n)
    g2.run(1, 21)
    a, b = g1.download_state(), g2.download_state()
    for k in FIELDS:
        assert _same(a[k], b[k]), k


def test_monitor_saturation_macro():
    case, gpu, orc = _pair(MP_CASES["walled_velocity_inlet_convective"])
    gpu.run(1, 24)
    orc.run(1, 24)
    va, vb = gpu.saturation(), orc.saturation()
    np.testing.assert_allclose(va, vb, rtol=1e-13)
    pa, sa, st_a = gpu.monitor()
    pb, sb, st_b = orc.monitor()
    assert st_a == st_b == 0
    np.testing.assert_allclose(pa, pb, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(sa, sb, rtol=1e-12, atol=1e-30)
    ma, mb = gpu.macro(), orc.macro()
    for k in ("u", "v", "w", "rho"):
        assert _same(ma[k][1:-1, 1:-1, 1:-1], mb[k][1:-1, 1:-1, 1:-1]), k
    assert _same(ma["phi"], mb["phi"])


def test_init_equilibrium_matches_oracle():
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1)
    gpu, orc = Solver(case["params"]), Oracle(case["params"])
    for s in (gpu, orc):
        s.set_geometry(case["walls"], case["solid"], case["fluid"], case["w_in"])
        s.init_equilibrium(case["phi"])
    a, b = gpu.download_state(), orc.download_state()
    for k in FIELDS:
        assert _same(a[k], b[k]), k


def test_list_outside_halo_rejected():
    case = mp_case()
    gpu = Solver(case["params"])
    bad = case["solid"].copy()
    bad["ix"][0] = case["params"].nx + 9
    from mflbm import MflbmError
    with pytest.raises(MflbmError):
        gpu.set_geometry(case["walls"], bad, case["fluid"])
    bad = case["solid"].copy()
    bad["neighbor_list"][0, 0] = 19
    bad["i_fluid_num"][0] = max(1, bad["i_fluid_num"][0])
    with pytest.raises(MflbmError):
        gpu.set_geometry(case["walls"], bad, case["fluid"])


@pytest.mark.parametrize("name", ["periodic_yz", "walled_velocity_inlet_convective", "ragged_sizes"])
def test_fma_build_gradient_fields(name):
    """Default build: the colour-gradient step runs over fluid-cell lists and compact
    solid-boundary records.  Normals on every cell of the halo-2 box (wall cells 0, solid
    boundary cells extrapolated) and curvature at every fluid node track the oracle after
    10 steps, away from cells whose |grad phi| lies near the reference's 1e-6 cut-off (and
    their stencil neighbours); curvature at wall nodes is 0 (never read)."""
    case, gpu, orc = _pair(MP_CASES[name], strict=0)
    gpu.run(1, 10)
    orc.run(1, 10)
    ga, gb = gpu.get_gradient(), orc.get_gradient()
    # the reference zeroes the normal where |grad phi| < 1e-6: a cell within rounding of that
    # cut-off may fall on different sides in two builds, so the band around it is left out
    band = ((ga["c_norm"] > 5e-7) & (ga["c_norm"] < 2e-6)) | ((gb["c_norm"] > 5e-7) & (gb["c_norm"] < 2e-6))
    print(f"{name}: {int(band.sum())} cells near the 1e-6 cut-off left out")
    for k in ("cn_x", "cn_y", "cn_z", "c_norm"):
        assert np.abs(ga[k] - gb[k])[~band].max() <= 1e-9, k
    fluid1 = case["walls"][1:-1, 1:-1, 1:-1] == 0         # halo-1 box
    inner = np.zeros_like(fluid1)
    inner[1:-1, 1:-1, 1:-1] = True
    fl = fluid1 & inner
    # curvature differences the cut-off band's normals feed (its stencil reaches one cell)
    near = np.zeros_like(band)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                near |= np.roll(band, (dz, dy, dx), axis=(0, 1, 2))
    fl = fl & ~near[1:-1, 1:-1, 1:-1]
    assert np.abs(ga["curv"][fl] - gb["curv"][fl]).max() <= 1e-7
    assert np.all(ga["curv"][inner & ~fluid1] == 0.0)


@pytest.mark.parametrize("strict", [1, 0])
def test_unordered_neighbour_lists_use_record_kernels(strict):
    """Solid-boundary records whose neighbour lists are not ascending keep the 96-byte
    record kernels, which sum in the list's order, as the oracle does: the strict build is
    bit-identical to the oracle after 3 steps, the default build within its tolerance."""
    case = mp_case(strict=strict, **MP_CASES["walled_velocity_inlet_convective"])
    solid = case["solid"].copy()
    for r in solid:
        n = int(r["i_fluid_num"])
        r["neighbor_list"][:n] = r["neighbor_list"][:n][::-1].copy()
    assert any(int(r["i_fluid_num"]) > 1 for r in solid)
    case["solid"] = solid
    gpu = Solver(case["params"])
    orc = Oracle(case["params"])
    load_case(gpu, case)
    load_case(orc, case)
    for n in range(1, 4):
        gpu.step(n)
        orc.step(n)
    a, b = gpu.download_state(), orc.download_state()
    for k in ("f", "g", "phi"):
        if strict:
            assert _same(a[k], b[k]), k
        else:
            assert np.abs(a[k] - b[k]).max() <= 1e-12, k
    gpu.close()
    orc.close()


def test_gradient_tables_ready_in_every_context():
    """Device tables filled right after allocation (the gradient cell lists, boundary
    records, fluid-list tables) hold their uploaded contents in every new context: a zero
    fill still queued on the context's stream once landed after the upload, emptied the
    normals list and sent its threads outside the box.  Sixteen contexts from the same
    deck give the same phase field and gradient fields, with the normals computed."""
    case = mp_case(strict=0, **MP_CASES["ragged_sizes"])
    ref = None
    for _ in range(16):
        with Solver(case["params"]) as gpu:
            load_case(gpu, case)
            phi = gpu.download_state()["phi"]
            gr = gpu.get_gradient()
        assert np.count_nonzero(gr["c_norm"]) > 100
        if ref is None:
            ref = (phi, gr)
            continue
        assert np.array_equal(phi, ref[0])
        for k in gr:
            assert np.array_equal(gr[k], ref[1][k]), k


@pytest.mark.parametrize("precision", [1, 0])
def test_fused_gradient_steps_equal_separate_kernels(monkeypatch, precision):
    """The default build applies the wetting inside the normals kernel and, in FP32, computes
    the collision's curvature from the normal records; MFLBM_SPLIT_GRADIENT=1 runs both in
    their own kernels.  FP64 (only the wetting fused): gradient fields after the load, state
    after 1-6 steps and monitor sums bit-identical.  FP32: the fused kernels are separately
    compiled, and the FMA build may contract their multiply-adds differently, so the results
    agree to FP32 rounding: normals after the load within 2e-6, f and g within 1e-6 and phi
    within 2e-6 after 6 steps (measured 2.4e-7, 4.5e-8, 2.4e-7)."""
    import copy
    kw = MP_CASES["walled_velocity_inlet_convective"]
    out = []
    for split in ("0", "1"):
        monkeypatch.setenv("MFLBM_SPLIT_GRADIENT", split)
        case = mp_case(strict=0, precision=precision, **kw)
        p = copy.copy(case["params"])
        with Solver(p) as gpu:
            load_case(gpu, case)
            g0 = gpu.get_gradient()
            states = []
            for n in range(1, 7):
                gpu.step(n)
                states.append(gpu.download_state())
            out.append((states, gpu.get_gradient(), gpu.monitor(), g0))
    if precision == 0:
        for k in out[0][3]:
            assert _same(out[0][3][k], out[1][3][k]), k
        for a, b in zip(out[0][0], out[1][0]):
            for k in FIELDS:
                assert _same(a[k], b[k]), k
        for k in out[0][1]:
            assert _same(out[0][1][k], out[1][1][k]), k
        assert np.array_equal(out[0][2][0], out[1][2][0]) and np.array_equal(out[0][2][1], out[1][2][1])
    else:
        dn = max(np.abs(out[0][3][k] - out[1][3][k]).max() for k in ("cn_x", "cn_y", "cn_z"))
        a, b = out[0][0][-1], out[1][0][-1]
        df = max(np.abs(a[k] - b[k]).max() for k in ("f", "g"))
        dphi = np.abs(a["phi"] - b["phi"]).max()
        print(f"FP32 fused vs separate: normals after the load max|dn|={dn:.2e}; after 6 steps "
              f"max|df|={df:.2e} max|dphi|={dphi:.2e}")
        assert dn <= 2e-6 and df <= 1e-6 and dphi <= 2e-6
