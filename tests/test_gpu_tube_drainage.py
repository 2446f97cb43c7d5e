"""The 64x64x160 tube-drainage case after 2000 steps: GPU against the oracle.

strict build: bit-identical phi, PDFs and convective memory at ntime = 2000 (even), in the
dense layout on every slot and in the fluid-list layout (the default) on every fluid node.
default (FMA) build: max|dphi| <= 1e-6, max|du| <= 1e-10, |dS|/S <= 1e-10 against the
oracle, velocities from compute_macro_vars (valid after even steps).
mixed form (FP32 storage and arithmetic, FP64 reductions): phi L1 error (mean |dphi| over
the interior fluid nodes) <= 1e-3, |dS|/S <= 1e-3, max|du| <= 2e-5 (u ~ 1e-4; the largest
deviations sit on the interface), mean|du| <= 5e-6.
"""
import copy

import numpy as np
import pytest

from mflbm import Solver
from mflbm._capi import LAYOUT_AUTO, LAYOUT_DENSE, LAYOUT_LIST
from mflbm.workloads import tube_drainage
from pyoracle import Oracle

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

STEPS = 2000


def _setup(sim, case):
    sim.set_geometry(case["walls"], case["solid"], case["fluid"], case["w_in"])
    sim.init_equilibrium(case["phi"])
    sim.color_gradient()


@pytest.fixture(scope="module")
def oracle_result():
    case = tube_drainage(strict_fp=1)
    orc = Oracle(case["params"])
    _setup(orc, case)
    orc.run(1, STEPS)
    st = orc.download_state()
    sat = orc.saturation()
    mac = orc.macro()
    orc.close()
    return case, st, sat, mac


@pytest.mark.parametrize("layout", [LAYOUT_DENSE, LAYOUT_AUTO])
def test_strict_bit_identical_after_2000_steps(oracle_result, layout):
    case, st, sat, _ = oracle_result
    p = copy.copy(case["params"])
    p.layout = layout
    gpu = Solver(p)
    _setup(gpu, case)
    assert gpu.layout == (LAYOUT_DENSE if layout == LAYOUT_DENSE else LAYOUT_LIST)
    gpu.run(1, STEPS)
    a = gpu.download_state()
    fluid = case["walls"][2:-2, 2:-2, 2:-2] == 0
    for k in ("phi", "f", "g", "f_convec", "g_convec", "phi_convec"):
        x, y = a[k], st[k]
        if k in ("f", "g") and layout != LAYOUT_DENSE:
            x, y = x[:, 1:-1, 1:-1, 1:-1][:, fluid], y[:, 1:-1, 1:-1, 1:-1][:, fluid]
        assert np.array_equal(x, y), (k, np.abs(x - y).max())
    # identical state; the FP64 sums over ~5e5 nodes differ only in summation order
    np.testing.assert_allclose(gpu.saturation(), sat, rtol=1e-11)
    gpu.close()


def test_fma_build_within_tolerance_after_2000_steps(oracle_result):
    case, st, sat, mac = oracle_result
    p = copy.copy(case["params"])
    p.strict_fp = 0
    gpu = Solver(p)
    _setup(gpu, case)
    gpu.run(1, STEPS)
    a = gpu.download_state()
    inner = (slice(4, -4),) * 3
    dphi = np.abs(a["phi"][inner] - st["phi"][inner]).max()
    m = gpu.macro()
    du = max(np.abs(m[k][1:-1, 1:-1, 1:-1] - mac[k][1:-1, 1:-1, 1:-1]).max() for k in ("u", "v", "w"))
    v1, v2 = gpu.saturation()
    s_gpu, s_orc = v1 / (v1 + v2), sat[0] / (sat[0] + sat[1])
    print(f"FMA build after {STEPS} steps: max|dphi|={dphi:.3e} max|du|={du:.3e} dS/S={abs(s_gpu - s_orc) / s_orc:.3e}")
    assert dphi <= 1e-6
    assert du <= 1e-10
    assert abs(s_gpu - s_orc) / s_orc <= 1e-10
    gpu.close()


def test_mixed_fp32_form_within_tolerance_after_2000_steps(oracle_result):
    case, st, sat, mac = oracle_result
    p = copy.copy(case["params"])
    p.strict_fp = 0
    p.precision = 1
    gpu = Solver(p)
    _setup(gpu, case)
    gpu.run(1, STEPS)
    a = gpu.download_state()
    walls = case["walls"][2:-2, 2:-2, 2:-2]          # interior (nz, ny, nx)
    fluid = walls == 0
    dphi = np.abs(a["phi"][4:-4, 4:-4, 4:-4] - st["phi"][4:-4, 4:-4, 4:-4])[fluid]
    m = gpu.macro()
    dus = [np.abs(m[k][1:-1, 1:-1, 1:-1] - mac[k][1:-1, 1:-1, 1:-1])[fluid] for k in ("u", "v", "w")]
    du = max(d.max() for d in dus)
    du_mean = max(d.mean() for d in dus)
    v1, v2 = gpu.saturation()
    s_gpu, s_orc = v1 / (v1 + v2), sat[0] / (sat[0] + sat[1])
    ds = abs(s_gpu - s_orc) / s_orc
    print(f"FP32 form after {STEPS} steps: phi L1={dphi.mean():.3e} max|dphi|={dphi.max():.3e} "
          f"max|du|={du:.3e} mean|du|={du_mean:.3e} dS/S={ds:.3e}")
    assert dphi.mean() <= 1e-3
    assert ds <= 1e-3
    assert du <= 2e-5
    assert du_mean <= 5e-6
    gpu.close()


def test_double_word_collision_after_2000_steps(oracle_result):
    """FP64 storage with the double-word collision (about 48-bit arithmetic) against the
    FP64 oracle: max|dphi| <= 1e-7, max|du| <= 1e-9, |dS|/S <= 1e-9."""
    case, st, sat, mac = oracle_result
    p = copy.copy(case["params"])
    p.strict_fp = 0
    p.precision = 3
    gpu = Solver(p)
    _setup(gpu, case)
    gpu.run(1, STEPS)
    a = gpu.download_state()
    inner = (slice(4, -4),) * 3
    dphi = np.abs(a["phi"][inner] - st["phi"][inner]).max()
    m = gpu.macro()
    du = max(np.abs(m[k][1:-1, 1:-1, 1:-1] - mac[k][1:-1, 1:-1, 1:-1]).max() for k in ("u", "v", "w"))
    v1, v2 = gpu.saturation()
    s_gpu, s_orc = v1 / (v1 + v2), sat[0] / (sat[0] + sat[1])
    print(f"double-word collision after {STEPS} steps: max|dphi|={dphi:.3e} max|du|={du:.3e} "
          f"dS/S={abs(s_gpu - s_orc) / s_orc:.3e}")
    assert dphi <= 1e-7
    assert du <= 1e-9
    assert abs(s_gpu - s_orc) / s_orc <= 1e-9
    gpu.close()


def test_double_word_storage_after_2000_steps(oracle_result):
    """Double-word storage of f and g (FP32 pairs, about 48 bits) with the double-word
    collision and stencils, against the FP64 oracle: the gates of the FP64-storage form."""
    case, st, sat, mac = oracle_result
    p = copy.copy(case["params"])
    p.strict_fp = 0
    p.precision = 4
    gpu = Solver(p)
    _setup(gpu, case)
    gpu.run(1, STEPS)
    a = gpu.download_state()
    inner = (slice(4, -4),) * 3
    dphi = np.abs(a["phi"][inner] - st["phi"][inner]).max()
    m = gpu.macro()
    du = max(np.abs(m[k][1:-1, 1:-1, 1:-1] - mac[k][1:-1, 1:-1, 1:-1]).max() for k in ("u", "v", "w"))
    v1, v2 = gpu.saturation()
    s_gpu, s_orc = v1 / (v1 + v2), sat[0] / (sat[0] + sat[1])
    print(f"double-word storage after {STEPS} steps: max|dphi|={dphi:.3e} max|du|={du:.3e} "
          f"dS/S={abs(s_gpu - s_orc) / s_orc:.3e}")
    assert dphi <= 1e-7
    assert du <= 1e-9
    assert abs(s_gpu - s_orc) / s_orc <= 1e-9
    gpu.close()
