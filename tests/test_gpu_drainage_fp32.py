"""Multiphase mixed form on a sphere-packing drainage (the C3 set-up at 96^2 x 96 plus
8-layer buffers, contact angle 30 deg): stays finite and tracks the FP64 form (saturation
within 1e-3 relative, phi L1 within 1e-2) over 2000 steps."""
import copy

import numpy as np
import pytest

from mflbm import Solver, workloads

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_fp32_packing_drainage_tracks_fp64():
    case = workloads.packing_drainage(nxy=96, nzp=96, buffer=8, gpu_preprocess=True)
    res = {}
    for prec in (0, 1):
        p = copy.copy(case["params"])
        p.precision = prec
        with Solver(p) as sim:
            sim.set_geometry(case["walls"], case["solid"], case["fluid"], case["w_in"])
            sim.init_equilibrium(case["phi"])
            sim.color_gradient()
            sats = []
            for c in range(4):
                sim.run(1 + 500 * c, 500)
                v1, v2 = sim.saturation()
                sats.append(v1 / (v1 + v2))
            res[prec] = (np.array(sats), sim.macro()["phi"][4:-4, 4:-4, 4:-4].copy())
    s64, s32 = res[0][0], res[1][0]
    fl = case["walls"][2:-2, 2:-2, 2:-2] == 0
    l1 = np.abs(res[1][1] - res[0][1])[fl].mean()
    print("saturation fp64", s64, "fp32", s32, "phi L1", l1)
    assert np.isfinite(s32).all()
    assert np.abs(s32 - s64).max() <= 1e-3 * s64.max()
    assert l1 <= 1e-2
