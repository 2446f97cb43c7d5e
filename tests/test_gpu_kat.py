"""Known-answer physics of the colour-gradient model on the GPU (FP64 drop-in, default
build), at sizes the CPU oracle cannot afford: the Laplace law over three drop radii
and the static contact angle of an attached drop for three prescribed angles.

Laplace (option 5, 80^3 box, 3000 steps: the pressure waves of the initial sharp drop have
died out, the R = 18 drop still reads 4 % low after 1000 steps): dp R / (2 gamma) within 4 %
at R = 10, 2 % at R = 14 and R = 18 (the interface has a fixed width of a few nodes).
Contact angle (option 3, 32 x 64 x 64, R0 = 16, 16000 steps): the drop's angle is
180 - theta within 3 degrees at the plane of the wetting nodes (x = 2); the angles at the
bounce-back wall (x = 1.5) are printed beside them.  The GPU Laplace result also equals
the oracle's on the CPU test's case.
"""
import os

import numpy as np
import pytest

import kat
from mflbm import Solver
from pyoracle import Oracle

pytestmark = pytest.mark.gpu


def test_laplace_law_three_radii():
    ratios = []
    for R0 in (10.0, 14.0, 18.0):
        case = kat.drop_case(82, 80, 5, R0)
        with Solver(case["params"]) as sim:
            kat.start(sim, case)
            sim.run(1, 3000)
            dp, R, umax = kat.laplace(sim, case)
        ratio = dp * R / (2.0 * case["params"].gamma)
        print(f"GPU Laplace: R={R:.3f} dp={dp:.5e} 2g/R={2 * case['params'].gamma / R:.5e} ratio={ratio:.4f} "
              f"umax={umax:.2e}")
        ratios.append(ratio)
        assert umax < 1e-4
    assert abs(ratios[0] - 1.0) < 0.04
    assert abs(ratios[1] - 1.0) < 0.02
    assert abs(ratios[2] - 1.0) < 0.02


def test_laplace_drop_matches_oracle():
    case = kat.drop_case(42, 40, 5, 10.0)
    o = Oracle(case["params"], variant="fast", threads=min(16, os.cpu_count() or 1))
    kat.start(o, case)
    o.run(1, 600)
    ref = kat.laplace(o, case)
    o.close()
    with Solver(case["params"]) as sim:
        kat.start(sim, case)
        sim.run(1, 600)
        got = kat.laplace(sim, case)
    np.testing.assert_allclose(got[:2], ref[:2], rtol=1e-9)


@pytest.mark.parametrize("theta", [45.0, 90.0, 135.0])
def test_static_contact_angle(theta):
    case = kat.drop_case(32, 64, 3, 16.0, theta_deg=theta)
    with Solver(case["params"]) as sim:
        kat.start(sim, case)
        sim.run(1, 16000)
        a2, a15, umax = kat.drop_angle(sim)
    want = 180.0 - theta
    print(f"GPU contact angle: theta={theta} drop angle expected {want:.1f}: {a2:.2f} deg at x=2, "
          f"{a15:.2f} deg at x=1.5, umax={umax:.2e}")
    assert abs(a2 - want) < 3.0
