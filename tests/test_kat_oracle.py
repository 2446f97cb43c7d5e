"""Known-answer physics of the colour-gradient model on the oracle (CPU).

These pin the multiphase restatement itself, independently of its agreement with the
GPU kernels: the Laplace law of a free drop (the reference's option-5 surface-tension
set-up) and the contact angle of an attached drop (option 3).  Small lattices, so the
CPU suite stays short; the GPU tests run larger drops to tighter gates.
"""
import os

import pytest

import kat
from pyoracle import Oracle

THREADS = min(16, os.cpu_count() or 1)


def test_laplace_law_free_drop():
    """R = 10 in a 40^3 box after 600 steps: dp = 2 gamma / R within 5 % (measured 2.7 %),
    spurious currents below 1e-4."""
    case = kat.drop_case(42, 40, 5, 10.0)
    o = Oracle(case["params"], variant="fast", threads=THREADS)
    kat.start(o, case)
    o.run(1, 600)
    dp, R, umax = kat.laplace(o, case)
    o.close()
    ratio = dp * R / (2.0 * case["params"].gamma)
    print(f"oracle Laplace: R={R:.3f} dp={dp:.4e} 2g/R={2 * case['params'].gamma / R:.4e} ratio={ratio:.4f} "
          f"umax={umax:.2e}")
    assert abs(ratio - 1.0) < 0.05
    assert umax < 1e-4


def test_neutral_contact_angle_attached_drop():
    """theta = 90: the attached drop settles to a hemisphere, 90 +- 2 degrees."""
    case = kat.drop_case(24, 40, 3, 10.0, theta_deg=90.0)
    o = Oracle(case["params"], variant="fast", threads=THREADS)
    kat.start(o, case)
    o.run(1, 3000)
    a2, a15, umax = kat.drop_angle(o)
    o.close()
    print(f"oracle contact angle (theta=90): {a2:.2f} deg at x=2, {a15:.2f} deg at x=1.5, umax={umax:.2e}")
    assert abs(a2 - 90.0) < 2.0
