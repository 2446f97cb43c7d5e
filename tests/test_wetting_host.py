"""The per-node wetting step (mf-lbm_gb300/csrc/wetting.cuh) built for the host.

The reference's expression, cos nw +- sin (n - t nw) / sqrt(1 - t^2) with t = nw.n, gives a
unit normal at the contact angle only for a unit n; near t = +-1 it divides the departure of
|n| from 1 by sqrt(1 - t^2) and has no value at |t| >= 1 (Phase_gradient.F90:240).  The
bounded form (the FP32 and double-word forms) normalises the perpendicular part by its own
length, bounded below by sqrt(min_one_m).  Checked: the two agree within 1e-12 on
well-conditioned unit inputs; near-parallel inputs whose |n| is off by 1e-14 give the
reference's expression a non-unit result and the bounded form a unit one while the
perpendicular part is longer than the bound (below it, a result between cos theta and 1);
exactly parallel inputs leave the bounded form finite."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    build = os.path.join(HERE, "_build")
    os.makedirs(build, exist_ok=True)
    out = os.path.join(build, "libwetting_host.so")
    tmp = out + f".{os.getpid()}"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-std=c++17",
                    os.path.join(HERE, "wetting_host.cpp"), "-o", tmp], check=True)
    os.replace(tmp, out)
    L = C.CDLL(out)
    P64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    P32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    L.wh_f64.argtypes = [P64, P64, C.c_double, C.c_double, C.c_double]
    L.wh_f32.argtypes = [P32, P32, C.c_float, C.c_float, C.c_float]
    return L


def unit(v):
    return v / np.linalg.norm(v)


def wet64(lib, n, nw, theta, bound):
    out = np.ascontiguousarray(n, dtype=np.float64).copy()
    lib.wh_f64(out, np.ascontiguousarray(nw, dtype=np.float64), np.cos(theta), np.sin(theta), bound)
    return out


def test_bounded_form_equals_reference_on_unit_inputs(lib):
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(2000):
        nw = unit(rng.normal(size=3))
        n = unit(rng.normal(size=3))
        if abs(nw @ n) > 0.985:     # angle below 10 deg: the ill-conditioned band
            continue
        theta = rng.uniform(0.2, 2.9)
        a = wet64(lib, n, nw, theta, 0.0)
        b = wet64(lib, n, nw, theta, 1e-12)
        worst = max(worst, np.abs(a - b).max())
        assert abs(np.linalg.norm(b) - 1.0) <= 1e-14
        # the result makes the contact angle with the wall normal
        assert abs(b @ nw - np.cos(theta)) <= 1e-13
    assert worst <= 1e-12


def test_near_parallel_inputs(lib):
    """Perpendicular parts of 1e-5 to 1e-3 (above the double-word bound of 1e-6): the bounded
    form stays unit, the reference's expression does not.  Below the bound (1e-8 to 1e-6)
    the bounded form shortens the perpendicular part: |result| between cos theta and 1."""
    rng = np.random.default_rng(4)
    theta = np.pi / 6
    ref_dev, bnd_dev = 0.0, 0.0
    for lo, hi, above in ((-5, -3, True), (-8, -6, False)):
        for _ in range(500):
            nw = unit(rng.normal(size=3))
            perp = unit(np.cross(nw, rng.normal(size=3)))
            n = unit(nw + 10.0 ** rng.uniform(lo, hi) * perp) * (1.0 + 1e-14 * rng.choice([-1, 1]))
            a = wet64(lib, n, nw, theta, 0.0)
            b = wet64(lib, n, nw, theta, 1e-12)
            if above:
                if np.all(np.isfinite(a)):
                    ref_dev = max(ref_dev, abs(np.linalg.norm(a) - 1.0))
                bnd_dev = max(bnd_dev, abs(np.linalg.norm(b) - 1.0))
            else:
                assert np.all(np.isfinite(b))
                assert np.cos(theta) - 1e-12 <= np.linalg.norm(b) <= 1.0 + 1e-12
    print(f"perpendicular 1e-5..1e-3: max ||n| - 1| reference expression {ref_dev:.3e}, bounded form {bnd_dev:.3e}")
    assert ref_dev > 1e-6
    assert bnd_dev <= 1e-9


@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_exactly_parallel_inputs_stay_finite(lib, sign):
    nw = unit(np.array([1.0, 2.0, -2.0]))
    b = wet64(lib, sign * nw, nw, np.pi / 6, 1e-12)
    assert np.all(np.isfinite(b)) and np.linalg.norm(b) <= 1.0 + 1e-12
    n32 = (sign * nw).astype(np.float32)
    lib.wh_f32(n32, nw.astype(np.float32), np.float32(np.cos(np.pi / 6)), np.float32(0.5), np.float32(1e-6))
    assert np.all(np.isfinite(n32)) and np.linalg.norm(n32) <= 1.0 + 1e-5
