"""The MRT collision forms of mf-lbm_gb300/csrc/collide.cuh built for the host: the
double-word collisions (the singlephase mrt_collide_ff, unit-rate and general; the pair form
instantiated with the double-word type and per-node rates folded at run time, as the
multiphase double-word kernel uses it) against the FP64 pair form on random states near rest
and at velocities up to 0.05: every post-collision population within 2e-14 (populations of
order 0.1; about 48-bit arithmetic).  The FP64 pair form conserves mass (singlephase) and the
unit-rate specialisation equals the general code at unit rates."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


@pytest.fixture(scope="module")
def lib():
    gxx = shutil.which("g++")
    inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if gxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers not available")
    build = os.path.join(HERE, "_build")
    os.makedirs(build, exist_ok=True)
    out = os.path.join(build, "libcollide_host.so")
    tmp = out + f".{os.getpid()}"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-std=c++17", f"-I{inc}",
                    os.path.join(HERE, "collide_host.cpp"), "-o", tmp], check=True)
    os.replace(tmp, out)
    L = C.CDLL(out)
    P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    d = C.c_double
    L.ch_sp.argtypes = [P, d, d, d, d, d, d, d, C.c_int, P, P]
    L.ch_mp.argtypes = [P, d, d, d, d, d, P, P]
    return L


def states(rng, n):
    """Equilibria at density 1 +- 1e-2 and velocity up to 0.05, plus 1e-3 relative noise."""
    out = []
    for _ in range(n):
        rho = 1.0 + 1e-2 * rng.uniform(-1, 1)
        u = 0.05 * rng.uniform(-1, 1, 3) * rng.choice([1e-3, 1e-1, 1.0])
        cu = EX * u[0] + EY * u[1] + EZ * u[2]
        feq = W * rho * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * (u @ u))
        out.append(np.ascontiguousarray(feq * (1 + 1e-3 * rng.uniform(-1, 1, 19))))
    return out


def rates(nu, preset1=True):
    om = 1.0 / (3.0 * nu + 0.5)
    sq = 8.0 * (2.0 - om) / (8.0 - om) if preset1 else om
    return (om, om, sq, om, om, sq)


@pytest.mark.parametrize("nu,preset1,unit", [(1 / 6, True, 1), (1 / 6, True, 0), (0.1, True, 0), (0.02, True, 0),
                                             (0.05, False, 0)])
def test_singlephase_double_word_collision(lib, nu, preset1, unit):
    rng = np.random.default_rng(11)
    r = rates(nu, preset1)
    worst = 0.0
    for f in states(rng, 400):
        a, b = np.empty(19), np.empty(19)
        lib.ch_sp(f, *r, 1e-5, unit, a, b)
        worst = max(worst, np.abs(a - b).max())
        # the collision conserves mass
        assert abs(a.sum() - f.sum()) <= 1e-15
    print(f"nu {nu} preset1 {preset1} unit {unit}: max |ff - f64| {worst:.3e}")
    assert worst <= 2e-14


def test_unit_rate_specialisation_equals_general_code(lib):
    rng = np.random.default_rng(12)
    r = rates(1 / 6)
    for f in states(rng, 100):
        a1, b1, a0, b0 = (np.empty(19) for _ in range(4))
        lib.ch_sp(f, *r, 1e-5, 1, a1, b1)
        lib.ch_sp(f, *r, 1e-5, 0, a0, b0)
        assert np.abs(a1 - a0).max() <= 1e-16
        assert np.abs(b1 - b0).max() <= 2e-14


@pytest.mark.parametrize("omega", [0.6, 1.0, 1.3, 1.9])
def test_multiphase_double_word_collision(lib, omega):
    rng = np.random.default_rng(13)
    worst = 0.0
    for f in states(rng, 300):
        den = f.sum() * (1 + 1e-3 * rng.uniform(-1, 1))
        fx, fy, fz = 1e-4 * rng.uniform(-1, 1, 3)
        a, b = np.empty(19), np.empty(19)
        lib.ch_mp(f, den, fx, fy, fz, omega, a, b)
        worst = max(worst, np.abs(a - b).max())
    print(f"omega {omega}: max |ff - f64| {worst:.3e}")
    assert worst <= 2e-14
