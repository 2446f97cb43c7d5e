"""Double-word (float-float) arithmetic of the FP64-storage / FP32-pipe collision
(mf-lbm_gb300/csrc/ffloat.cuh), built for the host with the CUDA rounding intrinsics
mapped onto IEEE operations, against exact rational arithmetic:
  - FP64 -> (hi, lo) on the integer pipe: |d - (hi + lo)| <= 2^-47 |d|
  - FP32 -> FP64 on the integer pipe: exact for normal numbers, subnormals flush to a
    signed zero, infinities and NaN kept
  - (hi, lo) -> FP64: hi + lo rounded once
  - sum, difference: absolute error <= 2^-46 (|x| + |y|), also for unnormalised inputs
  - products and quotients: relative error <= 2^-45 (2^-44 for quotients); power-of-two
    scaling exact
"""
import ctypes as C
import os
import shutil
import subprocess
from fractions import Fraction

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
    out = os.path.join(build, "libffloat_host.so")
    tmp = out + f".{os.getpid()}"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-std=c++17",
                    os.path.join(HERE, "ffloat_host.cpp"), "-o", tmp], check=True)
    os.replace(tmp, out)
    L = C.CDLL(out)
    P = np.ctypeslib.ndpointer
    L.ffh_from_f64.argtypes = [P(np.float64), P(np.float32), P(np.float32), C.c_int]
    L.ffh_from_f64_in_range.argtypes = [P(np.float64), P(np.float32), P(np.float32), P(np.int32), C.c_int]
    L.ffh_to_f64.argtypes = [P(np.float32), P(np.float32), P(np.float64), C.c_int]
    L.ffh_f32_to_f64.argtypes = [P(np.float32), P(np.float64), C.c_int]
    L.ffh_op.argtypes = [C.c_int] + [P(np.float32)] * 6 + [C.c_int]
    L.ffh_const.argtypes = [C.c_double, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    return L


def split(L, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    hi, lo = np.empty(d.size, np.float32), np.empty(d.size, np.float32)
    L.ffh_from_f64(d, hi, lo, d.size)
    return hi, lo


def op(L, k, x, y):
    n = x[0].size
    zh, zl = np.empty(n, np.float32), np.empty(n, np.float32)
    L.ffh_op(k, x[0], x[1], y[0], y[1], zh, zl, n)
    return zh, zl


def exact(h, l):
    return [Fraction(float(a)) + Fraction(float(b)) for a, b in zip(h, l)]


def rand_doubles(rng, n, lo=-20, hi=5):
    return rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(lo, hi, n) * (1 + rng.random(n))


def test_split_bound_and_round_trip(lib):
    rng = np.random.default_rng(1)
    d = np.concatenate([rand_doubles(rng, 3000), rng.random(500) * 0.3, [1.0, -1.0, 0.5, 1 / 3, 2.0 ** -103,
                                                                       2.0 ** 127 * 1.5]])
    hi, lo = split(lib, d)
    for v, e in zip(d, exact(hi, lo)):
        assert abs(Fraction(float(v)) - e) <= Fraction(2) ** -47 * abs(Fraction(float(v))), v
    back = np.empty(d.size)
    lib.ffh_to_f64(hi, lo, back, d.size)
    assert np.all(np.abs(back - d) <= 2.0 ** -46 * np.abs(d))


def test_split_special_values(lib):
    d = np.array([0.0, -0.0, 1e-35, -1e-40, 1e300, np.inf, -np.inf, np.nan, -np.nan, 2.0 ** -126, 2.0 ** -127])
    hi, lo = split(lib, d)
    assert np.array_equal(hi[:2], [0.0, 0.0]) and np.array_equal(np.signbit(hi[:2]), [False, True])
    assert np.all(lo[:7] == 0) and np.all(lo[9:] == 0)
    assert abs(float(hi[2]) - 1e-35) <= 2.0 ** -23 * 1e-35          # hi truncated, lo below range
    assert hi[3] == 0.0 and np.signbit(hi[3])                         # below 2^-126: signed zero
    assert np.isposinf(hi[4]) and np.isposinf(hi[5]) and np.isneginf(hi[6]) and np.isnan(hi[7]) and np.isnan(hi[8])
    assert hi[9] == np.float32(2.0 ** -126) and hi[10] == 0.0


def test_in_range_split_matches_general_split(lib):
    """The select-free split of the sweeps: bit-identical hi and lo for every |d| in
    [2^-103, 2^128), and every value outside that range reported (zero, subnormals, tiny,
    huge, infinities, NaN), so the sweep falls back to the general split for it."""
    rng = np.random.default_rng(7)
    inside = np.concatenate([rand_doubles(rng, 4000, -30, 30), rng.random(1000) * 0.3, 1 / 3 + 1e-9 * rng.random(500),
                             [2.0 ** -103, -(2.0 ** -103), np.nextafter(2.0 ** 128, 0), 1.0, -1.0]])
    outside = np.array([0.0, -0.0, 2.0 ** -103 * (1 - 2.0 ** -52), 1e-35, -1e-40, 5e-324, 2.0 ** 128, 1e300,
                        np.inf, -np.inf, np.nan, -np.nan])
    d = np.concatenate([inside, outside])
    hi, lo = np.empty(d.size, np.float32), np.empty(d.size, np.float32)
    ok = np.empty(d.size, np.int32)
    lib.ffh_from_f64_in_range(d, hi, lo, ok, d.size)
    ghi, glo = split(lib, d)
    n = inside.size
    assert ok[:n].all() and not ok[n:].any()
    assert np.array_equal(hi[:n].view(np.uint32), ghi[:n].view(np.uint32))
    assert np.array_equal(lo[:n].view(np.uint32), glo[:n].view(np.uint32))


def test_f32_to_f64_exact(lib):
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = np.concatenate([x, np.array([0.0, -0.0, 1e-45, -1e-40, np.inf, -np.inf, np.nan, 3.4e38],
                                    dtype=np.float32)])
    out = np.empty(x.size)
    lib.ffh_f32_to_f64(x, out, x.size)
    with np.errstate(invalid="ignore"):
        ref = x.astype(np.float64)
    # FP32 subnormals flush to a signed zero
    ref = np.where(np.abs(ref) < 2.0 ** -126, np.copysign(0.0, ref), ref)
    same = (out == ref) | (np.isnan(out) & np.isnan(ref))
    assert same.all()
    assert np.array_equal(np.signbit(out), np.signbit(ref))


def test_constants(lib):
    for v in (0.1, 1 / 19, -475 / 63 / 252, 1e-6, 2.0):
        h, l = C.c_float(), C.c_float()
        lib.ffh_const(v, C.byref(h), C.byref(l))
        assert abs(Fraction(h.value) + Fraction(l.value) - Fraction(v)) <= Fraction(2) ** -48 * abs(Fraction(v))


@pytest.mark.parametrize("k", [0, 1])
def test_sum_and_difference(lib, k):
    rng = np.random.default_rng(3 + k)
    n = 3000
    # populations of similar magnitude (cancellation) and of very different magnitudes
    a = np.concatenate([0.05 + 1e-6 * rng.normal(size=n // 2), rand_doubles(rng, n // 2, -8, 1)])
    b = np.concatenate([0.05 + 1e-6 * rng.normal(size=n // 2), rand_doubles(rng, n // 2, -8, 1)])
    x, y = split(lib, a), split(lib, b)
    z = op(lib, k, x, y)
    ex, ey, ez = exact(*x), exact(*y), exact(*z)
    sgn = 1 if k == 0 else -1
    for u, v, w in zip(ex, ey, ez):
        assert abs(w - (u + sgn * v)) <= Fraction(2) ** -46 * (abs(u) + abs(v))


def test_unnormalised_chain(lib):
    """Twenty chained sums without renormalisation (the collision's moment sums)."""
    rng = np.random.default_rng(5)
    n = 1000
    terms = [rng.choice([-1, 1], n) * (0.01 + 0.3 * rng.random(n)) for _ in range(20)]
    acc = split(lib, terms[0])
    ref = exact(*acc)
    mag = [abs(r) for r in ref]
    for t in terms[1:]:
        y = split(lib, t)
        acc = op(lib, 0, acc, y)
        ey = exact(*y)
        ref = [r + v for r, v in zip(ref, ey)]
        mag = [m + abs(v) for m, v in zip(mag, ey)]
    for w, r, m in zip(exact(*acc), ref, mag):
        assert abs(w - r) <= 20 * Fraction(2) ** -46 * m


def test_products(lib):
    rng = np.random.default_rng(6)
    n = 3000
    x, y = split(lib, rand_doubles(rng, n, -10, 2)), split(lib, rand_doubles(rng, n, -10, 2))
    for k in (2, 3):
        z = op(lib, k, x, y)
        yy = exact(*y) if k == 2 else [Fraction(float(h)) for h in y[0]]
        for u, v, w in zip(exact(*x), yy, exact(*z)):
            assert abs(w - u * v) <= Fraction(2) ** -45 * abs(u * v)
    z = op(lib, 4, x, y)
    for u, w in zip(exact(*x), exact(*z)):
        assert w == u / 2


def test_quotients(lib):
    rng = np.random.default_rng(7)
    n = 3000
    x = split(lib, rand_doubles(rng, n, -8, 3))
    # divisors of the collision: densities near 1, viscosity terms, la_weight sums
    y = split(lib, np.concatenate([1.0 + 1e-3 * rng.normal(size=n // 2), rand_doubles(rng, n // 2, -3, 2)]))
    z = op(lib, 5, x, y)
    for u, v, w in zip(exact(*x), exact(*y), exact(*z)):
        assert abs(w - u / v) <= Fraction(2) ** -44 * abs(u / v)


def test_square_roots(lib):
    rng = np.random.default_rng(8)
    n = 3000
    v = np.abs(rand_doubles(rng, n, -20, 6))
    x = split(lib, v)
    z = op(lib, 6, x, x)
    for u, w in zip(exact(*x), exact(*z)):
        # |w - sqrt(u)| <= 2^-45 sqrt(u)  <=>  |w^2 - u| <= ~2^-44 u
        assert abs(w * w - u) <= Fraction(2) ** -44 * u
    z0 = op(lib, 6, split(lib, np.zeros(4)), split(lib, np.zeros(4)))
    assert np.all(z0[0] == 0) and np.all(z0[1] == 0)
