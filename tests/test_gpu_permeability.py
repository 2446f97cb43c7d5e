"""Time-to-steady permeability on a 48^3 sphere packing (porosity 0.3): the GPU FP64 form
against the oracle, and the FP32 / FP16-deviation forms against the GPU FP64 result.

FP64 (default FMA build): same number of steps to |du|/u < 1e-7 and |dk|/k <= 1e-9.
FP32 deviation storage: converges to 1e-7, |dk|/k <= 1e-3 against FP64.
FP16 deviation storage: its rounding noise floor sits above 1e-7, so it is run to 1e-5;
its 11-bit significand leaves a systematic k error of several 1e-3: |dk|/k <= 2e-2.
FP64 storage with the double-word collision, and double-word storage with it: the same
number of steps as FP64 (+-100, one check interval) and |dk|/k <= 1e-8.
"""
import numpy as np
import pytest

from mflbm import Solver, workloads
from mflbm.permeability import run_to_steady
from pyoracle import Oracle

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

TOL = 1e-7


def _case(precision):
    return workloads.packing_permeability(n=48, porosity=0.3, seed=5, precision=precision)


def _solve(sim, case, tol=TOL):
    sim.set_geometry(case["walls"])
    sim.init_equilibrium()
    return run_to_steady(sim, case["params"], check_every=100, tol=tol, max_steps=60000)


@pytest.fixture(scope="module")
def fp64():
    case = _case(0)
    with Solver(case["params"]) as sim:
        return _solve(sim, case)


def test_fp64_matches_oracle(fp64):
    case = _case(0)
    o = Oracle(case["params"], variant="fast")
    ref = _solve(o, case)
    o.close()
    assert ref.converged and fp64.converged
    assert fp64.steps == ref.steps
    print(f"k oracle {ref.k:.15e} gpu {fp64.k:.15e} steps {ref.steps}")
    assert abs(fp64.k - ref.k) / abs(ref.k) <= 1e-9


@pytest.mark.parametrize("precision", [3, 4])
def test_double_word_collision_matches_fp64(fp64, precision):
    case = _case(precision)
    with Solver(case["params"]) as sim:
        r = _solve(sim, case)
    err = abs(r.k - fp64.k) / abs(fp64.k)
    print(f"double-word precision {precision}: k {r.k:.15e} vs fp64 {fp64.k:.15e} rel {err:.3e} steps {r.steps} vs {fp64.steps}")
    assert r.converged and r.status == 0
    assert abs(r.steps - fp64.steps) <= 100
    assert err <= 1e-8


@pytest.mark.parametrize("precision", [1, 2])
def test_mixed_forms_within_1e3(fp64, precision):
    case = _case(precision)
    with Solver(case["params"]) as sim:
        r = _solve(sim, case, tol=TOL if precision == 1 else 1e-5)
    err = abs(r.k - fp64.k) / abs(fp64.k)
    print(f"precision {precision}: k {r.k:.10e} vs fp64 {fp64.k:.10e} rel {err:.3e} steps {r.steps} vs {fp64.steps}")
    assert r.converged and r.status == 0
    assert err <= (1e-3 if precision == 1 else 2e-2)
