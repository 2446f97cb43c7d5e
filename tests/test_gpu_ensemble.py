"""Ensembles: samples of uneven sizes in one arena against independent single-sample
runs of the same geometry, on the GPU and on the oracle.

Same arithmetic as the single-sample fluid-list sweep, so the per-sample flow sums agree
to summation order (rtol 1e-12); persistent and per-step launch shapes agree exactly;
inactive samples stay frozen; steady-state permeability per sample equals the
single-sample result (rtol 1e-9, FP64), the double-word ensembles (FP64 storage, and
double-word storage) within 1e-8 of FP64 at the same step counts, and the FP32 ensemble
within 1e-3 of FP64.
"""
import numpy as np
import pytest

from mflbm import Solver, workloads
from mflbm.ensemble import Ensemble, run_to_steady, tune_cached
from mflbm.permeability import run_to_steady as single_steady

pytestmark = pytest.mark.gpu


def _ens(precision=0, n=5, seed=3):
    return workloads.packing_ensemble(n_samples=n, edge_lo=16, edge_hi=30, por_lo=0.3, por_hi=0.4, seed=seed,
                                      precision=precision)


def _single_flux(case, s, steps):
    import copy
    nx, ny, nz, walls = case["samples"][s]
    p = copy.copy(case["params"])
    p.nx, p.ny, p.nz = nx, ny, nz
    with Solver(p) as sim:
        sim.set_geometry(walls)
        sim.init_equilibrium()
        sim.run(1, steps)
        prof, _, _ = sim.monitor()
    return prof[0].sum()


def test_flux_matches_single_sample_runs():
    case = _ens()
    with Ensemble(case["params"], case["samples"]) as ens:
        ens.init()
        ens.run(1, 24)
        w, um, st = ens.flux()
    assert st == 0
    for s in range(len(case["samples"])):
        np.testing.assert_allclose(w[s], _single_flux(case, s, 24), rtol=1e-12)


@pytest.mark.parametrize("strict", [1, 0])
def test_flux_matches_oracle(strict):
    """Every sample of one arena against the oracle's run of that sample alone: strict build
    (no FMA contraction, the populations bit-identical to the oracle's) to summation order,
    rtol 1e-12; default build within 1e-10."""
    import copy
    from pyoracle import Oracle
    case = _ens()
    p = copy.copy(case["params"])
    p.strict_fp = strict
    with Ensemble(p, case["samples"]) as ens:
        ens.init()
        ens.run(1, 24)
        w, _, st = ens.flux()
    assert st == 0
    for s, (nx, ny, nz, walls) in enumerate(case["samples"]):
        ps = copy.copy(p)
        ps.nx, ps.ny, ps.nz = nx, ny, nz
        orc = Oracle(ps)
        orc.set_geometry(walls)
        orc.init_equilibrium()
        orc.run(1, 24)
        prof, _, ost = orc.monitor()
        orc.close()
        assert ost == 0
        np.testing.assert_allclose(w[s], prof[0].sum(), rtol=1e-12 if strict else 1e-10)


@pytest.mark.parametrize("precision", [0, 1, 3, 4])
def test_persistent_equals_per_step_and_inactive_frozen(precision):
    case = _ens(precision)
    out = []
    for pers in (0, 1):
        with Ensemble(case["params"], case["samples"]) as ens:
            ens.configure(128, pers)
            ens.init()
            ens.run(1, 10)
            ens.run(11, 10)
            out.append(ens.flux()[0])
            if pers:
                active = np.ones(ens.n, dtype=np.int32)
                active[1] = 0
                ens.set_active(active)
                ens.run(21, 10)
                w2 = ens.flux()[0]
                assert w2[1] == out[-1][1]
                assert w2[0] != out[-1][0]
                assert ens.info()["active_nodes"] == int(case["nf"].sum() - case["nf"][1])
    assert np.array_equal(out[0], out[1])


def test_tuner_reports_and_applies_a_shape(tmp_path):
    case = _ens()
    with Ensemble(case["params"], case["samples"]) as ens:
        rep = tune_cached(ens, str(tmp_path / "tune.json"), steps=4)
        assert len(rep["candidates"]) >= 2
        info = ens.info()
        assert (info["block"], info["persistent"]) == (rep["chosen"]["block"], rep["chosen"]["persistent"])
        rep2 = tune_cached(ens, str(tmp_path / "tune.json"))
        assert rep2["cached"]


def test_steady_permeability_per_sample():
    case = _ens(0, n=3, seed=5)
    with Ensemble(case["params"], case["samples"]) as ens:
        ens.init()
        r64 = run_to_steady(ens, case["nf"], check_every=100, tol=1e-7, max_steps=40000)
    assert r64.converged.all()
    import copy
    for s in range(3):
        nx, ny, nz, walls = case["samples"][s]
        p = copy.copy(case["params"])
        p.nx, p.ny, p.nz = nx, ny, nz
        with Solver(p) as sim:
            sim.set_geometry(walls)
            sim.init_equilibrium()
            r = single_steady(sim, p, check_every=100, tol=1e-7, max_steps=40000)
        assert r.steps == r64.steps[s]
        np.testing.assert_allclose(r64.k[s], r.k, rtol=1e-9)
    for prec in (3, 4):
        cdw = _ens(prec, n=3, seed=5)
        with Ensemble(cdw["params"], cdw["samples"]) as ens:
            ens.init()
            rdw = run_to_steady(ens, cdw["nf"], check_every=100, tol=1e-7, max_steps=40000)
        print("precision", prec, "k", rdw.k, "rel", np.abs(rdw.k - r64.k) / np.abs(r64.k))
        assert rdw.converged.all()
        assert np.array_equal(rdw.steps, r64.steps)
        assert (np.abs(rdw.k - r64.k) / np.abs(r64.k)).max() <= 1e-8
    case32 = _ens(1, n=3, seed=5)
    with Ensemble(case32["params"], case32["samples"]) as ens:
        ens.init()
        r32 = run_to_steady(ens, case32["nf"], check_every=100, tol=1e-7, max_steps=40000)
    print("k64", r64.k, "k32", r32.k, "steps", r64.steps, r32.steps)
    assert r32.converged.all()
    assert (np.abs(r32.k - r64.k) / np.abs(r64.k)).max() <= 1e-3
