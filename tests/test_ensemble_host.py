"""Host logic of the ensemble driver (mflbm/ensemble.py) on the CPU, with a scripted stand-in
for the device ensemble: samples leave the active set one by one as each meets the
stopping rule, the update count follows the active samples, a failure status ends the
loop, and the autotuner's choice is cached per precision and arena size."""
import json
import types

import numpy as np

from mflbm.ensemble import run_to_steady, tune_cached


class _FakeEnsemble:
    """flux() reports scripted mean velocities (one list per sample) times the volumes."""

    def __init__(self, series, precision=1, nodes=5000, fail_at=None):
        self.series = [list(s) for s in series]
        self.n = len(series)
        self.p = types.SimpleNamespace(precision=precision, la_nu1=1.0 / 6.0, force_z=1e-6)
        self.volume = np.full(self.n, 8.0)
        self.checks = 0
        self.active_log = []
        self.nodes = nodes
        self.fail_at = fail_at
        self.tuned = 0
        self.configured = None

    def set_active(self, active):
        self.active_log.append(np.array(active).copy())

    def run(self, ntime0, nsteps):
        self.checks += 1

    def flux(self):
        u = np.array([s[min(self.checks, len(s)) - 1] for s in self.series])
        st = 3 if self.fail_at is not None and self.checks >= self.fail_at else 0
        return u * self.volume, np.zeros(self.n), st

    def info(self):
        return {"active_nodes": self.nodes}

    def tune(self, steps):
        self.tuned += 1
        return {"chosen": {"block": 256, "persistent": 1}, "candidates": [{"block": 128}, {"block": 256}]}

    def configure(self, block, persistent):
        self.configured = (block, persistent)


def test_samples_leave_the_active_set_one_by_one():
    # sample 0 settles at the 2nd check, sample 1 at the 4th, sample 2 never within the cap
    ens = _FakeEnsemble([[1.0, 1.0, 5.0, 5.0, 5.0],
                         [1.0, 2.0, 3.0, 3.0, 3.0],
                         [1.0, 2.0, 4.0, 8.0, 16.0]])
    nf = np.array([10, 20, 30])
    r = run_to_steady(ens, nf, check_every=100, tol=1e-7, max_steps=500)
    assert list(r.converged) == [True, True, False]
    assert list(r.steps) == [200, 400, 500]
    np.testing.assert_allclose(r.k, np.array([1.0, 3.0, 16.0]) * (1.0 / 6.0) / 1e-6)
    # the device's active set: all, then without sample 0, then without samples 0 and 1
    assert [list(a) for a in ens.active_log] == [[1, 1, 1], [0, 1, 1], [0, 0, 1]]
    # fluid-node updates of the active samples only
    assert r.fluid_updates == 100 * (60 + 60 + 50 + 50 + 30)
    assert r.status == 0


def test_failure_status_ends_the_loop():
    ens = _FakeEnsemble([[1.0, 2.0, 3.0]] * 2, fail_at=2)
    r = run_to_steady(ens, np.array([5, 5]), check_every=100, tol=1e-7, max_steps=10000)
    assert r.status == 3 and not r.converged.any() and ens.checks == 2


def test_tuner_choice_cached_per_precision_and_size(tmp_path):
    cache = tmp_path / "sub" / "tune.json"
    a = _FakeEnsemble([[1.0]], precision=1, nodes=5000)
    rep = tune_cached(a, str(cache), steps=4)
    assert a.tuned == 1 and "cached" not in rep
    b = _FakeEnsemble([[1.0]], precision=1, nodes=6000)      # same power-of-two size class
    rep = tune_cached(b, str(cache))
    assert rep["cached"] and b.tuned == 0 and b.configured == (256, 1)
    c = _FakeEnsemble([[1.0]], precision=4, nodes=5000)      # another precision: tuned again
    tune_cached(c, str(cache))
    assert c.tuned == 1
    assert sorted(json.load(open(cache))) == ["prec1_nodes2^12", "prec4_nodes2^12"]
    cache.write_text("{not json")                             # a damaged cache is replaced
    d = _FakeEnsemble([[1.0]], precision=1, nodes=5000)
    tune_cached(d, str(cache))
    assert d.tuned == 1 and list(json.load(open(cache))) == ["prec1_nodes2^12"]
