"""Checkpoint files through a GPU context (save_checkpoint, IO_multiphase.F90:562-642;
initialization_old_multi, Init_multiphase.F90:477-557).

A run saved by the library resumes on the oracle, and a run saved by the oracle resumes
on the library; in the strict build both continuations are bit-identical to the run that
never stopped.  The singlephase fluid-list layout writes the dense picture of its state
(fluid nodes and bounce-back slots exact, unused slots at rest); the oracle resumed from
it matches on every fluid node.
"""
import numpy as np
import pytest

from cases import load_case, mp_case, periodic_ghosts, sp_case
from mflbm import Solver, checkpoint
from pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _fresh(cls, case):
    sim = cls(case["params"])
    load_case(sim, case)
    return sim


@pytest.mark.parametrize("first,second", [(Solver, Oracle), (Oracle, Solver)])
def test_multiphase_resume_across_gpu_and_oracle(tmp_path, first, second):
    case = mp_case(nx=12, ny=10, nz=16, per=(0, 0, 0), inlet=1, outlet=1, strict=1)
    a = _fresh(first, case)
    a.run(1, 6)
    checkpoint.save(a, str(tmp_path), ntime=6)
    a.run(7, 6)                                  # the run that never stopped
    b = second(case["params"])
    b.set_geometry(case["walls"], case["solid"], case["fluid"], case["w_in"])
    ntime0, fz, rin = checkpoint.load(b, str(tmp_path))
    assert ntime0 == 7 and fz == case["params"].force_z
    b.run(ntime0, 6)
    sa, sb = a.download_state(), b.download_state()
    for k in ("f", "g", "phi", "f_convec", "g_convec", "phi_convec"):
        assert np.array_equal(sa[k], sb[k]), k
    a.close()
    b.close()


def test_singlephase_list_layout_checkpoint_resumes_on_oracle(tmp_path):
    case = sp_case(per=(1, 1, 1), force=1e-5, strict=1, rest="mrt")
    case["f"] = periodic_ghosts(case["f"], (1, 1, 1))
    gpu = _fresh(Solver, case)
    assert gpu.layout == 2
    gpu.run(1, 6)
    checkpoint.save(gpu, str(tmp_path), ntime=6)
    gpu.run(7, 6)
    orc = Oracle(case["params"])
    orc.set_geometry(case["walls"])
    ntime0, _, _ = checkpoint.load(orc, str(tmp_path))
    orc.run(ntime0, 6)
    fluid = case["walls"][2:-2, 2:-2, 2:-2] == 0
    a = gpu.download_state()["f"][:, 1:-1, 1:-1, 1:-1][:, fluid]
    b = orc.download_state()["f"][:, 1:-1, 1:-1, 1:-1][:, fluid]
    assert np.array_equal(a, b)
    gpu.close()
    orc.close()
