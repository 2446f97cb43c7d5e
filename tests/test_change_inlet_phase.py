"""change_inlet_fluid_phase (multiphase_3D/0.src/Misc.F90:507-621).

CPU: the oracle's restatement against numpy on the halo-1 state (f + g moved into one
species for z <= interface_z0, the other species emptied, every other slot untouched).
GPU: the library's device-side update against the oracle, strict build bit-identical on
the whole state right after the change and after 4 further steps, for both commands;
the FP32 form keeps f + g to FP32 rounding.
"""
import copy

import numpy as np
import pytest

from cases import load_case, mp_case
from pyoracle import Oracle

Z0 = 5.5


@pytest.mark.parametrize("cmd", [1, 2])
def test_oracle_change_against_numpy(cmd):
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1)
    o = Oracle(case["params"])
    load_case(o, case)
    a = o.download_state()
    o.change_inlet_fluid_phase(cmd, Z0)
    b = o.download_state()
    o.close()
    k = np.arange(a["f"].shape[1])            # halo-1 index k = z
    sel = (k <= Z0)[None, :, None, None]
    tot = a["f"] + a["g"]
    into, out = ("f", "g") if cmd == 1 else ("g", "f")
    assert np.array_equal(b[into], np.where(sel, tot, a[into]))
    assert np.array_equal(b[out], np.where(sel, 0.0, a[out]))
    assert np.array_equal(b["phi"], a["phi"])


@pytest.mark.gpu
@pytest.mark.parametrize("cmd", [1, 2])
def test_gpu_change_matches_oracle(cmd):
    from mflbm import Solver
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1, strict=1)
    sims = [Solver(case["params"]), Oracle(case["params"])]
    states = []
    for sim in sims:
        load_case(sim, case)
        sim.run(1, 2)
        sim.change_inlet_fluid_phase(cmd, Z0)
        s1 = sim.download_state()
        sim.color_gradient()                  # as the reference does before its first step
        sim.run(3, 4)
        states.append((s1, sim.download_state()))
        sim.close()
    (g1, g2), (o1, o2) = states
    for k in ("f", "g", "phi"):
        assert np.array_equal(g1[k], o1[k]), k
        assert np.array_equal(g2[k], o2[k]), k


@pytest.mark.gpu
def test_gpu_change_fp32_form():
    from mflbm import Solver
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1, strict=0)
    p = copy.copy(case["params"])
    p.precision = 1
    with Solver(p) as sim:
        load_case(sim, case)
        a = sim.download_state()
        sim.change_inlet_fluid_phase(2, Z0)
        b = sim.download_state()
    k = np.arange(a["f"].shape[1])
    sel = (k <= Z0)[None, :, None, None]
    np.testing.assert_allclose(b["g"], np.where(sel, a["f"] + a["g"], a["g"]), rtol=2e-7, atol=1e-7)
    assert np.all(np.where(sel, b["f"], 0.0) == 0.0)
    assert np.array_equal(np.where(sel, 0.0, b["f"]), np.where(sel, 0.0, a["f"]))
