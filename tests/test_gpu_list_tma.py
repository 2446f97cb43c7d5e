"""The even step of the fluid-list sweep through the tensor memory accelerator (tiled
cp.async.bulk.tensor loads and stores of 19 x 128 boxes, warp-specialised, persistent
grid) against the plain even step of the same build: bit-identical PDFs in every storage
form, on a packing whose fluid-node count is not a multiple of the 128-node tile (the
last tile is clipped by the tensor's extent) and large enough that blocks take several
tiles.  MFLBM_NO_TMA (read when the geometry is set) selects the plain even step.  The
strict-build list tests against the oracle run through the TMA path as well.
"""
import os

import numpy as np
import pytest

from mflbm import Solver, workloads

pytestmark = pytest.mark.gpu


def _run(case, steps, plain):
    if plain:
        os.environ["MFLBM_NO_TMA"] = "1"
    try:
        with Solver(case["params"]) as sim:
            sim.set_geometry(case["walls"])
            sim.init_equilibrium()
            sim.run(1, steps)
            st = sim.download_state()["f"]
            prof, _, status = sim.monitor() if steps % 2 == 0 else (None, None, 0)
    finally:
        os.environ.pop("MFLBM_NO_TMA", None)
    return st, prof, status


@pytest.mark.parametrize("precision", [0, 1, 2, 3, 4])
def test_small_odd_node_count(precision):
    """1,513 fluid nodes: eleven whole tiles plus 105 nodes for the plain tail, and nf * 8
    bytes not a multiple of 16 (a box clipped at the tensor's extent would reach the first
    link slot)."""
    from cases import periodic_ghosts, sp_case
    case = sp_case(per=(1, 1, 1), spheres=4, force=1e-5, rest="mrt", precision=precision, strict=0)
    case["f"] = periodic_ghosts(case["f"], (1, 1, 1))
    out = []
    for plain in (False, True):
        if plain:
            os.environ["MFLBM_NO_TMA"] = "1"
        try:
            with Solver(case["params"]) as sim:
                sim.set_geometry(case["walls"])
                sim.upload_state(case["f"])
                sim.run(1, 5)
                out.append(sim.download_state()["f"])
        finally:
            os.environ.pop("MFLBM_NO_TMA", None)
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("precision", [0, 1, 2, 3, 4])
def test_tma_even_step_equals_plain_even_step(precision):
    case = workloads.packing_permeability(n=96, porosity=0.22, seed=17, precision=precision, force_z=1e-5)
    nf = case["pore"]
    assert nf % 128 != 0 and nf // 128 > 4 * 152     # a clipped last tile, several tiles per block
    for steps in (2, 7):
        a, pa, sa = _run(case, steps, plain=False)
        b, pb, sb = _run(case, steps, plain=True)
        assert np.array_equal(a, b), (precision, steps, np.abs(a - b).max())
        if pa is not None:
            assert sa == 0 and np.array_equal(pa, pb)


