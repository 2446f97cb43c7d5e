"""mflbm_saturation_noalloc: the saturation sums for callers that cannot allocate.

A Fortran/OpenACC host keeps phi and walls in its own device arrays and passes their
device addresses; the library must not allocate.  This checks, through the C ABI, that
two calls in a row on two different phase fields give the same (vol1, vol2) as the
context-based mflbm_saturation and as the oracle's cal_saturation on the same data, that
the largest accepted nz fills the last scratch slot correctly (against a numpy sum), and
that oversized inputs are rejected before any device work.  Device buffers here come from
torch, standing in for the caller's own arrays.
"""
import ctypes as C

import numpy as np
import pytest

from cases import load_case, mp_case
from mflbm import Solver, _capi
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(lib, phi, walls, nx, ny, nz):
    d_phi = torch.from_numpy(np.ascontiguousarray(phi)).cuda()
    d_walls = torch.from_numpy(np.ascontiguousarray(walls)).cuda()
    d_vol = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.mflbm_saturation_noalloc(C.c_void_p(d_phi.data_ptr()), C.c_void_p(d_walls.data_ptr()), nx, ny, nz,
                                      C.c_void_p(d_vol.data_ptr()), None)
    assert rc == _capi.MFLBM_OK, lib.mflbm_last_error(None)
    torch.cuda.synchronize()
    return d_vol.cpu().numpy()


def test_two_calls_match_context_saturation():
    lib = _capi.load()
    case = mp_case(nx=20, ny=14, nz=24, per=(0, 1, 0), inlet=1, outlet=1, spheres=3, strict=0)
    p = case["params"]
    sim = Solver(p)
    load_case(sim, case)
    orc = Oracle(p)
    load_case(orc, case)
    # call 1: the initial phase field
    ref1 = np.array(sim.saturation())
    got1 = _noalloc(lib, case["phi"], case["walls"], p.nx, p.ny, p.nz)
    np.testing.assert_allclose(got1, ref1, rtol=1e-13)
    np.testing.assert_allclose(got1, np.array(orc.saturation()), rtol=1e-13)
    # call 2: the field after a few steps; the shared scratch still holds call 1's sums
    sim.run(1, 6)
    orc.run(1, 6)
    phi2 = sim.download_state()["phi"]
    ref2 = np.array(sim.saturation())
    got2 = _noalloc(lib, phi2, case["walls"], p.nx, p.ny, p.nz)
    np.testing.assert_allclose(got2, ref2, rtol=1e-13)
    # the oracle's cal_saturation on its own state after the same steps (default build: FMA)
    np.testing.assert_allclose(got2, np.array(orc.saturation()), rtol=1e-12)
    assert not np.allclose(got1, got2, rtol=0, atol=0)
    sim.close()
    orc.close()


def _numpy_saturation(phi, walls, nx, ny, nz):
    m = 1.0 - walls[2:nz + 2, 2:ny + 2, 2:nx + 2].astype(np.float64)
    ph = phi[4:nz + 4, 4:ny + 4, 4:nx + 4]
    return np.array([(0.5 * (1.0 + ph) * m).sum(), (0.5 * (1.0 - ph) * m).sum()])


@pytest.mark.parametrize("nx,ny,nz", [(1, 1, _capi.MFLBM_NOALLOC_MAX_NZ), (37, 29, 3)])
def test_scratch_edges_against_numpy(nx, ny, nz):
    """nz at the limit writes the last scratch slot and the finish kernel sums all of them;
    a slice of nx*ny > 256 cells makes every thread of a block loop."""
    lib = _capi.load()
    rng = np.random.default_rng(nz + nx)
    phi = rng.uniform(-1.0, 1.0, (nz + 8, ny + 8, nx + 8))
    walls = (rng.uniform(size=(nz + 4, ny + 4, nx + 4)) < 0.3).astype(np.int8)
    got = _noalloc(lib, phi, walls, nx, ny, nz)
    np.testing.assert_allclose(got, _numpy_saturation(phi, walls, nx, ny, nz), rtol=1e-11)


def test_oversized_input_rejected():
    lib = _capi.load()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.mflbm_saturation_noalloc(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), 4, 4,
                                      _capi.MFLBM_NOALLOC_MAX_NZ + 1, C.c_void_p(d.data_ptr()), None)
    assert rc == _capi.MFLBM_ERANGE
    assert b"exceeds the scratch limit" in lib.mflbm_last_error(None)
