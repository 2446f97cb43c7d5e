"""Bounded device waits in their timeout direction.

Every spin in device code has a limit, after which the kernel records an error that the
host reads, returns, and leaves the context usable.  These tests make two such waits run
out on purpose, without any fault: the persistent ensemble kernel is given a grid
barrier that waits for one block more than the grid holds, and the tensor-core GEMM is
told to issue no MMA and no commit, so its mbarrier phases never complete.  Each wait
gets a short limit (10^3 polls), the call must come back with the error reported, and
the same object must then compute correctly again.
"""
import time

import numpy as np
import pytest

from mflbm import _capi, workloads
from mflbm.ensemble import Ensemble

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _case():
    return workloads.packing_ensemble(n_samples=4, edge_lo=16, edge_hi=24, por_lo=0.3, por_hi=0.4, seed=9, precision=1)


def test_grid_barrier_timeout_is_reported_and_cleared():
    case = _case()
    with Ensemble(case["params"], case["samples"]) as ref:
        ref.configure(128, 0)
        ref.init()
        ref.run(1, 10)
        w_ref = ref.flux()[0]
    with Ensemble(case["params"], case["samples"]) as ens:
        ens.configure(128, 1)            # one cooperative launch per run, grid barriers between steps
        ens.set_wait(1000, unreachable=True)
        ens.init()
        t0 = time.perf_counter()
        ens.run(1, 6)
        with pytest.raises(_capi.MflbmError) as exc:
            ens.flux()
        assert exc.value.code == _capi.MFLBM_ETIMEOUT
        assert time.perf_counter() - t0 < 30.0
        # default limit, reachable barrier: the error word is cleared and the run is exact
        ens.set_wait(0, unreachable=False)
        ens.init()
        ens.run(1, 10)
        w, _, st = ens.flux()
        assert st == _capi.MFLBM_RUNNING
        assert np.array_equal(w, w_ref)


def _gemm(lib, A, B, Cm, err):
    M, K = A.shape
    N = B.shape[0]
    rc = lib.mflbm_nn_gemm_bf16(A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0), Cm.data_ptr(), Cm.stride(0),
                                M, N, K, 0, err.data_ptr(), None)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("K", [64, 512])
def test_gemm_mbarrier_timeout_is_reported_and_cleared(K):
    lib = _capi.load()
    g = torch.Generator(device="cuda").manual_seed(K)
    A = torch.randn(384, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(32, K, device="cuda", generator=g).to(torch.bfloat16)
    Cm = torch.zeros(384, 32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    try:
        assert lib.mflbm_nn_set_wait(1000, 1) == _capi.MFLBM_OK
        t0 = time.perf_counter()
        assert _gemm(lib, A, B, Cm, err) == _capi.MFLBM_OK
        assert int(err.item()) == 1
        assert time.perf_counter() - t0 < 30.0
    finally:
        lib.mflbm_nn_set_wait(0, 0)
    err.zero_()
    assert _gemm(lib, A, B, Cm, err) == _capi.MFLBM_OK
    assert int(err.item()) == 0
    torch.testing.assert_close(Cm, A.float() @ B.float().t(), rtol=1e-4, atol=1e-3)
