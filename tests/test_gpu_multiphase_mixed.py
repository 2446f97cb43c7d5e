"""Multiphase mixed form (FP32 storage of f, g, phi and the gradient fields, FP32
arithmetic) against the FP64 oracle on short runs of the small cases.

Tolerances (absolute, after 40 steps; PDFs ~0.1, phi in [-1, 1]): f, g <= 2e-5,
phi <= 2e-4.  The FP16 form is rejected for multiphase.
"""
import numpy as np
import pytest

from cases import load_case, mp_case
from mflbm import Solver
from mflbm._capi import MflbmError
from pyoracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "periodic_yz": dict(per=(0, 1, 1)),
    "walled_velocity_inlet_convective": dict(per=(0, 0, 0), inlet=1, outlet=1),
    "pressure_inlet_outlet": dict(per=(0, 1, 0), inlet=2, outlet=2, force=0.0),
    "viscosity_ratio_mrt1": dict(per=(0, 1, 1), mrt=1, nu1=0.1, nu2=0.3),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_form_close_to_fp64_oracle(name):
    kw = CASES[name]
    c64 = mp_case(**kw)
    c32 = mp_case(precision=1, strict=0, **kw)
    orc = Oracle(c64["params"])
    load_case(orc, c64)
    gpu = Solver(c32["params"])
    load_case(gpu, c32)
    orc.run(1, 40)
    gpu.run(1, 40)
    a, b = gpu.download_state(), orc.download_state()
    df = max(np.abs(a["f"] - b["f"]).max(), np.abs(a["g"] - b["g"]).max())
    dphi = np.abs(a["phi"] - b["phi"]).max()
    print(f"{name}: max|df|={df:.3e} max|dphi|={dphi:.3e}")
    assert df <= 2e-5
    assert dphi <= 2e-4
    # FP64 reductions of the FP32 state
    va, vb = gpu.saturation(), orc.saturation()
    np.testing.assert_allclose(va, vb, rtol=1e-5)
    gpu.close()
    orc.close()


def test_fp16_multiphase_rejected():
    c = mp_case(precision=2, strict=0)
    with pytest.raises(MflbmError):
        Solver(c["params"])
