"""The oracle's restatement of the steady-state and breakthrough monitors
(multiphase_3D/0.src/Monitor.F90:287-507) against numpy applied to the oracle's own
macroscopic fields: capillary pressure from the mean density of the two bulk phases,
the largest phase-field change since the last snapshot, and the breakthrough count."""
import numpy as np

from cases import load_case, mp_case
from pyoracle import Oracle

EPS = 1.110223025e-16


def test_oracle_steady_monitors_against_numpy():
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1)
    o = Oracle(case["params"])
    load_case(o, case)
    o.steady_monitor(0)
    phi0 = o.macro()["phi"][4:-4, 4:-4, 4:-4].copy()
    o.run(1, 6)
    m = o.macro()
    fl = case["walls"][2:-2, 2:-2, 2:-2] == 0
    phi = m["phi"][4:-4, 4:-4, 4:-4]
    rho = m["rho"][1:-1, 1:-1, 1:-1]
    uu = m["u"][1:-1, 1:-1, 1:-1] ** 2 + m["v"][1:-1, 1:-1, 1:-1] ** 2 + m["w"][1:-1, 1:-1, 1:-1] ** 2
    w_, nw = fl & (phi < -0.99), fl & (phi > 0.99)
    pre_w = rho[w_].sum() / (w_.sum() + EPS)
    pre_nw = rho[nw].sum() / (nw.sum() + EPS)
    cp = o.steady_monitor(1)
    np.testing.assert_allclose(cp, [(pre_nw - pre_w) / 3.0, pre_w, pre_nw, np.sqrt(uu[fl].max()), w_.sum(), nw.sum()],
                               rtol=1e-12, atol=1e-15)
    d = o.steady_monitor(2)
    assert d[0] == np.abs(phi - phi0)[fl].max()
    assert o.steady_monitor(2)[0] == 0.0
    nz = case["params"].nz
    assert o.steady_monitor(3)[0] == (fl[nz - 2] & (phi[nz - 2] > 0)).sum()
    o.close()
