"""Steady-state and breakthrough monitors (mflbm_steady_monitor) against numpy on the
state the library reports (compute_macro_vars fields and phi)."""
import numpy as np
import pytest

from cases import load_case, mp_case
from mflbm import Solver, output

pytestmark = pytest.mark.gpu
EPS = 1.110223025e-16


@pytest.mark.parametrize("precision", [0, 1])
def test_capillary_pressure_phase_field_and_breakthrough(precision, tmp_path):
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1, precision=precision, strict=0)
    sim = Solver(case["params"])
    load_case(sim, case)
    sim.steady_monitor(0)                    # phi_old <- phi
    phi0 = sim.macro()["phi"][4:-4, 4:-4, 4:-4].copy()
    sim.run(1, 6)
    m = sim.macro()
    fl = case["walls"][2:-2, 2:-2, 2:-2] == 0
    phi = m["phi"][4:-4, 4:-4, 4:-4]
    rho = m["rho"][1:-1, 1:-1, 1:-1]
    umax = np.sqrt(max((m["u"][1:-1, 1:-1, 1:-1] ** 2 + m["v"][1:-1, 1:-1, 1:-1] ** 2 +
                        m["w"][1:-1, 1:-1, 1:-1] ** 2)[fl].max(), 0.0))
    w_ = fl & (phi < -0.99)
    nw = fl & (phi > 0.99)
    pre_w = rho[w_].sum() / (w_.sum() + EPS)
    pre_nw = rho[nw].sum() / (nw.sum() + EPS)
    cp = sim.steady_monitor(1)
    np.testing.assert_allclose(cp[:4], [(pre_nw - pre_w) / 3.0, pre_w, pre_nw, umax], rtol=1e-12, atol=1e-15)
    assert cp[4] == w_.sum() and cp[5] == nw.sum()
    d = sim.steady_monitor(2)
    assert d[0] == np.abs(phi - phi0)[fl].max()
    d2 = sim.steady_monitor(2)               # phi_old was updated by the previous call
    assert d2[0] == 0.0
    nz = case["params"].nz
    cnt = sim.steady_monitor(3)[0]
    assert cnt == (fl[nz - 2] & (phi[nz - 2] > 0)).sum()
    mf = output.MonitorFiles(str(tmp_path), case["params"], fl.sum(axis=(1, 2)), ntime_monitor=0,
                             convergence_criteria=1e-30)
    assert output.write_capillary_pressure(mf, 6, cp) == output.RUNNING
    assert output.write_phase_field_change(mf, 6, d) == output.RUNNING
    assert (tmp_path / "out1.output" / "steady_monitor_capillary_pressure_error.dat").read_text().count("\n") == 1
    assert output.breakthrough(cnt) == (output.CONVERGED if cnt >= 1 else output.RUNNING)
    sim.close()


def test_steady_monitors_match_the_oracle():
    """The same monitors on the GPU (strict build) and on the oracle's restatement of
    Monitor.F90:287-507 after the same steps: maxima and counts exact, sums to rtol 1e-12."""
    from pyoracle import Oracle
    case = mp_case(per=(0, 0, 0), inlet=1, outlet=1, strict=1)
    sims = [Solver(case["params"]), Oracle(case["params"])]
    res = []
    for sim in sims:
        load_case(sim, case)
        sim.steady_monitor(0)
        sim.run(1, 8)
        r = {1: sim.steady_monitor(1), 2: sim.steady_monitor(2)}
        sim.run(9, 4)
        r["2b"] = sim.steady_monitor(2)
        r[3] = sim.steady_monitor(3)
        res.append(r)
        sim.close()
    g, o = res
    np.testing.assert_allclose(g[1][:3], o[1][:3], rtol=1e-12)
    assert g[1][3] == o[1][3] and g[1][4] == o[1][4] and g[1][5] == o[1][5]
    assert np.array_equal(g[2], o[2]) and np.array_equal(g["2b"], o["2b"])
    assert g[3][0] == o[3][0]
