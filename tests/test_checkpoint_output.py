"""Checkpoint byte layout and resume; monitor output records (CPU, oracle)."""
import os
import struct

import numpy as np

from mflbm import checkpoint, output
from cases import load_case, mp_case, sp_case
from pyoracle import Oracle


def _oracle(case):
    o = Oracle(case["params"])
    load_case(o, case)
    return o


def test_checkpoint_layout_and_resume_multiphase(tmp_path):
    case = mp_case(nx=10, ny=9, nz=14, per=(0, 0, 0), inlet=1, outlet=1)
    p = case["params"]
    a = _oracle(case)
    a.run(1, 6)
    path = checkpoint.save(a, str(tmp_path), ntime=6)
    assert os.path.basename(path) == "id0000"
    assert (tmp_path / "job_status.txt").read_text() == "continue_simulation\n"
    raw = open(path, "rb").read()
    assert len(raw) == checkpoint.expected_size(10, 9, 14, 1, 1)
    nt, fz, rin = struct.unpack("<idd", raw[:20])
    assert (nt, fz, rin) == (7, p.force_z, p.rho_in)
    st = a.download_state()
    # f0 follows the header, i fastest; phi follows the 38 PDF arrays
    n1 = 12 * 11 * 16
    assert np.frombuffer(raw[20:20 + 8 * n1], "<f8").tolist() == st["f"][0].ravel().tolist()
    off = 20 + 8 * 38 * n1
    assert np.frombuffer(raw[off:off + 8 * 18 * 17 * 22], "<f8").tolist() == st["phi"].ravel().tolist()
    # resume in a fresh context: 6 + 6 steps equal 12 steps in one go
    b = _oracle(case)
    ntime0, _, _ = checkpoint.load(b, str(tmp_path))
    assert ntime0 == 7
    b.run(ntime0, 6)
    a.run(7, 6)
    sa, sb = a.download_state(), b.download_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_checkpoint_singlephase_and_size_check(tmp_path):
    case = sp_case(nx=8, ny=7, nz=9, per=(0, 1, 1), spheres=1)
    o = _oracle(case)
    o.run(1, 4)
    path = checkpoint.save(o, str(tmp_path), ntime=4, secondary=True)
    assert "2rd_backup" in path
    assert not (tmp_path / "job_status.txt").exists()
    assert os.path.getsize(path) == 20 + 8 * 19 * 10 * 9 * 11
    nt, _, _, st = checkpoint.read_checkpoint(path, 8, 7, 9, 0, 0)
    assert nt == 5 and np.array_equal(st["f"], o.download_state()["f"])
    try:
        checkpoint.read_checkpoint(path, 8, 7, 10, 0, 0)
        raise AssertionError("size mismatch not detected")
    except ValueError:
        pass


def test_fortran_edit_descriptors():
    assert output.fortran_e(1.0) == " 0.1000000E+01"
    assert output.fortran_e(-0.00123456789) == "-0.1234568E-02"
    assert output.fortran_e(0.0) == " 0.0000000E+00"
    assert output.fortran_e(2.5e-7, 14, 6) == "  0.250000E-06"
    assert output.fortran_e(1e120) == " 0.1000000+121"
    assert output.fortran_i(1200) == "      1200"
    assert output.profile_name(1000) == "monitor  00001000.dat"


def test_monitor_files_multiphase(tmp_path):
    case = mp_case(nx=10, ny=9, nz=14, per=(0, 0, 0), inlet=1, outlet=1)
    p = case["params"]
    o = _oracle(case)
    o.run(1, 4)
    prof, scal, status = o.monitor()
    pore_z = (case["walls"][2:-2, 2:-2, 2:-2] == 0).sum(axis=(1, 2))
    mf = output.MonitorFiles(str(tmp_path), p, pore_z, n_exclude_inlet=2, n_exclude_outlet=2,
                             ntime_monitor_profile=4, steady_state_option=3)
    assert mf.write(4, prof, scal) == output.RUNNING
    d = tmp_path / "out1.output"
    sat = (d / "saturation.dat").read_text().splitlines()
    assert len(sat) == 1 and len(sat[0]) == 10 + 5 * 15
    v1, v2 = prof[2][2:12].sum(), prof[3][2:12].sum()
    assert float(sat[0].split()[1].replace("E", "e")) == float(output.fortran_e(v1 / (v1 + v2)).replace("E", "e"))
    assert len((d / "flowrate_time.dat").read_text().splitlines()[0]) == 10 + 6 * 15
    assert (d / "pre.dat").exists() and (d / "Ca_number.dat").exists()
    lines = (d / "profile" / "monitor  00000004.dat").read_text().splitlines()
    assert len(lines) == 14 and len(lines[0]) == 5 * 15


def test_monitor_files_singlephase_steady(tmp_path):
    case = sp_case(nx=8, ny=7, nz=9, per=(1, 1, 1), spheres=1)
    p = case["params"]
    o = _oracle(case)
    pore_z = np.full(p.nz, p.nx * p.ny)
    mf = output.MonitorFiles(str(tmp_path), p, pore_z, ntime_monitor=2, steady_state_option=1,
                             convergence_criteria=1e-30)
    ends = []
    for n in range(3):
        o.run(1 + 2 * n, 2)
        prof, scal, _ = o.monitor()
        ends.append(mf.write(2 * (n + 1), prof, scal))
    assert ends == [0, 0, 0]
    rows = (tmp_path / "out1.output" / "flowrate_time.dat").read_text().splitlines()
    assert len(rows) == 3 and len(rows[0]) == 10 + 2 * 15
    assert not (tmp_path / "out1.output" / "pre.dat").exists()   # periodic z
    assert len((tmp_path / "out1.output" / "steady_monitor_flowrate_error.dat").read_text().splitlines()) == 3
