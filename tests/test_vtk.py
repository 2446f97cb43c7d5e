"""Legacy VTK writers (multiphase_3D/0.src/IO_multiphase.F90:824-1149): byte layout of
the header and the big-endian scalar blocks, and values from a state (oracle on the CPU;
the GPU against the oracle in the -m gpu test)."""
import numpy as np
import pytest

from cases import load_case, mp_case
from mflbm import vtk
from pyoracle import Oracle


def _expected_header(nx, ny, nz):
    return ("# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS \n"
            f"DIMENSIONS {nx:>10} {ny:>10} {nz:>10}\n"
            "ORIGIN          1          1          1\nSPACING          1          1          1\n"
            f"POINT_DATA {nx * ny * nz:>14}\n").encode()


def _blocks(raw, names, dtype, n):
    out, pos = {}, 0
    for name in names:
        head = f"SCALARS {name} {'float' if dtype == '>f4' else 'double'}\nLOOKUP_TABLE default\n".encode()
        assert raw[pos:pos + len(head)] == head, name
        pos += len(head)
        size = np.dtype(dtype).itemsize * n
        out[name] = np.frombuffer(raw[pos:pos + size], dtype=dtype)
        pos += size
    assert pos == len(raw)
    return out


@pytest.mark.parametrize("precision_cmd,dtype", [(0, ">f4"), (1, ">f8")])
def test_full_flow_field_file(tmp_path, precision_cmd, dtype):
    case = mp_case(nx=9, ny=7, nz=11, per=(0, 0, 0), inlet=1, outlet=1)
    o = Oracle(case["params"])
    load_case(o, case)
    o.run(1, 4)
    path = vtk.save_field(o, str(tmp_path), 4, 1, precision_cmd=precision_cmd)
    assert path.endswith("out3.field_data/full_flow_field/full_flow_field_0000000004.vtk")
    raw = open(path, "rb").read()
    h = _expected_header(9, 7, 11)
    assert raw[:len(h)] == h
    blk = _blocks(raw[len(h):], ["phi", "density", "velocity_X", "velocity_Y", "velocity_Z"], dtype, 9 * 7 * 11)
    m = o.macro()
    for name, ref in (("phi", m["phi"][4:-4, 4:-4, 4:-4]), ("density", m["rho"][1:-1, 1:-1, 1:-1]),
                      ("velocity_Z", m["w"][1:-1, 1:-1, 1:-1])):
        assert np.array_equal(blk[name], ref.astype(dtype).ravel()), name
    o.close()


def test_phase_and_force_vector_files(tmp_path):
    case = mp_case(nx=8, ny=6, nz=10, per=(0, 0, 0), inlet=1, outlet=1)
    o = Oracle(case["params"])
    load_case(o, case)
    o.run(1, 2)
    p2 = vtk.save_field(o, str(tmp_path), 2, 2)
    raw = open(p2, "rb").read()
    h = _expected_header(8, 6, 10)
    blk = _blocks(raw[len(h):], ["phi"], ">f4", 480)
    phi = o.download_state()["phi"][4:-4, 4:-4, 4:-4]
    assert np.all(phi[case["walls"][2:-2, 2:-2, 2:-2] == 1] == 0.0)      # zeroed by the writer, as the reference
    assert np.array_equal(blk["phi"], phi.astype(">f4").ravel())
    p3 = vtk.save_field(o, str(tmp_path), 2, 3, precision_cmd=1)
    assert p3.endswith("full_flow_field/force_vector_0000000002.vtk")
    blk = _blocks(open(p3, "rb").read()[len(h):], ["phi", "density", "velocity_X", "velocity_Y", "velocity_Z"],
                  ">f8", 480)
    g = o.get_gradient()
    assert np.array_equal(blk["density"], g["c_norm"][2:-2, 2:-2, 2:-2].ravel())
    assert np.array_equal(blk["velocity_X"], g["cn_x"][2:-2, 2:-2, 2:-2].ravel())
    o.close()


def test_walls_and_2d_micromodel_files(tmp_path):
    rng = np.random.default_rng(3)
    wg = (rng.uniform(size=(5, 4, 6)) < 0.3).astype(np.int8)
    raw = open(vtk.write_walls(str(tmp_path), wg), "rb").read()
    h = _expected_header(6, 4, 5)
    assert raw[:len(h)] == h
    rest = raw[len(h):]
    head = b"SCALARS walls int\nLOOKUP_TABLE default\n"
    assert rest[:len(head)] == head
    assert np.array_equal(np.frombuffer(rest[len(head):], ">i4"), wg.ravel().astype(np.int32))
    phi = rng.uniform(-1, 1, size=(5, 7, 6))
    raw = open(vtk.write_phi_2d_micromodel(str(tmp_path), 12, phi), "rb").read()
    h2 = ("# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS \n"
          "DIMENSIONS          6          1          5\nORIGIN          1          1          1\n"
          "SPACING          1          0          1\nPOINT_DATA         30\n"
          "SCALARS phi float\nLOOKUP_TABLE default\n").encode()
    assert raw[:len(h2)] == h2
    want = (0.5 * (1.0 + phi[:, 1:-1, :].sum(axis=1) / 5)).astype(">f4").ravel()
    np.testing.assert_allclose(np.frombuffer(raw[len(h2):], ">f4"), want, rtol=1e-6)


@pytest.mark.gpu
def test_gpu_files_equal_oracle_files(tmp_path):
    """Strict build: the library's state gives byte-identical files to the oracle's."""
    from mflbm import Solver
    case = mp_case(nx=10, ny=8, nz=12, per=(0, 0, 0), inlet=1, outlet=1, strict=1)
    out = []
    for cls, sub in ((Solver, "gpu"), (Oracle, "orc")):
        sim = cls(case["params"])
        load_case(sim, case)
        sim.run(1, 6)
        root = str(tmp_path / sub)
        files = [vtk.save_field(sim, root, 6, t, precision_cmd=pc) for t, pc in ((1, 1), (3, 1), (2, 0))]
        files.append(vtk.save_phi_2d_micromodel(sim, root, 6))
        out.append([open(f, "rb").read() for f in files])
        sim.close()
    for a, b in zip(*out):
        assert a == b
