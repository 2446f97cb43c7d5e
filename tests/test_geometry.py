"""Host-side geometry setup against the oracle's restatement, and file formats."""
import numpy as np
import pytest

from cases import random_spheres
from mflbm import geometry
from mflbm.solver import make_params
import pyoracle


CASES = [
    dict(nx=12, ny=10, nz=14, iper=0, jper=0, kper=0, wall_y_min=1, wall_y_max=1),
    dict(nx=12, ny=10, nz=14, iper=0, jper=1, kper=1, wall_y_min=0, wall_y_max=0),
    dict(nx=9, ny=8, nz=7, iper=0, jper=1, kper=0, wall_y_min=0, wall_y_max=0),
    dict(nx=8, ny=9, nz=10, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0, wall_y_min=0, wall_y_max=0),
]


@pytest.mark.parametrize("kw", CASES)
def test_set_walls_matches_oracle(kw):
    p = make_params(**kw)
    wg = random_spheres((p.nz, p.ny, p.nx), 4, 1.0, 3.0, seed=11)
    a, pa, _ = geometry.set_walls(p, wg)
    b, pb = pyoracle.set_walls(p, wg)
    assert pa == pb
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("kw", CASES)
def test_boundary_lists_bit_identical_to_oracle(kw):
    p = make_params(multiphase=1, **kw)
    wg = random_spheres((p.nz, p.ny, p.nx), 4, 1.0, 3.0, seed=7)
    _, _, wchan = geometry.set_walls(p, wg)
    th = geometry.contact_angle_rad(30.0)
    s1, f1 = geometry.preprocess(p, wchan, th)
    s2, f2 = pyoracle.geometry_preprocess(p, wchan, th)
    assert s1.size == s2.size and f1.size == f2.size
    assert s1.tobytes() == s2.tobytes()
    assert f1.tobytes() == f2.tobytes()
    assert s1.size > 0 and f1.size > 0
    # every solid-boundary node has at least one fluid neighbour and a matching weight
    assert (s1["i_fluid_num"] >= 1).all()
    nrm = np.sqrt(f1["nwx"] ** 2 + f1["nwy"] ** 2 + f1["nwz"] ** 2)
    assert ((nrm > 0.999) | (nrm < 1e-6)).all()


def test_walls_file_round_trip(tmp_path):
    wg = random_spheres((7, 6, 5), 3, 1.0, 2.0, seed=2)
    path = tmp_path / "walls.dat"
    geometry.write_walls(path, wg)
    raw = path.read_bytes()
    assert raw[:12] == np.array([5, 6, 7], dtype="<i4").tobytes()
    assert len(raw) == 12 + wg.size
    np.testing.assert_array_equal(geometry.read_walls(path), wg)
    padded = geometry.read_walls(path, shape=(8, 8, 8))
    np.testing.assert_array_equal(padded[:7, :6, :5], wg)
    with pytest.raises(ValueError):
        geometry.read_walls(path, shape=(6, 6, 6))


def test_walls_file_truncated(tmp_path):
    path = tmp_path / "bad.dat"
    path.write_bytes(np.array([4, 4, 4], dtype="<i4").tobytes() + b"\0" * 10)
    with pytest.raises(ValueError):
        geometry.read_walls(path)


def test_boundary_info_round_trip(tmp_path):
    p = make_params(multiphase=1, nx=10, ny=10, nz=10)
    _, _, wchan = geometry.set_walls(p, random_spheres((10, 10, 10), 3, 1.0, 2.5, seed=4))
    th = geometry.contact_angle_rad(45.0)
    s, f = geometry.preprocess(p, wchan, th)
    path = tmp_path / "bnd.dat"
    geometry.write_boundary_info(path, s, f)
    assert path.stat().st_size == 8 + 96 * s.size + 40 * f.size
    s2, f2 = geometry.read_boundary_info(path, th)
    assert s2.tobytes() == s.tobytes() and f2.tobytes() == f.tobytes()
    path.write_bytes(path.read_bytes()[:-7])
    with pytest.raises(ValueError):
        geometry.read_boundary_info(path, th)


def test_sphere_packing_porosity_and_connectivity():
    from scipy import ndimage
    w = geometry.sphere_packing((32, 32, 32), 0.3, mean_r=4.0, sd_r=1.0, seed=3)
    por = float((w == 0).mean())
    assert 0.2 < por <= 0.3 + 1e-9
    lab, n = ndimage.label(w == 0, structure=ndimage.generate_binary_structure(3, 2))
    # one cluster after joining across periodic faces; unjoined labelling may split it
    sizes = np.bincount(lab.ravel())[1:]
    assert sizes.max() > 0.3 * (w == 0).sum()
    w2 = geometry.sphere_packing((32, 32, 32), 0.3, mean_r=4.0, sd_r=1.0, seed=3)
    np.testing.assert_array_equal(w, w2)


def test_tube_with_sphere_shape():
    w = geometry.tube_with_sphere()
    assert w.shape == (160, 64, 64)
    assert w[:8].sum() == 0 and w[-8:].sum() == 0
    assert w[79, 31, 31] == 1          # sphere centre (1-based 80, 32, 32)
    assert w[40, 31, 0] == 1           # (i-32)^2 = 31^2 > 30^2: outside the tube
    assert w[40, 31, 1] == 0           # (i-32)^2 = 30^2: on the tube radius, open


def test_contact_angle_transform():
    assert abs(geometry.contact_angle_rad(45.0) - 135.0 * np.pi / 180.0) < 1e-15
