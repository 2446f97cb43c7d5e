"""GPU geometry preprocessing (mflbm_preprocess_geometry) against the host restatement:
identical solid- and fluid-boundary lists, bit for bit."""
import numpy as np
import pytest

from cases import random_spheres
from mflbm import geometry
from mflbm.solver import make_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,per,nsph,seed", [((14, 12, 16), (0, 1, 1), 3, 1), ((20, 18, 24), (0, 0, 1), 5, 2),
                                                 ((16, 16, 20), (0, 0, 0), 4, 3), ((13, 11, 10), (0, 1, 0), 2, 4)])
def test_gpu_lists_equal_host_lists(dims, per, nsph, seed):
    nx, ny, nz = dims
    _, jper, kper = per
    p = make_params(multiphase=1, nx=nx, ny=ny, nz=nz, iper=0, jper=jper, kper=kper, wall_x_min=1, wall_x_max=1,
                    wall_y_min=0 if jper else 1, wall_y_max=0 if jper else 1, wall_z_min=0, wall_z_max=0)
    wg = random_spheres((nz, ny, nx), nsph, 1.5, 3.5, seed)
    _, _, wchan = geometry.set_walls(p, wg)
    th = geometry.contact_angle_rad(45.0)
    s_cpu, f_cpu = geometry.preprocess(p, wchan, th)
    s_gpu, f_gpu = geometry.preprocess_gpu(p, wchan, th)
    assert s_cpu.size == s_gpu.size and f_cpu.size == f_gpu.size
    assert s_cpu.tobytes() == s_gpu.tobytes()
    assert f_cpu.tobytes() == f_gpu.tobytes()


def test_tube_drainage_lists():
    from mflbm import workloads
    case = workloads.tube_drainage()
    p = case["params"]
    _, _, wchan = geometry.set_walls(p, geometry.tube_with_sphere(nx=64, ny=64, nz=160, radius=30.0, buffer=8,
                                                                  sphere_r=14.0, sphere_z=80))
    s_gpu, f_gpu = geometry.preprocess_gpu(p, wchan, geometry.contact_angle_rad(45.0))
    assert s_gpu.tobytes() == case["solid"].tobytes()
    assert f_gpu.tobytes() == case["fluid"].tobytes()
