"""The multiphase fluid-list layout on the CPU: the builder (mf-lbm_gb300/csrc/listlayout.cpp)
compiled for the host, and checks of every index it hands to the device (neighbour slots
and slot-map entries inside the arrays, one link slot per solid cell and array, every
boundary-plane cell resolved, a boundary-plane neighbour equal to the slot the boundary
conditions address, the porous-plate planes' private y ghosts and their exchange list),
for open and periodic z, periodic and walled y, and a porous plate."""
import ctypes as C

import numpy as np
import pytest

from cases import random_spheres
from mplist_lib import host_lib
from mflbm import geometry
from mflbm.solver import make_params

@pytest.fixture(scope="module")
def lib():
    L = host_lib()
    if L is None:
        pytest.skip("g++ or the CUDA headers not available")
    return L


@pytest.mark.parametrize("jper,kper,open_z,zpp", [(1, 1, 0, 0), (0, 0, 1, 0), (1, 0, 1, 0), (0, 1, 0, 7), (1, 0, 1, 9),
                                                      (1, 1, 0, 5)])
def test_multiphase_list_indices(lib, jper, kper, open_z, zpp):
    nx, ny, nz = 14, 12, 18
    p = make_params(multiphase=1, nx=nx, ny=ny, nz=nz, iper=0, jper=jper, kper=kper, wall_x_min=1, wall_x_max=1,
                    wall_y_min=0 if jper else 1, wall_y_max=0 if jper else 1, wall_z_min=0, wall_z_max=0,
                    inlet_bc=1 if open_z else 0, outlet_bc=1 if open_z else 0)
    wg = random_spheres((nz, ny, nx), 4, 1.5, 3.0, 5)
    walls, pore, _ = geometry.set_walls(p, wg)
    walls = np.ascontiguousarray(walls, dtype=np.int8)
    v = [C.c_int64() for _ in range(4)]
    bad = lib.mph_check(walls.ctypes.data, nx, ny, nz, jper, kper, open_z, zpp, *[C.byref(x) for x in v])
    print("nf, plane slots, links, stride:", [x.value for x in v])
    assert bad == 0
    assert v[0].value == pore
