"""The warp-compressed neighbour table of the fluid-list layout, on the CPU: the layout
builder (mf-lbm_gb300/csrc/listlayout.cpp) compiled for the host, and a decoder that
follows the odd-step kernel lane by lane (bases per warp and direction, one byte per node,
link slots from a ballot of the lanes with a link, 32-bit side entries for "wide"
warp-directions) must give back the 32-bit table entry for entry, on packings with
periodic wraps in every direction (the wrap in z makes wide warps) and with walls."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from mflbm import geometry
from mflbm.solver import make_params

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib():
    gxx = shutil.which("g++")
    inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if gxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers not available")
    build = os.path.join(HERE, "_build")
    os.makedirs(build, exist_ok=True)
    out = os.path.join(build, "liblistlayout_host.so")
    tmp = out + f".{os.getpid()}"
    subprocess.run([gxx, "-O2", "-shared", "-fPIC", "-std=c++17", f"-I{inc}", os.path.join(HERE, "listlayout_host.cpp"),
                    "-o", tmp], check=True)
    os.replace(tmp, out)
    L = C.CDLL(out)
    P64 = C.POINTER(C.c_int64)
    L.llh_check.restype = C.c_int64
    L.llh_check.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P64, P64, P64]
    return L


@pytest.mark.parametrize("n,por,per", [(48, 0.22, (1, 1, 1)), (40, 0.35, (0, 1, 1)), (33, 0.3, (0, 0, 1)),
                                       (64, 0.25, (1, 1, 1))])
def test_warp_table_decodes_to_the_32bit_table(lib, n, por, per):
    iper, jper, kper = per
    p = make_params(multiphase=0, nx=n, ny=n + 3, nz=n + 5, iper=iper, jper=jper, kper=kper,
                    wall_x_min=0 if iper else 1, wall_x_max=0 if iper else 1, wall_y_min=0 if jper else 1,
                    wall_y_max=0 if jper else 1, wall_z_min=0, wall_z_max=0, mrt=1)
    wg = geometry.sphere_packing((n + 5, n + 3, n), por, mean_r=5.0, sd_r=1.5, seed=n,
                                 periodic=(bool(kper), bool(jper), bool(iper)))
    walls, pore, _ = geometry.set_walls(p, wg)
    walls = np.ascontiguousarray(walls, dtype=np.int8)
    nf, nwide, nlink = C.c_int64(), C.c_int64(), C.c_int64()
    bad = lib.llh_check(walls.ctypes.data, p.nx, p.ny, p.nz, iper, jper, kper, C.byref(nf), C.byref(nwide),
                        C.byref(nlink))
    print(f"n={n} nf={nf.value} links={nlink.value} wide warp-directions={nwide.value}")
    assert bad == 0
    assert nf.value == pore and nlink.value > 0
    assert nwide.value < 18 * (nf.value // 32 + 1) // 4   # most warp-directions are compact
