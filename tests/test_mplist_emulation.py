"""The multiphase fluid-list layout's tables against the dense layout's update, on the CPU.

Both layouts are driven by the same AA sweep (odd: pull from x - e_q, push to x + e_q; even:
in place with swapped slots) with a stand-in collision (a nonlinear local map that mixes
the two species, so any mis-addressed population changes every later value).  The dense
side keeps the device's step order: sweep, the periodic exchange of the y and z faces and
x-aligned edges (pull after an even step, push after an odd one; the sets of directions
that cross each face, as k_wrap_faces / k_wrap_edges move them), then the porous plate
(both branches of Boundary_multiphase_other.F90:8-184, as k_porous_plate writes them).  The
list side runs the builder's neighbour table, link slots, slot map and the exchange of the
porous-plate planes' private ghosts.  The fluid nodes must agree exactly after 1-4 steps.

A planted mistake shows the test can fail: the same plate deck built without private ghosts
for the plate's planes (ghosts aliased to their images, which then see the plate's writes
that the dense ghosts miss) disagrees from the second step on.
"""
import ctypes as C

import numpy as np
import pytest

from cases import mp_case
from mplist_lib import host_lib

EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]
OPP = [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]
# directions that cross a face in the + and - sense, per axis (x, y, z)
PLUS = [[1, 7, 9, 11, 13], [3, 7, 8, 15, 17], [5, 11, 12, 15, 16]]
MINUS = [[2, 8, 10, 12, 14], [4, 10, 9, 16, 18], [6, 14, 13, 18, 17]]

CASES = {
    "periodic_yz": dict(per=(0, 1, 1)),
    "walled_open_z": dict(per=(0, 0, 0), inlet=1, outlet=1),
    "periodic_y_open_z_plate": dict(per=(0, 1, 0), inlet=1, outlet=1, plate=1, zplate=8),
    "periodic_yz_plate": dict(per=(0, 1, 1), plate=2, zplate=6),
    "walled_plate": dict(per=(0, 0, 0), inlet=1, outlet=1, plate=1, zplate=7),
    "ragged_periodic_yz": dict(nx=9, ny=7, nz=11, per=(0, 1, 1), spheres=1),
}


@pytest.fixture(scope="module")
def lib():
    L = host_lib()
    if L is None:
        pytest.skip("g++ or the CUDA headers not available")
    return L


def collide(ft):
    """Stand-in collision of one node: (2, 19) -> (2, 19), nonlinear, mixes the species."""
    s = ft.sum(axis=1, keepdims=True)
    return 0.8 * ft + 0.2 * ft[::-1, :] + 0.01 * (s * s) * (np.arange(19) + 1) / 19.0


def build(lib, case, private_ghosts=True):
    p = case["params"]
    nx, ny, nz = p.nx, p.ny, p.nz
    walls = np.ascontiguousarray(case["walls"], dtype=np.int8)
    planes = [0, 1, 2, nz - 1, nz, nz + 1] if not p.kper else []
    ghost = []
    if p.porous_plate_cmd:
        planes += [p.z_porous_plate - 1, p.z_porous_plate, p.z_porous_plate + 1]
        if private_ghosts:
            ghost = [p.z_porous_plate - 1, p.z_porous_plate, p.z_porous_plate + 1]
    pl = (C.c_int * max(1, len(planes)))(*planes)
    gp = (C.c_int * max(1, len(ghost)))(*ghost)
    info = (C.c_int64 * 7)()
    assert lib.mph_build(walls.ctypes.data, nx, ny, nz, p.jper, p.kper, pl, len(planes), gp, len(ghost), info) == 0
    nf, nplane, nlink, stride, spare, nmap, nwrap = list(info)
    mp = np.empty(nmap, np.int32)
    nb = np.empty(18 * nf, np.int32)
    link = np.empty(max(3, 3 * nlink), np.int32)
    cell1 = np.empty(nf, np.int32)
    wrap = np.empty(max(4, 4 * nwrap), np.int32)
    lib.mph_get(mp.ctypes.data, nb.ctypes.data, link.ctypes.data, cell1.ctypes.data, wrap.ctypes.data)
    return dict(nf=nf, stride=stride, spare=spare, map=mp, nb=nb.reshape(18, nf), link=link[:3 * nlink].reshape(-1, 3),
                cell1=cell1, wrap=wrap[:4 * nwrap].reshape(-1, 4))


def emulate(lib, case, steps=4, private_ghosts=True):
    """Returns, per step, the fluid nodes' populations of both layouts, (nf, 2, 19) each."""
    p = case["params"]
    nx, ny, nz, jper, kper = p.nx, p.ny, p.nz, p.jper, p.kper
    lay = build(lib, case, private_ghosts)
    nf, spare, mp, nb = lay["nf"], lay["spare"], lay["map"], lay["nb"]
    h1x, h1xy = nx + 2, (nx + 2) * (ny + 2)

    def slot(i, j, k):
        m = mp[i + h1x * j + h1xy * k]
        return m if m >= 0 else (-m - 2 if m <= -2 else spare)

    rng = np.random.default_rng(5)
    A = rng.random((2, 19, nz + 2, ny + 2, nx + 2))
    for ax, per in ((-2, jper), (-3, kper)):      # uploaded ghosts hold their periodic images
        if per:
            n = A.shape[ax] - 2
            lo, src_hi, hi, src_lo = ([slice(None)] * 5 for _ in range(4))
            lo[ax], src_hi[ax], hi[ax], src_lo[ax] = 0, n, n + 1, 1
            A[tuple(lo)] = A[tuple(src_hi)]
            A[tuple(hi)] = A[tuple(src_lo)]
    flat = A.reshape(2, 19, -1)
    B = np.zeros((2, 19, lay["stride"]))
    B[:, :, :nf] = flat[:, :, lay["cell1"]]
    for qa, sl, c in lay["link"]:
        B[:, qa, sl] = flat[:, qa, c]
    own = np.nonzero(mp >= nf)[0]
    B[:, :, mp[own]] = flat[:, :, own]
    nodes = [(c % h1x, (c // h1x) % (ny + 2), c // h1xy) for c in lay["cell1"]]

    def dense_sweep(odd):
        for (i, j, k) in nodes:
            ft = np.empty((2, 19))
            for q in range(19):
                ft[:, q] = A[:, q, k - EZ[q], j - EY[q], i - EX[q]] if odd else A[:, OPP[q], k, j, i]
            o = collide(ft)
            for q in range(19):
                if odd:
                    A[:, OPP[q], k + EZ[q], j + EY[q], i + EX[q]] = o[:, q]
                else:
                    A[:, q, k, j, i] = o[:, q]

    def list_sweep(odd):
        for x in range(nf):
            ft = np.empty((2, 19))
            for q in range(19):
                if odd:
                    ft[:, q] = B[:, 0, x] if q == 0 else B[:, q, nb[OPP[q] - 1, x]]
                else:
                    ft[:, q] = B[:, OPP[q], x]
            o = collide(ft)
            for q in range(19):
                if odd:
                    if q == 0:
                        B[:, 0, x] = o[:, 0]
                    else:
                        B[:, OPP[q], nb[q - 1, x]] = o[:, q]
                else:
                    B[:, q, x] = o[:, q]

    def dense_exchange(pull):
        per = (0, jper, kper)
        for d in (2, 1):
            if not per[d]:
                continue
            n = (nx, ny, nz)[d]
            n2 = ny if d == 2 else nz
            for b in range(1, n2 + 1):
                for a in range(1, nx + 1):
                    cell = (lambda L: (b, L, a)) if d == 1 else (lambda L: (L, b, a))
                    g0, inn, g1, in1 = cell(0), cell(n), cell(n + 1), cell(1)
                    for m in range(5):
                        qp, qm = PLUS[d][m], MINUS[d][m]
                        if pull:
                            A[(slice(None), qp) + g0] = A[(slice(None), qp) + inn]
                            A[(slice(None), qm) + g1] = A[(slice(None), qm) + in1]
                        else:
                            A[(slice(None), qm) + in1] = A[(slice(None), qm) + g1]
                            A[(slice(None), qp) + inn] = A[(slice(None), qp) + g0]
        if jper and kper:
            for i in range(1, nx + 1):
                pairs = [((18, ny + 1, nz + 1), (18, 1, 1)), ((16, ny + 1, 0), (16, 1, nz)),
                         ((17, 0, nz + 1), (17, ny, 1)), ((15, 0, 0), (15, ny, nz))]
                for (q, jg, kg), (_, ji, ki) in (pairs if pull else reversed(pairs)):
                    if pull:
                        A[:, q, kg, jg, i] = A[:, q, ki, ji, i]
                    else:
                        A[:, q, ki, ji, i] = A[:, q, kg, jg, i]

    def list_exchange(pull):
        for g0, inn, g1, in1 in lay["wrap"]:
            for m in range(5):
                qp, qm = PLUS[1][m], MINUS[1][m]
                if pull:
                    B[:, qp, g0] = B[:, qp, inn]
                    B[:, qm, g1] = B[:, qm, in1]
                else:
                    B[:, qm, in1] = B[:, qm, g1]
                    B[:, qp, inn] = B[:, qp, g0]

    def plate(before_odd, get, put):
        if not p.porous_plate_cmd:
            return
        z = p.z_porous_plate
        bs, cs = (0, 1) if p.porous_plate_cmd == 1 else (1, 0)
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                def b(q, ii, jj, kk):
                    return (bs, q, ii, jj, kk)

                def c(q, ii, jj, kk):
                    return (cs, q, ii, jj, kk)
                if before_odd:
                    ops = [(b(6, i, j, z), b(5, i, j, z - 1)), (b(13, i - 1, j, z), b(12, i, j, z - 1)),
                           (b(14, i + 1, j, z), b(11, i, j, z - 1)), (b(17, i, j - 1, z), b(16, i, j, z - 1)),
                           (b(18, i, j + 1, z), b(15, i, j, z - 1)), (b(5, i, j, z), b(6, i, j, z + 1)),
                           (b(12, i + 1, j, z), b(13, i, j, z + 1)), (b(11, i - 1, j, z), b(14, i, j, z + 1)),
                           (b(16, i, j + 1, z), b(17, i, j, z + 1)), (b(15, i, j - 1, z), b(18, i, j, z + 1))]
                    ops += [(c(q, i, j, z), c(q, i, j, z + 1)) for q in (6, 13, 14, 17, 18)]
                    ops += [(c(q, i, j, z), c(q, i, j, z - 1)) for q in (5, 12, 11, 16, 15)]
                else:
                    ops = [(b(5, i, j, z - 1), b(6, i, j, z)), (b(11, i, j, z - 1), b(14, i + 1, j, z)),
                           (b(12, i, j, z - 1), b(13, i - 1, j, z)), (b(15, i, j, z - 1), b(18, i, j + 1, z)),
                           (b(16, i, j, z - 1), b(17, i, j - 1, z)), (b(6, i, j, z + 1), b(5, i, j, z)),
                           (b(14, i, j, z + 1), b(11, i - 1, j, z)), (b(13, i, j, z + 1), b(12, i + 1, j, z)),
                           (b(18, i, j, z + 1), b(15, i, j - 1, z)), (b(17, i, j, z + 1), b(16, i, j + 1, z))]
                    ops += [(c(q, i, j, z - 1), c(q, i, j, z)) for q in (5, 11, 12, 15, 16)]
                    ops += [(c(q, i, j, z + 1), c(q, i, j, z)) for q in (6, 14, 13, 18, 17)]
                for dst, src in ops:
                    put(dst, get(src))

    def dget(t):
        return A[t[0], t[1], t[4], t[3], t[2]]

    def dput(t, v):
        A[t[0], t[1], t[4], t[3], t[2]] = v

    def lget(t):
        return B[t[0], t[1], slot(t[2], t[3], t[4])]

    def lput(t, v):
        B[t[0], t[1], slot(t[2], t[3], t[4])] = v

    out = []
    for n in range(1, steps + 1):
        even = n % 2 == 0
        dense_sweep(not even)
        dense_exchange(even)
        plate(even, dget, dput)
        list_sweep(not even)
        list_exchange(even)
        plate(even, lget, lput)
        d = np.array([A[:, :, k, j, i] for (i, j, k) in nodes])
        out.append((d, B[:, :, :nf].transpose(2, 0, 1).copy()))
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_list_tables_reproduce_the_dense_update(lib, name):
    case = mp_case(strict=1, **CASES[name])
    for n, (d, l) in enumerate(emulate(lib, case), start=1):
        assert np.array_equal(d, l), (name, n, int((d != l).sum()))


def test_plate_ghosts_aliased_to_their_images_disagree(lib):
    case = mp_case(strict=1, **CASES["periodic_y_open_z_plate"])
    res = emulate(lib, case, private_ghosts=False)
    assert np.array_equal(*res[0])
    assert not np.array_equal(*res[1])
