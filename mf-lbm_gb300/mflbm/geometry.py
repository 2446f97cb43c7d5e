"""Host-side geometry: wall arrays, boundary-node lists, inlet profile, synthetic media.

This mirrors the setup work that MF-LBM's Fortran host does before the time loop
(set_walls, geometry_preprocessing_new, inlet_vel_profile_rectangular) for one rank,
plus seeded generators for the synthetic porous media used in place of the missing
sample-rock files.  Arrays use the reference's column-major layout through numpy
C-order arrays indexed [k, j, i] (i fastest), with the reference's halos:
walls halo 2 -> shape (nz+4, ny+4, nx+4), index [k+1, j+1, i+1].

Every floating-point accumulation below keeps the reference's term order, so the
results are bit-identical to a sequential FP64 evaluation of the Fortran.
"""
import math
import struct

import numpy as np

from ._capi import FLUID_DTYPE, SOLID_DTYPE

EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W_EQU = np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12)


# ------------------------------------------------------------------------------------
# set_walls (multiphase_3D/0.src/Misc.F90:6-210) for one rank
# ------------------------------------------------------------------------------------
def apply_channel_walls(p, walls_global):
    """Channel walls on the global array (Misc.F90:90-109).  walls_global: (nz, ny, nx)."""
    g = np.array(walls_global, dtype=np.int8, copy=True)
    if p.wall_z_min == 1:
        g[0, :, :] = 1
    if p.wall_z_max == 1:
        g[-1, :, :] = 1
    if p.wall_x_min == 1:
        g[:, :, 0] = 1
    if p.wall_x_max == 1:
        g[:, :, -1] = 1
    if p.wall_y_min == 1:
        g[:, 0, :] = 1
    if p.wall_y_max == 1:
        g[:, -1, :] = 1
    return g


def set_walls(p, walls_global):
    """Return (walls with halo 2, pore_sum, walls after channel walls).

    Follows Misc.F90:24-207: local copy, channel walls over the halo, then the
    z, y, x halo transports (Mpi_misc.F90:337-502), which are periodic copies when the
    direction is periodic and no-ops otherwise on a single rank.
    """
    nx, ny, nz = p.nx, p.ny, p.nz
    g = apply_channel_walls(p, walls_global)
    w = np.zeros((nz + 4, ny + 4, nx + 4), dtype=np.int8)
    w[2:nz + 2, 2:ny + 2, 2:nx + 2] = g
    # local channel walls incl. the halo: index k maps to array row k+1
    if p.wall_z_min == 1:
        w[:3, :, :] = 1                     # k <= 1
    if p.wall_z_max == 1:
        w[nz + 1:, :, :] = 1                # k >= nz
    if p.wall_x_min == 1:
        w[:, :, :3] = 1
    if p.wall_x_max == 1:
        w[:, :, nx + 1:] = 1
    if p.wall_y_min == 1:
        w[:, :3, :] = 1
    if p.wall_y_max == 1:
        w[:, ny + 1:, :] = 1
    if p.kper == 1:   # i, j interior only
        w[0:2, 2:ny + 2, 2:nx + 2] = w[nz:nz + 2, 2:ny + 2, 2:nx + 2]
        w[nz + 2:nz + 4, 2:ny + 2, 2:nx + 2] = w[2:4, 2:ny + 2, 2:nx + 2]
    if p.jper == 1:   # i interior, all k
        w[:, 0:2, 2:nx + 2] = w[:, ny:ny + 2, 2:nx + 2]
        w[:, ny + 2:ny + 4, 2:nx + 2] = w[:, 2:4, 2:nx + 2]
    if p.iper == 1:
        w[:, :, 0:2] = w[:, :, nx:nx + 2]
        w[:, :, nx + 2:nx + 4] = w[:, :, 2:4]
    pore_sum = int(np.count_nonzero(w[2:nz + 2, 2:ny + 2, 2:nx + 2] <= 0))
    return w, pore_sum, g


# ------------------------------------------------------------------------------------
# geometry_preprocessing_new (multiphase_3D/0.src/Geometry_preprocessing.F90:9-512)
# ------------------------------------------------------------------------------------
ISO8 = (4.0 / 45.0, 1.0 / 21.0, 2.0 / 105.0, 5.0 / 504.0, 1.0 / 315.0, 1.0 / 630.0, 1.0 / 5040.0)

# ISO8 gradient terms (+, -) of each group, in the order the Fortran writes them
_NWX = [
    [((1, 0, 0), (-1, 0, 0))],
    [((1, 1, 0), (-1, -1, 0)), ((1, -1, 0), (-1, 1, 0)), ((1, 0, 1), (-1, 0, -1)), ((1, 0, -1), (-1, 0, 1))],
    [((1, 1, 1), (-1, -1, -1)), ((1, 1, -1), (-1, -1, 1)), ((1, -1, 1), (-1, 1, -1)), ((1, -1, -1), (-1, 1, 1))],
    [((2, 0, 0), (-2, 0, 0))],
    [((2, 1, 0), (-2, -1, 0)), ((2, -1, 0), (-2, 1, 0)), ((2, 0, 1), (-2, 0, -1)), ((2, 0, -1), (-2, 0, 1)),
     ((1, 2, 0), (-1, -2, 0)), ((1, -2, 0), (-1, 2, 0)), ((1, 0, 2), (-1, 0, -2)), ((1, 0, -2), (-1, 0, 2))],
    [((2, 1, 1), (-2, -1, -1)), ((2, 1, -1), (-2, -1, 1)), ((2, -1, 1), (-2, 1, -1)), ((2, -1, -1), (-2, 1, 1)),
     ((1, 2, 1), (-1, -2, -1)), ((1, 2, -1), (-1, -2, 1)), ((1, -2, 1), (-1, 2, -1)), ((1, -2, -1), (-1, 2, 1)),
     ((1, 1, 2), (-1, -1, -2)), ((1, 1, -2), (-1, -1, 2)), ((1, -1, 2), (-1, 1, -2)), ((1, -1, -2), (-1, 1, 2))],
    [((2, 2, 0), (-2, -2, 0)), ((2, -2, 0), (-2, 2, 0)), ((2, 0, 2), (-2, 0, -2)), ((2, 0, -2), (-2, 0, 2))],
]
_NWY = [
    [((0, 1, 0), (0, -1, 0))],
    [((1, 1, 0), (-1, -1, 0)), ((-1, 1, 0), (1, -1, 0)), ((0, 1, 1), (0, -1, -1)), ((0, 1, -1), (0, -1, 1))],
    [((1, 1, 1), (-1, -1, -1)), ((1, 1, -1), (-1, -1, 1)), ((-1, 1, -1), (1, -1, 1)), ((-1, 1, 1), (1, -1, -1))],
    [((0, 2, 0), (0, -2, 0))],
    [((2, 1, 0), (-2, -1, 0)), ((-2, 1, 0), (2, -1, 0)), ((0, 2, 1), (0, -2, -1)), ((0, 2, -1), (0, -2, 1)),
     ((1, 2, 0), (-1, -2, 0)), ((-1, 2, 0), (1, -2, 0)), ((0, 1, 2), (0, -1, -2)), ((0, 1, -2), (0, -1, 2))],
    [((2, 1, 1), (-2, -1, -1)), ((2, 1, -1), (-2, -1, 1)), ((-2, 1, 1), (2, -1, -1)), ((-2, 1, -1), (2, -1, 1)),
     ((1, 2, 1), (-1, -2, -1)), ((1, 2, -1), (-1, -2, 1)), ((-1, 2, 1), (1, -2, -1)), ((-1, 2, -1), (1, -2, 1)),
     ((1, 1, 2), (-1, -1, -2)), ((1, 1, -2), (-1, -1, 2)), ((-1, 1, 2), (1, -1, -2)), ((-1, 1, -2), (1, -1, 2))],
    [((2, 2, 0), (-2, -2, 0)), ((-2, 2, 0), (2, -2, 0)), ((0, 2, 2), (0, -2, -2)), ((0, 2, -2), (0, -2, 2))],
]
_NWZ = [
    [((0, 0, 1), (0, 0, -1))],
    [((0, 1, 1), (0, -1, -1)), ((0, -1, 1), (0, 1, -1)), ((1, 0, 1), (-1, 0, -1)), ((-1, 0, 1), (1, 0, -1))],
    [((1, 1, 1), (-1, -1, -1)), ((1, -1, 1), (-1, 1, -1)), ((-1, 1, 1), (1, -1, -1)), ((-1, -1, 1), (1, 1, -1))],
    [((0, 0, 2), (0, 0, -2))],
    [((0, 1, 2), (0, -1, -2)), ((0, -1, 2), (0, 1, -2)), ((2, 0, 1), (-2, 0, -1)), ((-2, 0, 1), (2, 0, -1)),
     ((0, 2, 1), (0, -2, -1)), ((0, -2, 1), (0, 2, -1)), ((1, 0, 2), (-1, 0, -2)), ((-1, 0, 2), (1, 0, -2))],
    [((2, 1, 1), (-2, -1, -1)), ((2, -1, 1), (-2, 1, -1)), ((-2, 1, 1), (2, -1, -1)), ((-2, -1, 1), (2, 1, -1)),
     ((1, 2, 1), (-1, -2, -1)), ((1, -2, 1), (-1, 2, -1)), ((-1, 2, 1), (1, -2, -1)), ((-1, -2, 1), (1, 2, -1)),
     ((1, 1, 2), (-1, -1, -2)), ((1, -1, 2), (-1, 1, -2)), ((-1, 1, 2), (1, -1, -2)), ((-1, -1, 2), (1, 1, -2))],
    [((0, 2, 2), (0, -2, -2)), ((0, -2, 2), (0, 2, -2)), ((2, 0, 2), (-2, 0, -2)), ((-2, 0, 2), (2, 0, -2))],
]


def _iso8(s2, ki, ji, ii, groups):
    total = None
    for coef, terms in zip(ISO8, groups):
        acc = None
        for plus, minus in terms:
            a = s2[ki + plus[2], ji + plus[1], ii + plus[0]]
            b = s2[ki + minus[2], ji + minus[1], ii + minus[0]]
            acc = a - b if acc is None else (acc + a) - b
        term = coef * acc
        total = term if total is None else total + term
    return total


def preprocess(p, walls_channel, theta_rad):
    """Boundary-node lists of geometry_preprocessing_new for one rank.

    walls_channel: global wall array after channel walls, shape (nz, ny, nx).
    Returns (solid, fluid) numpy structured arrays with the byte layout of
    mflbm_solid_bnd / mflbm_fluid_bnd, in the reference's k, j, i order.
    """
    nx, ny, nz = p.nx, p.ny, p.nz
    gl = 6 + 4
    wt = np.zeros((nz + 2 * gl, ny + 2 * gl, nx + 2 * gl), dtype=np.int8)
    # array index of lattice coordinate c is c - 1 + gl
    wt[gl:gl + nz, gl:gl + ny, gl:gl + nx] = walls_channel
    I = slice(gl, gl + nx)
    J = slice(gl, gl + ny)
    if p.kper == 0:
        wt[:gl, J, I] = wt[gl, J, I]
        wt[gl + nz:, J, I] = wt[gl + nz - 1, J, I]
    else:
        wt[:gl, J, I] = wt[nz:nz + gl, J, I]
        wt[gl + nz:, J, I] = wt[gl:2 * gl, J, I]
    if p.jper == 0:
        wt[:, :gl, I] = wt[:, gl:gl + 1, I]
        wt[:, gl + ny:, I] = wt[:, gl + ny - 1:gl + ny, I]
    else:
        wt[:, :gl, I] = wt[:, ny:ny + gl, I]
        wt[:, gl + ny:, I] = wt[:, gl:2 * gl, I]
    if p.iper == 0:
        wt[:, :, :gl] = wt[:, :, gl:gl + 1]
        wt[:, :, gl + nx:] = wt[:, :, gl + nx - 1:gl + nx]
    else:
        wt[:, :, :gl] = wt[:, :, nx:nx + gl]
        wt[:, :, gl + nx:] = wt[:, :, gl:2 * gl]

    s1 = wt.astype(np.float64)
    # classification over the inner region (Geometry_preprocessing.F90:121-143)
    inner = (slice(1, -1),) * 3
    sh = wt.shape
    nb_min = None
    nb_max = None
    for n in range(1, 19):
        v = wt[1 + EZ[n]:sh[0] - 1 + EZ[n], 1 + EY[n]:sh[1] - 1 + EY[n], 1 + EX[n]:sh[2] - 1 + EX[n]]
        nb_min = v.copy() if nb_min is None else np.minimum(nb_min, v)
        nb_max = v.copy() if nb_max is None else np.maximum(nb_max, v)
    cls = wt.copy()
    core = wt[inner]
    c = cls[inner]
    c[(core == 1) & (nb_min <= 0)] = 2
    c[(core == 0) & (nb_max >= 1)] = -1

    # 4 iterations of 27-point smoothing (:145-169), accumulation in n = 0..26 order
    iex = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1]
    iey = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1]
    iez = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1]
    we = (8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0)
    s2 = s1.copy()
    for _ in range(4):
        acc = np.zeros(tuple(d - 2 for d in sh))
        for n in range(27):
            m = iex[n] ** 2 + iey[n] ** 2 + iez[n] ** 2
            v = s1[1 + iez[n]:sh[0] - 1 + iez[n], 1 + iey[n]:sh[1] - 1 + iey[n], 1 + iex[n]:sh[2] - 1 + iex[n]]
            acc = acc + v * we[m]
        s2[inner] = acc
        s1[inner] = acc
    # lists (:171-225 global over [1-4, n+4], local filters :429-507)
    o = gl - 1  # array index of lattice coordinate c is c + o
    sub = cls[o - 3:o + nz + 5, o - 3:o + ny + 5, o - 3:o + nx + 5]
    ks, js, is_ = np.nonzero(sub == 2)
    kk, jj, ii = ks - 3, js - 3, is_ - 3
    keep = (ii >= -2) & (ii <= nx + 3) & (jj >= -2) & (jj <= ny + 3) & (kk >= -2) & (kk <= nz + 3)
    kk, jj, ii = kk[keep], jj[keep], ii[keep]
    solid = np.zeros(kk.size, dtype=SOLID_DTYPE)
    solid["ix"], solid["iy"], solid["iz"] = ii, jj, kk
    lw = np.zeros(kk.size)
    cnt = np.zeros(kk.size, dtype=np.int32)
    nbl = np.zeros((kk.size, 18), dtype=np.int32)
    rows = np.arange(kk.size)
    for n in range(1, 19):
        fl = cls[kk + o + EZ[n], jj + o + EY[n], ii + o + EX[n]] <= 0
        lw = np.where(fl, lw + W_EQU[n], lw)
        nbl[rows[fl], cnt[fl]] = n
        cnt = cnt + fl
    solid["la_weight"] = lw
    solid["i_fluid_num"] = cnt
    solid["neighbor_list"] = nbl

    ks, js, is_ = np.nonzero(sub == -1)
    kk, jj, ii = ks - 3, js - 3, is_ - 3
    keep = (ii >= -1) & (ii <= nx + 2) & (jj >= -1) & (jj <= ny + 2) & (kk >= -1) & (kk <= nz + 2)
    kk, jj, ii = kk[keep], jj[keep], ii[keep]
    fluid = np.zeros(kk.size, dtype=FLUID_DTYPE)
    fluid["ix"], fluid["iy"], fluid["iz"] = ii, jj, kk
    if kk.size:
        ka, ja, ia = kk + o, jj + o, ii + o
        nwx = _iso8(s2, ka, ja, ia, _NWX)
        nwy = _iso8(s2, ka, ja, ia, _NWY)
        nwz = _iso8(s2, ka, ja, ia, _NWZ)
        tmp = 1.0 / (np.sqrt(nwx * nwx + nwy * nwy + nwz * nwz) + 1e-14)
        fluid["nwx"], fluid["nwy"], fluid["nwz"] = nwx * tmp, nwy * tmp, nwz * tmp
    fluid["theta"] = theta_rad
    return solid, fluid


def preprocess_gpu(p, walls_channel, theta_rad, lib=None):
    """preprocess() on the GPU through mflbm_preprocess_geometry: the same lists, bit for
    bit, in a fraction of the time for large grids (periodic dimensions >= 10)."""
    import ctypes as C
    from . import _capi
    lib = lib or _capi.load()
    w = np.ascontiguousarray(walls_channel, dtype=np.int8)
    assert w.shape == (p.nz, p.ny, p.nx)
    ns, nf = C.c_int32(), C.c_int32()
    rc = lib.mflbm_preprocess_geometry(C.byref(p), w.ctypes.data, float(theta_rad), None, 0, C.byref(ns), None, 0,
                                       C.byref(nf))
    if rc and rc != _capi.MFLBM_ERANGE:
        raise _capi.MflbmError(rc, lib.mflbm_preprocess_last_error().decode())
    solid = np.zeros(ns.value, dtype=SOLID_DTYPE)
    fluid = np.zeros(nf.value, dtype=FLUID_DTYPE)
    rc = lib.mflbm_preprocess_geometry(C.byref(p), w.ctypes.data, float(theta_rad), solid.ctypes.data, solid.size,
                                       C.byref(ns), fluid.ctypes.data, fluid.size, C.byref(nf))
    if rc:
        raise _capi.MflbmError(rc, lib.mflbm_preprocess_last_error().decode())
    return solid, fluid


def contact_angle_rad(theta_deg):
    """theta transform of read_parameter_multi (IO_multiphase.F90:467-468)."""
    theta = 180.0 - theta_deg
    return theta * 3.14159265358979323846 / 180.0


# ------------------------------------------------------------------------------------
# inlet_vel_profile_rectangular (multiphase_3D/0.src/Misc.F90:625-665)
# ------------------------------------------------------------------------------------
def _ipow32(n, e):
    """Fortran default-integer n**e: 32-bit two's complement wrap (n**5 wraps for n >= 75)."""
    r = 1
    for _ in range(e):
        r = (r * n) & 0xFFFFFFFF
    return r - (1 << 32) if r >= (1 << 31) else r


def inlet_profile(nx, ny, vel_avg, num_terms=1000):
    """Analytic duct profile w_in with shape (ny+2, nx+2), halo 1 (i, j in 0..n+1)."""
    pi = 3.14159265358979323846
    la_x = float(nx) - 2.0
    la_y = float(ny) - 2.0
    a, b = 0.5 * la_x, 0.5 * la_y
    tmp1 = 0.0
    for n in range(1, num_terms + 1, 2):
        tmp1 = tmp1 + math.tanh(0.5 * float(n) * pi * b / a) / float(_ipow32(n, 5))
    pi2 = pi * pi
    pi5 = (pi2 * pi2) * pi
    tmp2 = 1.0 - 192.0 / pi5 * (a / b) * tmp1
    tmp2 = -3.0 * vel_avg / (tmp2 * (a * a))
    w = np.zeros((ny + 2, nx + 2))
    i = np.arange(2, nx).astype(np.float64)   # x in 2..nx-1
    j = np.arange(2, ny).astype(np.float64)
    xx = (i - 1.5 - a)[None, :]
    yy = (j - 1.5 - b)[:, None]
    tmp3 = np.zeros((ny - 2, nx - 2))
    for n in range(1, num_terms + 1, 2):
        sgn = math.pow(-1.0, 0.5 * float(n - 1))
        cosx = np.cos(0.5 * n * pi * xx / a)
        ey = (np.exp(0.5 * n * pi * (yy - b) / a) + np.exp(0.5 * n * pi * (-yy - b) / a)) / (1.0 + math.exp(0.5 * n * pi * (-b - b) / a))
        tmp3 = tmp3 + sgn * cosx / float(_ipow32(n, 3)) * (1.0 - ey)
    w[2:ny, 2:nx] = tmp3 * (-16.0 * tmp2 * (a * a) * (1.0 / (pi * pi * pi)))
    return w


# ------------------------------------------------------------------------------------
# wall-array and boundary-info file formats
# ------------------------------------------------------------------------------------
def write_walls(path, walls_global):
    """Stream file: int32 nx, ny, nz then int8 walls in Fortran order (Misc.F90:264-271)."""
    nz, ny, nx = walls_global.shape
    with open(path, "wb") as fh:
        fh.write(struct.pack("<3i", nx, ny, nz))
        fh.write(np.ascontiguousarray(walls_global, dtype=np.int8).tobytes())


def read_walls(path, shape=None):
    """Read a wall file; shape=(nz, ny, nx) pads a smaller sample with fluid (value 0)."""
    with open(path, "rb") as fh:
        hdr = fh.read(12)
        if len(hdr) != 12:
            raise ValueError("truncated wall file header")
        nx, ny, nz = struct.unpack("<3i", hdr)
        if min(nx, ny, nz) <= 0:
            raise ValueError("invalid wall file dimensions")
        data = np.frombuffer(fh.read(), dtype=np.int8)
    if data.size != nx * ny * nz:
        raise ValueError(f"wall file holds {data.size} bytes, expected {nx * ny * nz}")
    sample = data.reshape(nz, ny, nx)
    if shape is None:
        return sample.copy()
    out = np.zeros(shape, dtype=np.int8)
    if nz > shape[0] or ny > shape[1] or nx > shape[2]:
        raise ValueError("Domain size is smaller than porous media sample size")
    out[:nz, :ny, :nx] = sample
    return out


_FLUID_FILE_DTYPE = [("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4"), ("_pad", "<i4"),
                     ("nwx", "<f8"), ("nwy", "<f8"), ("nwz", "<f8")]


def write_boundary_info(path, solid, fluid):
    """Boundary-info file: int32 nsolid, nfluid, then 96-byte solid records and
    40-byte fluid records (3d_wall_boundary_process.f90:624-645)."""
    with open(path, "wb") as fh:
        fh.write(struct.pack("<2i", solid.size, fluid.size))
        fh.write(solid.tobytes())
        rec = np.zeros(fluid.size, dtype=_FLUID_FILE_DTYPE)
        for name in ("ix", "iy", "iz", "nwx", "nwy", "nwz"):
            rec[name] = fluid[name]
        fh.write(rec.tobytes())


def read_boundary_info(path, theta_rad):
    with open(path, "rb") as fh:
        hdr = fh.read(8)
        if len(hdr) != 8:
            raise ValueError("truncated boundary-info header")
        ns, nf = struct.unpack("<2i", hdr)
        if ns < 0 or nf < 0:
            raise ValueError("negative boundary-node counts")
        sb = fh.read(96 * ns)
        fb = fh.read(40 * nf)
    if len(sb) != 96 * ns or len(fb) != 40 * nf:
        raise ValueError("truncated boundary-info file")
    solid = np.frombuffer(sb, dtype=SOLID_DTYPE).copy()
    rec = np.frombuffer(fb, dtype=_FLUID_FILE_DTYPE)
    fluid = np.zeros(nf, dtype=FLUID_DTYPE)
    for name in ("ix", "iy", "iz", "nwx", "nwy", "nwz"):
        fluid[name] = rec[name]
    fluid["theta"] = theta_rad
    return solid, fluid


# ------------------------------------------------------------------------------------
# synthetic geometries
# ------------------------------------------------------------------------------------
def tube_with_sphere(nx=64, ny=64, nz=160, radius=30.0, buffer=8, sphere_r=14.0, sphere_z=80):
    """Tube with a spherical obstacle (1-based coordinates): solid outside the z-aligned
    cylinder (i-32)^2+(j-32)^2 > r^2 for buffer < k <= nz-buffer, plus a solid sphere."""
    k, j, i = np.meshgrid(np.arange(1, nz + 1), np.arange(1, ny + 1), np.arange(1, nx + 1), indexing="ij")
    xc, yc = nx / 2.0, ny / 2.0
    w = np.zeros((nz, ny, nx), dtype=np.int8)
    w[((i - xc) ** 2 + (j - yc) ** 2 > radius ** 2) & (k > buffer) & (k <= nz - buffer)] = 1
    w[(i - xc) ** 2 + (j - yc) ** 2 + (k - sphere_z) ** 2 <= sphere_r ** 2] = 1
    return w


def modify_geometry(nx, ny, nz, buffer=10):
    """Hard-coded tube + sphere of modify_geometry (multiphase_3D/0.src/Misc.F90:213-244)."""
    xc, yc, zc = 0.5 * (nx + 1), 0.5 * (ny + 1), 0.5 * (nz + 1)
    r1, r2 = 0.25 * ny, ny * 0.5
    k, j, i = np.meshgrid(np.arange(1, nz + 1), np.arange(1, ny + 1), np.arange(1, nx + 1), indexing="ij")
    w = np.zeros((nz, ny, nx), dtype=np.int8)
    w[(i - xc) ** 2 + (j - yc) ** 2 + (k - zc) ** 2 < r1 ** 2] = 1
    w[((i - xc) ** 2 + (j - yc) ** 2 > r2 ** 2) & (k > buffer) & (k < nz - buffer + 1)] = 1
    return w


def sphere_packing(shape, porosity, mean_r=8.0, sd_r=2.0, seed=0, periodic=(True, True, True)):
    """Overlapping solid spheres with lognormal radii added until the porosity reaches
    the target, then pores not connected to the main pore cluster removed.

    shape = (nz, ny, nx).  Centres are uniform; spheres wrap across periodic faces.
    Returns int8 walls (1 solid, 0 pore).
    """
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    solid = np.zeros(shape, dtype=bool)
    total = solid.size
    n_solid = 0
    target = int(round((1.0 - porosity) * total))
    s2 = math.log(1.0 + (sd_r / mean_r) ** 2)
    mu = math.log(mean_r) - 0.5 * s2
    sg = math.sqrt(s2)
    while n_solid < target:
        r = float(rng.lognormal(mu, sg))
        c = rng.uniform(0.0, 1.0, 3) * np.array([nz, ny, nx])
        R = int(math.ceil(r))
        offs = [np.arange(int(math.floor(c[d])) - R, int(math.floor(c[d])) + R + 2) for d in range(3)]
        idx = []
        for d, (o, n, per) in enumerate(zip(offs, (nz, ny, nx), (periodic[2], periodic[1], periodic[0]))):
            if per:
                idx.append(o % n)
            else:
                idx.append(o[(o >= 0) & (o < n)])
        dz = (idx[0] + 0.5 - c[0])
        dy = (idx[1] + 0.5 - c[1])
        dx = (idx[2] + 0.5 - c[2])
        if periodic[2]:
            dz = (dz + nz / 2.0) % nz - nz / 2.0
        if periodic[1]:
            dy = (dy + ny / 2.0) % ny - ny / 2.0
        if periodic[0]:
            dx = (dx + nx / 2.0) % nx - nx / 2.0
        mask = (dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2) <= r * r
        block = solid[np.ix_(idx[0], idx[1], idx[2])]
        new = mask & ~block
        add = int(np.count_nonzero(new))
        if n_solid + add > target and add > 0:
            # finish exactly at the target: keep the new voxels nearest the centre
            d2 = (dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2)[new]
            order = np.argsort(d2, kind="stable")[: target - n_solid]
            flat = np.flatnonzero(new)[order]
            keep = np.zeros(new.size, dtype=bool)
            keep[flat] = True
            new = keep.reshape(new.shape)
            add = target - n_solid
        solid[np.ix_(idx[0], idx[1], idx[2])] = block | new
        n_solid += add
    walls = solid.astype(np.int8)
    return remove_isolated_pores(walls, periodic)


def remove_isolated_pores(walls, periodic=(True, True, True)):
    """Fill pores that are not part of the largest 18-connected pore cluster (clusters
    are joined across periodic faces)."""
    from scipy import ndimage

    pore = walls == 0
    struct18 = ndimage.generate_binary_structure(3, 2)
    lab, n = ndimage.label(pore, structure=struct18)
    if n <= 1:
        return walls
    parent = np.arange(n + 1)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    def join(a, b):
        m = (a > 0) & (b > 0)
        for x, y in set(zip(a[m].tolist(), b[m].tolist())):
            rx, ry = find(x), find(y)
            if rx != ry:
                parent[max(rx, ry)] = min(rx, ry)

    if periodic[2]:
        join(lab[0], lab[-1])
    if periodic[1]:
        join(lab[:, 0], lab[:, -1])
    if periodic[0]:
        join(lab[:, :, 0], lab[:, :, -1])
    roots = np.array([find(x) for x in range(n + 1)])
    lab = roots[lab]
    sizes = np.bincount(lab.ravel())
    sizes[0] = 0
    keep = int(np.argmax(sizes))
    out = walls.copy()
    out[(lab != keep) & pore] = 1
    return out
