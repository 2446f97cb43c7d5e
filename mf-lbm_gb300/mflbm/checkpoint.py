"""Checkpoint files byte-compatible with the reference's save_checkpoint / initialization_old.

Layout (Fortran unformatted stream, little-endian, no record markers), one file per
rank named ``id%04d`` under ``out2.checkpoint/`` (``out2.checkpoint/2rd_backup/`` for the
secondary copy):

  int32 ntime_next, float64 force_z, float64 rho_in
  f0 .. f18          (nx+2)(ny+2)(nz+2) float64 each, halo 1, i fastest
  g0 .. g18          same                                      (multiphase only)
  phi                (nx+8)(ny+8)(nz+8) float64, halo 4         (multiphase only)
  f_convec_bc        (nx+2)(ny+2)*19 float64                    (outlet_BC == 1)
  g_convec_bc        same                                       (multiphase, outlet_BC == 1)
  phi_convec_bc      (nx+2)(ny+2) float64                       (multiphase, outlet_BC == 1)

multiphase_3D/0.src/IO_multiphase.F90:562-642 writes it and Init_multiphase.F90:477-557
reads it back; the singlephase pair is singlephase_3D/0.src/IO.F90:490-547 and
Initialization.F90:314-371.  ntime_next is the ntime the resumed run starts with
(the writer stores ntime+1).  The arrays are exactly what ``Solver.download_state``
returns, so a file written here resumes a reference run and the other way round.
"""
import os
import struct

import numpy as np

_HEADER = struct.Struct("<idd")


def file_name(rank=0):
    return "id%04d" % rank


def checkpoint_path(root, rank=0, secondary=False):
    d = os.path.join(root, "out2.checkpoint", "2rd_backup") if secondary else os.path.join(root, "out2.checkpoint")
    return os.path.join(d, file_name(rank))


def expected_size(nx, ny, nz, multiphase, outlet_bc):
    n1 = (nx + 2) * (ny + 2) * (nz + 2)
    n4 = (nx + 8) * (ny + 8) * (nz + 8)
    plane = (nx + 2) * (ny + 2)
    words = 19 * n1
    if multiphase:
        words += 19 * n1 + n4
    if outlet_bc == 1:
        words += 19 * plane
        if multiphase:
            words += 19 * plane + plane
    return _HEADER.size + 8 * words


def _arrays(state, multiphase, outlet_bc):
    out = [state["f"]]
    if multiphase:
        out += [state["g"], state["phi"]]
    if outlet_bc == 1:
        out.append(state["f_convec"])
        if multiphase:
            out += [state["g_convec"], state["phi_convec"]]
    return out


def write_checkpoint(path, state, ntime_next, force_z, rho_in, multiphase, outlet_bc):
    """Write `state` (the dict of Solver.download_state) in the reference's layout."""
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "wb") as fh:
        fh.write(_HEADER.pack(int(ntime_next), float(force_z), float(rho_in)))
        for a in _arrays(state, multiphase, outlet_bc):
            fh.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
    os.replace(tmp, path)


def read_checkpoint(path, nx, ny, nz, multiphase, outlet_bc):
    """Read a checkpoint; returns (ntime_next, force_z, rho_in, state dict)."""
    size = os.path.getsize(path)
    want = expected_size(nx, ny, nz, multiphase, outlet_bc)
    if size != want:
        raise ValueError(f"{path}: {size} bytes, expected {want} for {nx}x{ny}x{nz} "
                         f"multiphase={int(bool(multiphase))} outlet_BC={outlet_bc}")
    s1 = (19, nz + 2, ny + 2, nx + 2)
    s4 = (nz + 8, ny + 8, nx + 8)
    sp = (19, ny + 2, nx + 2)
    with open(path, "rb") as fh:
        ntime_next, force_z, rho_in = _HEADER.unpack(fh.read(_HEADER.size))

        def take(shape):
            n = int(np.prod(shape))
            return np.frombuffer(fh.read(8 * n), dtype="<f8").reshape(shape).astype(np.float64)

        state = {"f": take(s1)}
        if multiphase:
            state["g"] = take(s1)
            state["phi"] = take(s4)
        if outlet_bc == 1:
            state["f_convec"] = take(sp)
            if multiphase:
                state["g_convec"] = take(sp)
                state["phi_convec"] = take((ny + 2, nx + 2))
    return ntime_next, force_z, rho_in, state


def save(sim, root, ntime, rank=0, secondary=False, job_status=True):
    """save_checkpoint for a Solver after step `ntime` (stores ntime+1)."""
    p = sim.p
    path = checkpoint_path(root, rank, secondary)
    write_checkpoint(path, sim.download_state(), ntime + 1, p.force_z, p.rho_in, p.multiphase, p.outlet_bc)
    if job_status and rank == 0 and not secondary:
        with open(os.path.join(root, "job_status.txt"), "w") as fh:
            fh.write("continue_simulation\n")
    return path


def load(sim, root, rank=0):
    """initialization_old for a Solver whose geometry is set: uploads the state and, for
    multiphase, recomputes the colour gradient from the loaded phi as the reference does
    right after loading (multiphase_3D/0.src/Main_multiphase.F90:120).  Returns ntime0
    and the file's force_z and rho_in for the caller to compare with (or adopt into)
    its parameters."""
    p = sim.p
    ntime0, force_z, rho_in, st = read_checkpoint(checkpoint_path(root, rank), p.nx, p.ny, p.nz, p.multiphase,
                                                  p.outlet_bc)
    sim.upload_state(st["f"], st.get("g"), st.get("phi"), st.get("f_convec"), st.get("g_convec"),
                     st.get("phi_convec"))
    if p.multiphase:
        sim.color_gradient()
    return ntime0, force_z, rho_in
