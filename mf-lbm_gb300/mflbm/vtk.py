"""Legacy VTK field files in the reference's byte layout (``out3.field_data/``).

The reference writes structured-points files as Fortran unformatted streams in big-endian
order: ASCII header lines (each trimmed of trailing blanks, ended by a line feed), then
the values of each scalar over the interior nodes, i fastest, then j, then k.

  VTK_legacy_writer_3D (multiphase_3D/0.src/IO_multiphase.F90:824-1006)
    vtk_type 1  full_flow_field/full_flow_field_<I10.10>.vtk: phi, density, velocity_X/Y/Z
                after compute_macro_vars; float32 (output_fieldData_precision_cmd = 0) or
                float64 (otherwise)
    vtk_type 2  phase_distribution/small_<I10.10>.vtk: phi, float32, zeroed at wall nodes
    vtk_type 3  full_flow_field/force_vector_<I10.10>.vtk: the same five labels holding
                phi, c_norm, cn_x, cn_y, cn_z (the reference reuses the labels)
  VTK_phi_2d_micromodel (:1011-1089)
                phase_distribution/small_2d_<I10.10>.vtk: 0.5 (1 + mean of phi over
                j = 2 .. ny-1) on an nx x 1 x nz grid, float32.  The reference gathers
                phi with its FP64 gather into an array declared real(4) (a mismatch its
                build tolerates through -fallow-argument-mismatch, with undefined
                contents); this writer stores the values the routine describes: the mean
                in FP64, rounded to float32.
  VTK_walls_bin (:1095-1149)
                walls_bin.vtk: the global wall array as int32

Values come from the library through ``Solver`` (or anything with its interface): one
device reduction or download per file, the file itself written on the host.
"""
import os

import numpy as np

LF = "\n"


def _i(n, w):
    return str(int(n)).rjust(w)


def header(dims, npoints, spacing=(1, 1, 1), point_width=14):
    """Header lines of a structured-points file, as the reference assembles them."""
    lines = ["# vtk DataFile Version 3.0", "vtk output", "BINARY", "DATASET STRUCTURED_POINTS ",
             "DIMENSIONS " + " ".join(_i(d, 10) for d in dims),
             "ORIGIN " + " ".join(_i(1, 10) for _ in range(3)),
             "SPACING " + " ".join(_i(s, 10) for s in spacing),
             "POINT_DATA " + _i(npoints, point_width)]
    return "".join(line + LF for line in lines).encode("ascii")


def scalar_block(name, values, vtype):
    """'SCALARS <name> <type>' + lookup-table line + big-endian values (i fastest)."""
    big = {"float": ">f4", "double": ">f8", "int": ">i4"}[vtype]
    head = f"SCALARS {name} {vtype}{LF}LOOKUP_TABLE default{LF}".encode("ascii")
    return head + np.ascontiguousarray(values).astype(big).tobytes()


def field_name(nt):
    return "%010d.vtk" % int(nt)


def _interior(a, h):
    return a[h:-h, h:-h, h:-h]


def write_3d(root, nt, vtk_type, fields, precision_cmd=0):
    """Write one VTK_legacy_writer_3D file from interior arrays (nz, ny, nx).

    fields: dict with phi (and, for vtk_type 1, rho, u, v, w; for vtk_type 3, c_norm,
    cn_x, cn_y, cn_z).  Returns the path."""
    phi = fields["phi"]
    nz, ny, nx = phi.shape
    if vtk_type == 1:
        sub, base = "full_flow_field", "full_flow_field_"
        cols = [fields[k] for k in ("phi", "rho", "u", "v", "w")]
    elif vtk_type == 3:
        sub, base = "full_flow_field", "force_vector_"
        cols = [fields[k] for k in ("phi", "c_norm", "cn_x", "cn_y", "cn_z")]
    elif vtk_type == 2:
        sub, base = "phase_distribution", "small_"
        cols = [phi]
    else:
        raise ValueError("vtk_type must be 1, 2 or 3")
    d = os.path.join(root, "out3.field_data", sub)
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, base + field_name(nt))
    out = [header((nx, ny, nz), nx * ny * nz)]
    if vtk_type == 2:
        out.append(scalar_block("phi", phi, "float"))
    else:
        vtype = "float" if precision_cmd == 0 else "double"
        for name, a in zip(("phi", "density", "velocity_X", "velocity_Y", "velocity_Z"), cols):
            out.append(scalar_block(name, a, vtype))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))
    return path


def save_field(sim, root, nt, vtk_type, precision_cmd=0):
    """VTK_legacy_writer_3D for a Solver at time step nt (after an even step for
    vtk_type 1, whose velocities come from compute_macro_vars).  vtk_type 1 and 2 take phi
    from compute_macro_vars, which zeroes it at wall nodes in the device state as well, as
    the reference's writers do; vtk_type 3 reads the colour-gradient fields."""
    if vtk_type in (1, 2):
        m = sim.macro()
        fields = {"phi": _interior(m["phi"], 4)}
        if vtk_type == 1:
            fields.update(rho=_interior(m["rho"], 1), u=_interior(m["u"], 1), v=_interior(m["v"], 1),
                          w=_interior(m["w"], 1))
    elif vtk_type == 3:
        g = sim.get_gradient()
        fields = {"phi": _interior(sim.download_state()["phi"], 4), "c_norm": _interior(g["c_norm"], 2),
                  "cn_x": _interior(g["cn_x"], 2), "cn_y": _interior(g["cn_y"], 2), "cn_z": _interior(g["cn_z"], 2)}
    else:
        raise ValueError("vtk_type must be 1, 2 or 3")
    return write_3d(root, nt, vtk_type, fields, precision_cmd)


def write_phi_2d_micromodel(root, nt, phi):
    """VTK_phi_2d_micromodel from the interior phase field (nz, ny, nx), zeroed at walls:
    0.5 (1 + sum over j = 2 .. ny-1 / (ny - 2)), summed in the reference's j order."""
    nz, ny, nx = phi.shape
    tmp = np.zeros((nz, nx))
    for j in range(1, ny - 1):          # j = 2 .. ny-1 (1-based), sequential like the Fortran
        tmp = tmp + phi[:, j, :]
    avg = (0.5 * (1.0 + tmp / (ny - 2))).astype(np.float32)
    d = os.path.join(root, "out3.field_data", "phase_distribution")
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, "small_2d_" + field_name(nt))
    body = header((nx, 1, nz), nx * nz, spacing=(1, 0, 1), point_width=10)
    body += scalar_block("phi", avg, "float")
    with open(path, "wb") as fh:
        fh.write(body)
    return path


def save_phi_2d_micromodel(sim, root, nt):
    return write_phi_2d_micromodel(root, nt, _interior(sim.macro()["phi"], 4))


def write_walls(root, walls_global):
    """VTK_walls_bin: the global wall array (nz, ny, nx) as big-endian int32."""
    nz, ny, nx = walls_global.shape
    d = os.path.join(root, "out3.field_data")
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, "walls_bin.vtk")
    with open(path, "wb") as fh:
        fh.write(header((nx, ny, nz), nx * ny * nz) + scalar_block("walls", walls_global.astype(np.int32), "int"))
    return path
