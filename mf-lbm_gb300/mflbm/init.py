"""Initial phase field of initialization_new_multi (multiphase_3D/0.src/Init_multiphase.F90:
243-337) for one rank, over the halo-4 box, as a (nz+8, ny+8, nx+8) array indexed [k+3, j+3, i+3].

Options 1-5 follow the reference exactly.  Option 6 (random saturation) draws from a seeded
numpy generator instead of Fortran's unseeded RANDOM_NUMBER, so runs are reproducible.
"""
import numpy as np


def initial_phase(p, option, interface_z0, sa_target=0.0, seed=0):
    nx, ny, nz = p.nx, p.ny, p.nz
    k = np.arange(-3, nz + 5, dtype=np.float64)[:, None, None]
    j = np.arange(-3, ny + 5, dtype=np.float64)[None, :, None]
    i = np.arange(-3, nx + 5, dtype=np.float64)[None, None, :]
    x, y, z = i, j, k
    shape = (nz + 8, ny + 8, nx + 8)
    if option == 1:      # drainage
        phi = np.where(z <= interface_z0, 1.0, -1.0) * np.ones(shape)
    elif option == 2:    # imbibition
        phi = np.where(z <= interface_z0, -1.0, 1.0) * np.ones(shape)
    elif option in (3, 4):   # drop attached to the x = 0 wall
        d = (x - (nx + 1) * 0.0) ** 2 + (z - (nz + 1) * 0.5) ** 2 + (y - (ny + 1) * 0.5) ** 2
        inside = d <= interface_z0 ** 2
        phi = np.where(inside, 1.0, -1.0) if option == 3 else np.where(inside, -1.0, 1.0)
    elif option == 5:    # free drop in the centre
        d = (x - (nx + 1) * 0.5) ** 2 + (z - (nz + 1) * 0.5) ** 2 + (y - (ny + 1) * 0.5) ** 2
        phi = np.where(d <= interface_z0 ** 2, 1.0, -1.0)
    elif option == 6:    # random distribution at the target saturation
        rng = np.random.default_rng(seed)
        phi = np.where(rng.random(shape) > sa_target, -1.0, 1.0)
    else:
        raise ValueError("initial_fluid_distribution_option must be 1..6")
    phi = np.ascontiguousarray(np.broadcast_to(phi, shape), dtype=np.float64).copy()
    if p.kper == 0 and p.wall_z_min == 0 and p.wall_z_max == 0:
        phi[: 3 + 1] = 2.0 * p.sa_inject - 1.0   # z <= 0 gets the injected phase (:323-337)
    return phi
