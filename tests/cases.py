"""Seeded input builders shared by the CPU and GPU tests.

Every case is a complete, reproducible set of inputs for one context: parameters,
walls (halo 2), boundary lists, inlet profile and an initial halo'd state.  The same
inputs go to the GPU library and to the oracle.
"""
import numpy as np

from mflbm import geometry
from mflbm.solver import make_params

W = np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12)
# rest state of the reference MRT (equilibrium e2 moment 0)
W_MRT = np.array([4.0 / 21.0] + [13.0 / 126.0] * 6 + [1.0 / 63.0] * 12)


def random_spheres(shape, n, rmin, rmax, seed):
    """n random solid spheres (no wrap) in a (nz, ny, nx) box."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    w = np.zeros(shape, dtype=np.int8)
    for _ in range(n):
        c = rng.uniform(0, 1, 3) * np.array([nz, ny, nx])
        r = rng.uniform(rmin, rmax)
        w[(k - c[0]) ** 2 + (j - c[1]) ** 2 + (i - c[2]) ** 2 <= r * r] = 1
    return w


def perturbed_pdfs(shape1, seed, rho1=None, amp=1e-3, weights=W):
    """Equilibrium-like PDFs w_q*rho*(1 + amp*noise) over the whole halo'd box."""
    rng = np.random.default_rng(seed)
    if rho1 is None:
        rho1 = np.ones(shape1)
    noise = rng.uniform(-1.0, 1.0, (19,) + shape1)
    return weights[:, None, None, None] * rho1[None] * (1.0 + amp * noise)


def sp_case(nx=12, ny=10, nz=14, per=(0, 1, 1), inlet=0, outlet=0, force=1e-5, nu=0.1, mrt=1, spheres=3, seed=1,
            precision=0, strict=1, uin=5e-3, rho_in=1.001, rest="bgk", layout=0):
    iper, jper, kper = per
    p = make_params(multiphase=0, nx=nx, ny=ny, nz=nz, iper=iper, jper=jper, kper=kper,
                    wall_x_min=0 if iper else 1, wall_x_max=0 if iper else 1,
                    wall_y_min=0 if jper else 1, wall_y_max=0 if jper else 1,
                    wall_z_min=0, wall_z_max=0, inlet_bc=inlet, outlet_bc=outlet, mrt=mrt, la_nu1=nu,
                    force_z=force, uin_avg=uin, rho_in=rho_in, rho_out=1.0, precision=precision, strict_fp=strict,
                    layout=layout)
    wg = random_spheres((nz, ny, nx), spheres, 1.5, 3.0, seed) if spheres else np.zeros((nz, ny, nx), np.int8)
    walls, pore, _ = geometry.set_walls(p, wg)
    w_in = geometry.inlet_profile(nx, ny, uin) if inlet == 1 else None
    shape1 = (nz + 2, ny + 2, nx + 2)
    f = perturbed_pdfs(shape1, seed + 100, weights=W_MRT if rest == "mrt" else W)
    fconv = f[:, nz, :, :].copy() if outlet == 1 else None
    return dict(params=p, walls=walls, pore=pore, w_in=w_in, f=f, f_convec=fconv)


def smooth_phase(shape4, seed, kind="blob"):
    """A smooth phase field in [-1, 1] over the halo-4 box."""
    nz, ny, nx = shape4
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    rng = np.random.default_rng(seed)
    if kind == "slab":
        z0 = nz * 0.4
        return np.tanh((z0 - k) / 1.5)
    c = np.array([nz, ny, nx]) * rng.uniform(0.35, 0.65, 3)
    r = min(nx, ny, nz) * 0.3
    d = np.sqrt((k - c[0]) ** 2 + (j - c[1]) ** 2 + (i - c[2]) ** 2)
    return np.tanh((r - d) / 1.5)


def mp_case(nx=14, ny=12, nz=16, per=(0, 1, 1), inlet=0, outlet=0, force=0.0, spheres=2, seed=3, theta_deg=45.0,
            mrt=2, nu1=1.0 / 6.0, nu2=1.0 / 6.0, gamma=0.01, beta=0.95, strict=1, uin=1e-3, rho_in=1.001,
            plate=0, zplate=0, sa_inject=1.0, precision=0, layout=1):
    _, jper, kper = per
    p = make_params(multiphase=1, nx=nx, ny=ny, nz=nz, iper=0, jper=jper, kper=kper, wall_x_min=1, wall_x_max=1,
                    wall_y_min=0 if jper else 1, wall_y_max=0 if jper else 1, wall_z_min=0, wall_z_max=0,
                    inlet_bc=inlet, outlet_bc=outlet, mrt=mrt, la_nu1=nu1, la_nu2=nu2, gamma=gamma, beta=beta,
                    sa_inject=sa_inject, force_z=force, uin_avg=uin, rho_in=rho_in, rho_out=1.0, strict_fp=strict,
                    porous_plate_cmd=plate, z_porous_plate=zplate, precision=precision, layout=layout)
    wg = random_spheres((nz, ny, nx), spheres, 1.5, 3.0, seed) if spheres else np.zeros((nz, ny, nx), np.int8)
    walls, pore, wchan = geometry.set_walls(p, wg)
    solid, fluid = geometry.preprocess(p, wchan, geometry.contact_angle_rad(theta_deg))
    w_in = geometry.inlet_profile(nx, ny, uin) if inlet == 1 else None
    shape1 = (nz + 2, ny + 2, nx + 2)
    shape4 = (nz + 8, ny + 8, nx + 8)
    phi = smooth_phase(shape4, seed, "blob")
    ph1 = phi[3:nz + 5, 3:ny + 5, 3:nx + 5]
    f = perturbed_pdfs(shape1, seed + 10, 0.5 * (1.0 + ph1))
    g = perturbed_pdfs(shape1, seed + 20, 0.5 * (1.0 - ph1))
    out = dict(params=p, walls=walls, pore=pore, solid=solid, fluid=fluid, w_in=w_in, f=f, g=g, phi=phi)
    if outlet == 1:
        out.update(f_convec=f[:, nz].copy(), g_convec=g[:, nz].copy(), phi_convec=phi[nz + 3, 3:ny + 5, 3:nx + 5].copy())
    return out


def load_case(sim, case):
    """Geometry + state upload through the common Solver/Oracle interface."""
    sim.set_geometry(case["walls"], case.get("solid"), case.get("fluid"), case.get("w_in"))
    sim.upload_state(case["f"], case.get("g"), case.get("phi"), case.get("f_convec"), case.get("g_convec"),
                     case.get("phi_convec"))
    if case["params"].multiphase:
        sim.color_gradient()


def periodic_ghosts(a, per):
    """Fill the halo-1 ghost layers of the periodic axes of a (..., nz+2, ny+2, nx+2)
    array with their periodic images (x, then y, then z, so edges and corners follow)."""
    a = a.copy()
    for axis, p in zip((-1, -2, -3), per):
        if not p:
            continue
        n = a.shape[axis] - 2
        src_hi = [slice(None)] * a.ndim
        dst_lo = [slice(None)] * a.ndim
        src_lo = [slice(None)] * a.ndim
        dst_hi = [slice(None)] * a.ndim
        src_hi[axis], dst_lo[axis] = slice(n, n + 1), slice(0, 1)
        src_lo[axis], dst_hi[axis] = slice(1, 2), slice(n + 1, n + 2)
        a[tuple(dst_lo)] = a[tuple(src_hi)]
        a[tuple(dst_hi)] = a[tuple(src_lo)]
    return a
