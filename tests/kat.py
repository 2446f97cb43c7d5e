"""Known-answer cases of the colour-gradient model, shared by the CPU (oracle) and GPU tests.

The reference ships two measurement set-ups among its initial phase options
(multiphase_3D/0.src/Init_multiphase.F90:294-308): option 5, a free drop in the middle of
the domain (surface-tension measurement), and option 3, a drop attached to the x = 0 wall
(contact-angle measurement).  Their known answers are the Laplace law and the prescribed
contact angle.  Both runs here use walls at x = 1 and x = nx (required for multiphase),
periodic y and z, tau = 1 for both fluids, gamma = 0.01, beta = 0.95, mrt = 2.

  Laplace: p = rho / 3 with rho = rho1 + rho2; dp = p(inside) - p(outside) against
           2 gamma / R, R from the drop volume sum 0.5 (1 + phi) = 4/3 pi R^3.
  Contact angle: a sphere fitted to the phi = 0 crossings (linear interpolation along the
           lattice axes, points more than 3 nodes from the wall) gives the angle through
           fluid 1 (the drop): cos(angle) = (x_w - x_c) / R.  The geometric wetting step
           imposes the angle on the phase normals of the fluid-boundary nodes, the first
           fluid layer i = 2, so x_w = 2 is the plane where the angle is measured (the
           bounce-back wall itself is halfway, at 1.5; both are reported).  The deck's
           contact angle theta is that of fluid 2: the drop's angle is 180 - theta.
"""
import numpy as np

from mflbm import geometry
from mflbm.init import initial_phase
from mflbm.solver import make_params


def drop_case(n_x, n_yz, option, radius, theta_deg=90.0, strict=0, precision=0):
    p = make_params(multiphase=1, nx=n_x, ny=n_yz, nz=n_yz, iper=0, jper=1, kper=1, wall_x_min=1, wall_x_max=1,
                    wall_y_min=0, wall_y_max=0, wall_z_min=0, wall_z_max=0, inlet_bc=0, outlet_bc=0, mrt=2,
                    la_nu1=1.0 / 6.0, la_nu2=1.0 / 6.0, gamma=0.01, beta=0.95, strict_fp=strict, precision=precision)
    wg = np.zeros((n_yz, n_yz, n_x), np.int8)
    walls, pore, wchan = geometry.set_walls(p, wg)
    solid, fluid = geometry.preprocess(p, wchan, geometry.contact_angle_rad(theta_deg))
    phi = initial_phase(p, option, radius)
    return dict(params=p, walls=walls, solid=solid, fluid=fluid, phi=phi)


def start(sim, case):
    sim.set_geometry(case["walls"], case["solid"], case["fluid"])
    sim.init_equilibrium(case["phi"])
    sim.color_gradient()


def laplace(sim, case):
    """(dp, R, max |u|) of a centred drop after an even step."""
    p = case["params"]
    m = sim.macro()
    rho = m["rho"][1:-1, 1:-1, 1:-1]
    ph = m["phi"][4:-4, 4:-4, 4:-4]
    fl = case["walls"][2:-2, 2:-2, 2:-2] == 0
    k, j, i = np.meshgrid(np.arange(1, p.nz + 1), np.arange(1, p.ny + 1), np.arange(1, p.nx + 1), indexing="ij")
    c = 0.5 * np.array([p.nz + 1, p.ny + 1, p.nx + 1])
    d = np.sqrt((k - c[0]) ** 2 + (j - c[1]) ** 2 + (i - c[2]) ** 2)
    v1 = (0.5 * (1.0 + ph))[fl].sum()
    R = (3.0 * v1 / (4.0 * np.pi)) ** (1.0 / 3.0)
    p_in = rho[(d < R - 4.0) & fl].mean() / 3.0
    p_out = rho[(d > R + 5.0) & fl & (i > 3) & (i < p.nx - 2)].mean() / 3.0
    umax = np.sqrt(m["u"] ** 2 + m["v"] ** 2 + m["w"] ** 2).max()
    return p_in - p_out, R, umax


def interface_points(ph):
    """phi = 0 crossings between axis neighbours, linearly interpolated, (k, j, i) with
    the array's own 0-based indices."""
    pts = []
    for ax in range(3):
        a = np.moveaxis(ph, ax, 0)
        s0, s1 = a[:-1], a[1:]
        m = s0 * s1 < 0
        idx = np.nonzero(m)
        t = s0[m] / (s0[m] - s1[m])
        coords = [c.astype(np.float64) for c in idx]
        coords[0] = coords[0] + t
        order = [ax] + [d for d in range(3) if d != ax]
        full = [None] * 3
        for pos, d in enumerate(order):
            full[d] = coords[pos]
        pts.append(np.stack(full, 1))
    return np.concatenate(pts)


def fit_sphere(P):
    """Algebraic least-squares sphere: |x|^2 = 2 c.x + (r^2 - |c|^2)."""
    A = np.c_[2.0 * P, np.ones(len(P))]
    b = (P ** 2).sum(1)
    sol = np.linalg.lstsq(A, b, rcond=None)[0]
    c = sol[:3]
    return c, float(np.sqrt(sol[3] + (c ** 2).sum()))


def drop_angle(sim):
    """Angle through the attached drop (degrees) at the wetting-node plane x = 2 and at
    the bounce-back wall x = 1.5, and max |u|."""
    m = sim.macro()
    ph = m["phi"][4:-4, 4:-4, 4:-4]
    P = interface_points(ph) + 1.0          # lattice coordinates (k, j, i), i = 1..nx
    c, r = fit_sphere(P[P[:, 2] > 1.5 + 3.0])
    ang = lambda xw: float(np.degrees(np.arccos(np.clip((xw - c[2]) / r, -1.0, 1.0))))
    umax = np.sqrt(m["u"] ** 2 + m["v"] ** 2 + m["w"] ** 2).max()
    return ang(2.0), ang(1.5), umax
