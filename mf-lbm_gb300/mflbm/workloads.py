"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference's sample rock images are not available; these generators stand in for them
with the sizes, porosities and flow settings of each configuration.

  tube_drainage         64x64x160 tube with a spherical obstacle, multiphase drainage
  packing_permeability  n^3 sphere packing, singlephase body-force permeability
  packing_throughflow   n^3 sphere packing between inlet/outlet buffers, singlephase
  packing_drainage      sphere packing with inlet/outlet buffers, multiphase drainage
"""
import numpy as np

from . import geometry
from .init import initial_phase
from .solver import make_params


def _assemble_multiphase(p, walls_global, theta_deg, interface_z0, option=1, gpu_preprocess=False):
    walls, pore, wchan = geometry.set_walls(p, walls_global)
    prep = geometry.preprocess_gpu if gpu_preprocess else geometry.preprocess
    solid, fluid = prep(p, wchan, geometry.contact_angle_rad(theta_deg))
    w_in = geometry.inlet_profile(p.nx, p.ny, p.uin_avg) if p.inlet_bc == 1 else None
    phi = initial_phase(p, option, interface_z0)
    return dict(params=p, walls=walls, pore=pore, solid=solid, fluid=fluid, w_in=w_in, phi=phi)


def tube_drainage(strict_fp=0, device=0, nx=64, ny=64, nz=160, precision=0):
    """Plain FP64 multiphase drainage through a tube with a spherical obstacle.

    Walls at x = 1, nx and y = 1, ny; solid outside the z-aligned cylinder of radius 30
    centred at (32, 32) for 9 <= k <= nz-8 (8-layer open buffers); solid sphere of radius
    14 at (32, 32, 80).  phi = +1 for z <= 27, -1 elsewhere; density and viscosity ratio 1
    (tau = 1), gamma = 0.01, contact angle 45 deg, velocity inlet 1e-4 (capillary number
    1e-4 * (1/6) / 0.01), convective outlet, mrt = 2.
    """
    nu = 1.0 / 6.0
    gamma = 0.01
    uin = 1e-4
    p = make_params(multiphase=1, nx=nx, ny=ny, nz=nz, iper=0, jper=0, kper=0, wall_x_min=1, wall_x_max=1,
                    wall_y_min=1, wall_y_max=1, wall_z_min=0, wall_z_max=0, inlet_bc=1, outlet_bc=1, mrt=2,
                    la_nu1=nu, la_nu2=nu, gamma=gamma, beta=0.95, sa_inject=1.0, force_z=0.0, uin_avg=uin,
                    strict_fp=strict_fp, device=device, precision=precision)
    wg = geometry.tube_with_sphere(nx=nx, ny=ny, nz=nz, radius=30.0, buffer=8, sphere_r=14.0, sphere_z=80)
    return _assemble_multiphase(p, wg, theta_deg=45.0, interface_z0=27.0)


def packing_permeability(n=256, porosity=0.22, seed=2024, precision=0, strict_fp=0, device=0, force_z=1e-6):
    """Singlephase permeability: n^3 overlapping spheres (lognormal radii, mean 8, sd 2),
    porosity target, isolated pores removed; periodic x, y, z; body force along z; tau = 1;
    MRT preset 1."""
    p = make_params(multiphase=0, nx=n, ny=n, nz=n, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                    wall_y_min=0, wall_y_max=0, wall_z_min=0, wall_z_max=0, inlet_bc=0, outlet_bc=0, mrt=1,
                    la_nu1=1.0 / 6.0, force_z=force_z, precision=precision, strict_fp=strict_fp, device=device)
    wg = geometry.sphere_packing((n, n, n), porosity, mean_r=8.0, sd_r=2.0, seed=seed)
    walls, pore, _ = geometry.set_walls(p, wg)
    return dict(params=p, walls=walls, pore=pore, walls_global=wg)


def packing_throughflow(n=256, buffer=16, porosity=0.22, seed=11, precision=0, strict_fp=0, device=0, uin=1e-4):
    """Singlephase flow through an n^3 sphere packing (as packing_permeability, not periodic)
    between open inlet and outlet buffers of `buffer` layers: walls on the x and y faces,
    velocity inlet (rectangular-duct profile, mean uin), convective outlet, tau = 1, MRT
    preset 1."""
    nz = n + 2 * buffer
    p = make_params(multiphase=0, nx=n, ny=n, nz=nz, iper=0, jper=0, kper=0, wall_x_min=1, wall_x_max=1,
                    wall_y_min=1, wall_y_max=1, wall_z_min=0, wall_z_max=0, inlet_bc=1, outlet_bc=1, mrt=1,
                    la_nu1=1.0 / 6.0, uin_avg=uin, precision=precision, strict_fp=strict_fp, device=device)
    pack = geometry.sphere_packing((n, n, n), porosity, mean_r=8.0, sd_r=2.0, seed=seed,
                                   periodic=(False, False, False))
    wg = np.zeros((nz, n, n), dtype=np.int8)
    wg[buffer:buffer + n] = pack
    walls, pore, _ = geometry.set_walls(p, wg)
    return dict(params=p, walls=walls, pore=pore, w_in=geometry.inlet_profile(n, n, uin))


def packing_drainage(nxy=512, nzp=512, buffer=32, porosity=0.22, seed=7, strict_fp=0, device=0, precision=0,
                     gpu_preprocess=False):
    """Multiphase drainage of a sphere packing: nxy x nxy x nzp packing plus open inlet and
    outlet buffers of `buffer` layers; walls on the x and y faces; phi = +1 in the inlet
    buffer; injection velocity 5e-5, viscosity ratio 1, gamma = 0.01, contact angle 30 deg."""
    nz = nzp + 2 * buffer
    nu, gamma, uin = 1.0 / 6.0, 0.01, 5e-5
    p = make_params(multiphase=1, nx=nxy, ny=nxy, nz=nz, iper=0, jper=0, kper=0, wall_x_min=1, wall_x_max=1,
                    wall_y_min=1, wall_y_max=1, wall_z_min=0, wall_z_max=0, inlet_bc=1, outlet_bc=1, mrt=2,
                    la_nu1=nu, la_nu2=nu, gamma=gamma, beta=0.95, sa_inject=1.0, force_z=0.0, uin_avg=uin,
                    strict_fp=strict_fp, device=device, precision=precision)
    pack = geometry.sphere_packing((nzp, nxy, nxy), porosity, mean_r=8.0, sd_r=2.0, seed=seed,
                                   periodic=(False, False, False))
    wg = np.zeros((nz, nxy, nxy), dtype=np.int8)
    wg[buffer:buffer + nzp] = pack
    return _assemble_multiphase(p, wg, theta_deg=30.0, interface_z0=float(buffer), gpu_preprocess=gpu_preprocess)


def _ensemble_sample(args):
    e, por, sd = args
    q = make_params(multiphase=0, nx=e, ny=e, nz=e, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                    wall_y_min=0, wall_y_max=0, wall_z_min=0, wall_z_max=0, mrt=1)
    wg = geometry.sphere_packing((e, e, e), float(por), mean_r=8.0, sd_r=2.0, seed=int(sd))
    walls, pore, _ = geometry.set_walls(q, wg)
    return (e, e, e, walls), int(pore)


def packing_ensemble(n_samples=256, edge_lo=48, edge_hi=160, por_lo=0.15, por_hi=0.35, seed=11, precision=1,
                     device=0, force_z=1e-6, workers=0):
    """Batched permeability ensemble: cubic samples with edges drawn uniformly from
    [edge_lo, edge_hi], porosity uniform in [por_lo, por_hi], each a seeded sphere packing
    (lognormal radii mean 8, sd 2, isolated pores removed), periodic x, y, z, body force
    along z, tau = 1, MRT preset 1.  Returns the common params and the sample list
    (nx, ny, nz, halo-2 walls) for mflbm.ensemble.Ensemble, plus the fluid counts.
    workers > 1 builds the samples in a spawn-started process pool (call before any GPU
    work)."""
    rng = np.random.default_rng(seed)
    edges = rng.integers(edge_lo, edge_hi + 1, size=n_samples)
    pors = rng.uniform(por_lo, por_hi, size=n_samples)
    seeds = rng.integers(0, 2**31 - 1, size=n_samples)
    p = make_params(multiphase=0, nx=8, ny=8, nz=8, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                    wall_y_min=0, wall_y_max=0, wall_z_min=0, wall_z_max=0, inlet_bc=0, outlet_bc=0, mrt=1,
                    la_nu1=1.0 / 6.0, force_z=force_z, precision=precision, device=device)
    jobs = [(int(e), float(por), int(sd)) for e, por, sd in zip(edges, pors, seeds)]
    if workers > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            res = pool.map(_ensemble_sample, jobs)
    else:
        res = [_ensemble_sample(j) for j in jobs]
    samples = [r[0] for r in res]
    nf = [r[1] for r in res]
    return dict(params=p, samples=samples, nf=np.array(nf, dtype=np.int64), edges=edges, porosity=pors)
