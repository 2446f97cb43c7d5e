"""Deck parsing and the host-side parameter derivations (CPU only)."""
import numpy as np

from mflbm import deck
from mflbm.init import initial_phase
from mflbm.solver import make_params

MULTI = """
initial_fluid_distribution_option 1
steady_state_option 0
convergence_criteria 1d-6
lattice_dimensions 64,64,160
excluded_layers 8,8
domain_wall_status_x 1,1
domain_wall_status_y 1,1
domain_wall_status_z 0,0
periodic_indicator 0,0,0
fluid1_viscosity 0.1666666666666667
fluid2_viscosity 0.1666666666666667
surface_tension 0.01
theta 45
RK_beta 0.95
inlet_BC 1
outlet_BC 1
saturation_injection 1.0
initial_interface_position 27.0
capillary_number 1.6666666666666667d-3
body_force_0 0d-6
max_time_step 2000
monitor_timer 100
unknown_key 42
"""

SINGLE = """
MRT_collision_parameter_preset 1
lattice_dimensions 40,40,60
domain_wall_status_x 1,1
domain_wall_status_y 1,1
domain_wall_status_z 0,0
periodic_indicator 0,0,0
fluid_viscosity 0.05
inlet_BC 2
outlet_BC 2
rho_drop 0.01
body_force_0 1d-6
"""


def test_parse_multiphase_deck():
    d = deck.parse_deck(MULTI)
    assert d["lattice_dimensions"] == [64, 64, 160]
    assert d["capillary_number"] == [1.6666666666666667e-3]
    assert "unknown_key" in d  # kept, ignored by make_run
    run = deck.make_run(d, multiphase=True)
    p = run.params
    assert (p.nx, p.ny, p.nz) == (64, 64, 160)
    assert p.inlet_bc == 1 and p.outlet_bc == 1 and p.mrt == 2
    # velocity inlet: force off, uin = Ca * gamma / nu1 (Init_multiphase.F90:143, 203)
    assert p.force_z == 0.0
    assert abs(p.uin_avg - 1e-4) < 1e-15
    assert run.a_xy == 62.0 * 62.0
    assert run.theta_deg == 45 and run.interface_z0 == 27.0


def test_parse_singlephase_pressure_deck():
    run = deck.make_run(deck.parse_deck(SINGLE), multiphase=False)
    p = run.params
    assert p.mrt == 1 and p.la_nu1 == 0.05
    assert abs(p.rho_in - 1.01) < 1e-15 and p.rho_out == 1.0
    assert p.force_z == 1e-6  # singlephase keeps the body force


def test_initial_phase_options():
    p = make_params(multiphase=1, nx=10, ny=8, nz=12, inlet_bc=1, outlet_bc=1, sa_inject=0.0)
    phi = initial_phase(p, 1, 5.0)
    assert phi.shape == (20, 16, 18)
    assert (phi[4:9] == 1.0).all()          # z = 1..5
    assert (phi[9:] == -1.0).all()
    assert (phi[:4] == -1.0).all()          # z <= 0: phi_inlet = 2*0-1
    phi5 = initial_phase(p, 5, 3.0)
    assert phi5[3 + 6, 3 + 4, 3 + 5] == 1.0 or phi5[3 + 7, 3 + 5, 3 + 6] == 1.0
    assert set(np.unique(phi5)) <= {-1.0, 1.0}
    a = initial_phase(p, 6, 0.0, sa_target=0.4, seed=1)
    b = initial_phase(p, 6, 0.0, sa_target=0.4, seed=1)
    assert np.array_equal(a, b)
