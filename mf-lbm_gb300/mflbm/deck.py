"""simulation_control.txt decks and the host-side derivation of the run parameters.

Parsing follows read_parameter_multi / read_parameter (multiphase_3D/0.src/IO_multiphase.F90:
73-278; singlephase_3D/0.src/IO.F90:80-229): one key per line, the first whitespace-delimited
token is the key, the rest is a list read with Fortran list-directed input (commas or blanks,
`d` exponents).  Unknown keys are ignored, as the reference's `select case` does.

``make_run`` then applies the host-side derivations of initialization_basic_multi
(Init_multiphase.F90:116-150) or initialization_basic (singlephase Initialization.F90:80-129)
and returns the mflbm_params plus the settings the host keeps for itself.
"""
import dataclasses

from ._capi import MFLBM_ABI_VERSION, Params

_INT_KEYS = {
    "initial_fluid_distribution_option", "breakthrough_check", "steady_state_option", "benchmark_cmd",
    "output_fieldData_precision_cmd", "extreme_large_sim_cmd", "modify_geometry_cmd", "external_geometry_read_cmd",
    "geometry_preprocess_cmd", "porous_plate_cmd", "change_inlet_fluid_phase_cmd", "lattice_dimensions",
    "excluded_layers", "domain_wall_status_x", "domain_wall_status_y", "domain_wall_status_z", "periodic_indicator",
    "MPI_async_layers_num", "MPI_process_num", "inlet_BC", "outlet_BC", "Z_porous_plate", "max_time_step",
    "max_time_step_benchmark", "ntime_visual", "ntime_animation", "monitor_timer", "monitor_profile_timer_ratio",
    "computation_time_timer", "display_steps_timer", "MRT_collision_parameter_preset", "double_bak_checkpoint_pdf_cmd",
}


def _value(tok):
    return float(tok.replace("d", "e").replace("D", "e"))


def parse_deck(text):
    """Return {key: list of numbers} for every recognised `key value...` line."""
    out = {}
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line.startswith("#") or line.startswith("!"):
            continue
        parts = line.split(None, 1)
        if len(parts) < 2:
            continue
        key, rest = parts
        rest = rest.split("!")[0]
        toks = [t for t in rest.replace(",", " ").split() if t]
        vals = []
        for t in toks:
            try:
                vals.append(_value(t))
            except ValueError:
                break
        if not vals:
            continue
        if key in _INT_KEYS:
            vals = [int(round(v)) for v in vals]
        out[key] = vals
    return out


def read_deck(path):
    with open(path) as fh:
        return parse_deck(fh.read())


@dataclasses.dataclass
class Run:
    params: Params
    multiphase: bool
    theta_deg: float = 90.0
    interface_z0: float = 0.0
    initial_option: int = 1
    sa_target: float = 0.0
    ntime_max: int = 0
    ntime_monitor: int = 1000
    n_exclude_inlet: int = 0
    n_exclude_outlet: int = 0
    convergence_criteria: float = 1e-6
    steady_state_option: int = 0
    change_inlet_fluid_phase_cmd: int = 0
    flowrate: float = 0.0
    a_xy: float = 0.0


def _get(d, key, default):
    v = d.get(key)
    if v is None:
        return default
    return v if len(v) > 1 else v[0]


def make_run(deck, multiphase=True, device=0, precision=0, strict_fp=0):
    """mflbm_params from a parsed deck, with the reference's host-side derivations; precision
    selects the storage form (see solver.make_params), which the deck itself does not name."""
    nx, ny, nz = _get(deck, "lattice_dimensions", [40, 40, 60])
    wx = _get(deck, "domain_wall_status_x", [1, 1])
    wy = _get(deck, "domain_wall_status_y", [1, 1])
    wz = _get(deck, "domain_wall_status_z", [0, 0])
    per = _get(deck, "periodic_indicator", [0, 0, 0])
    excl = _get(deck, "excluded_layers", [0, 0])
    p = Params()
    p.abi_version = MFLBM_ABI_VERSION
    p.multiphase = 1 if multiphase else 0
    p.nx, p.ny, p.nz = nx, ny, nz
    p.iper, p.jper, p.kper = per
    p.wall_x_min, p.wall_x_max = wx
    p.wall_y_min, p.wall_y_max = wy
    p.wall_z_min, p.wall_z_max = wz
    p.inlet_bc = _get(deck, "inlet_BC", 0)
    p.outlet_bc = _get(deck, "outlet_BC", 0)
    p.porous_plate_cmd = _get(deck, "porous_plate_cmd", 0)
    p.z_porous_plate = _get(deck, "Z_porous_plate", 0)
    p.precision = precision
    p.strict_fp = strict_fp
    p.device = device
    p.relaxation = 1.0
    p.rho_out = 1.0
    p.rho_in = 1.0
    force_z0 = _get(deck, "body_force_0", 0.0)
    p.force_z = force_z0
    open_z = p.kper == 0 and p.wall_z_min == 0 and p.wall_z_max == 0
    # effective open cross-section (Init_multiphase.F90:71-74): half-way walls on x, y
    la_x = float(nx) - 1.0 - 0.5 - 0.5
    la_y = float(ny) - 1.0 - 0.5 - 0.5
    a_xy = la_x * la_y
    run = Run(params=p, multiphase=multiphase, n_exclude_inlet=excl[0], n_exclude_outlet=excl[1],
              ntime_max=_get(deck, "max_time_step", 0), ntime_monitor=_get(deck, "monitor_timer", 1000),
              convergence_criteria=_get(deck, "convergence_criteria", 1e-6),
              steady_state_option=_get(deck, "steady_state_option", 0), a_xy=a_xy)
    if multiphase:
        p.mrt = 2  # the reference's compile-time default (preprocessor.h:2)
        p.la_nu1 = _get(deck, "fluid1_viscosity", 1.0 / 6.0)
        p.la_nu2 = _get(deck, "fluid2_viscosity", 1.0 / 6.0)
        p.gamma = _get(deck, "surface_tension", 0.01)
        p.beta = _get(deck, "RK_beta", 0.95)
        p.sa_inject = _get(deck, "saturation_injection", 1.0)
        run.theta_deg = _get(deck, "theta", 90.0)
        run.interface_z0 = _get(deck, "initial_interface_position", 0.0)
        run.initial_option = _get(deck, "initial_fluid_distribution_option", 1)
        run.sa_target = _get(deck, "target_fluid1_saturation", 0.0)
        # applied once after initialisation or restart (Main_multiphase.F90:96-99) through
        # Solver.change_inlet_fluid_phase(cmd, interface_z0)
        run.change_inlet_fluid_phase_cmd = _get(deck, "change_inlet_fluid_phase_cmd", 0)
        if open_z:
            if p.inlet_bc == 1:
                p.force_z = 0.0
                ca_0 = _get(deck, "capillary_number", 0.0)
                p.uin_avg = ca_0 * p.gamma / p.la_nu1
                run.flowrate = p.uin_avg * a_xy
            elif p.inlet_bc == 2:
                p_gradient = -force_z0 / 3.0
                p.rho_in = p.rho_out - p_gradient * nz
    else:
        p.mrt = _get(deck, "MRT_collision_parameter_preset", 1)
        p.la_nu1 = _get(deck, "fluid_viscosity", 0.05)
        p.la_nu2 = p.la_nu1
        if open_z:
            if p.inlet_bc == 1:
                re = _get(deck, "Reynolds_number", 0.0)
                char_length = _get(deck, "char_length", 1.0)
                p.uin_avg = re * p.la_nu1 / char_length
                run.flowrate = p.uin_avg * a_xy
            elif p.inlet_bc == 2:
                p.rho_in = p.rho_out + _get(deck, "rho_drop", 0.0)
    return run
