"""Monitor output files in the reference's layout (``out1.output/``).

Every record is appended with the reference's Fortran edit descriptors, reproduced by
``fortran_e`` / ``fortran_i``:

multiphase (multiphase_3D/0.src/Monitor.F90:157-260)
  saturation.dat              (I10,5(1x,e14.7))  ntime, S, vol1, vol2, mass1, mass2  over the sample
  Ca_number.dat               (I10,4(1x,e14.7))  ntime, Ca, umax, KE1, KE2
  flowrate_time.dat           (I10,6(1x,E14.6))  ntime, fl, fl1, fl2 (whole), fl, fl1, fl2 (sample)
  saturation_full_domain.dat  (I10,5(1x,e14.7))
  pre.dat                     (I10,3(1x,e14.7))  open z only: inlet, outlet pressure and drop
  profile/monitor<I10.8>.dat  (5(1x,e14.7))      every ntime_monitor_profile steps
  steady_monitor_saturation_error.dat (steady_state_option 3)
  steady_monitor_capillary_pressure_error.dat (I10,6(1x,e14.7))  steady_state_option 1
  steady_monitor_max_phi_change.dat            (I10,2(1x,e14.7))  steady_state_option 2
  (multiphase_3D/0.src/Monitor.F90:287-507 with Solver.steady_monitor)
singlephase (singlephase_3D/0.src/Monitor.F90:109-165)
  flowrate_time.dat           (I10,2(1x,E14.6))  ntime, flowrate, umax
  pre.dat, profile/monitor<I10.8>.dat (3(1x,e14.7)),
  steady_monitor_flowrate_error.dat (steady_state_option 1)

The per-slice sums come from ``Solver.monitor()`` (FP64 device reductions).
"""
import math
import os

import numpy as np

EPS = 1.110223025e-16  # eps of multiphase_3D/0.src/Module.F90:8

RUNNING, CONVERGED, FAILED = 0, 1, 3


def fortran_e(x, w=14, d=7):
    """Fortran Ew.d: 0.ddddddd E+xx, right-justified in w characters."""
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    if x == 0.0:
        s = "0." + "0" * d + "E+00"
    else:
        m, e = ("%.*e" % (d - 1, abs(x))).split("e")
        digits = m.replace(".", "")
        exp = int(e) + 1
        if abs(exp) <= 99:
            s = "0.%sE%+03d" % (digits, exp)
        else:
            s = "0.%s%+04d" % (digits, exp)
        if x < 0:
            s = "-" + s
    return s.rjust(w)


def fortran_i(n, w=10, m=None):
    s = str(abs(int(n)))
    if m is not None:
        s = s.rjust(m, "0")
    if n < 0:
        s = "-" + s
    return s.rjust(w)


def record(ntime, values, w=14, d=7):
    return fortran_i(ntime) + "".join(" " + fortran_e(v, w, d) for v in values) + "\n"


def profile_name(ntime):
    # write(flnm,'(I10.8,".dat")') ntime: width 10 with at least 8 digits
    return "monitor" + fortran_i(ntime, 10, 8) + ".dat"


class MonitorFiles:
    """Appends the reference's monitor records for one run.

    pore_profile_z : fluid nodes per z slice (length nz), the reference's pore_profile_z.
    """

    def __init__(self, root, params, pore_profile_z, n_exclude_inlet=0, n_exclude_outlet=0, a_xy=None,
                 ntime_monitor=1000, ntime_monitor_profile=None, steady_state_option=0,
                 convergence_criteria=1e-6):
        self.dir = os.path.join(root, "out1.output")
        os.makedirs(os.path.join(self.dir, "profile"), exist_ok=True)
        self.p = params
        self.pore_z = np.asarray(pore_profile_z, dtype=np.float64)
        self.n_in, self.n_out = n_exclude_inlet, n_exclude_outlet
        self.a_xy = a_xy if a_xy is not None else float(params.nx - 2) * float(params.ny - 2)
        self.ntime_monitor = ntime_monitor
        self.ntime_profile = ntime_monitor_profile
        self.steady = steady_state_option
        self.criteria = convergence_criteria
        self.current = 0.0
        self.previous = 0.0

    def _append(self, name, line):
        with open(os.path.join(self.dir, name), "a") as fh:
            fh.write(line)

    def _open_z(self):
        p = self.p
        return p.kper == 0 and p.wall_z_min == 0 and p.wall_z_max == 0

    def write(self, ntime, profiles, scalars):
        """Append one monitor call's records; returns the simulation_end_indicator."""
        return self._multi(ntime, profiles, scalars) if self.p.multiphase else self._single(ntime, profiles, scalars)

    def _pressure(self, ntime, pre):
        if not self._open_z():
            return
        nz = self.p.nz
        t1 = pre[self.n_in] / self.pore_z[self.n_in]
        t2 = pre[nz - self.n_out - 1] / self.pore_z[nz - self.n_out - 1]
        self._append("pre.dat", record(ntime, [t1, t2, t1 - t2]))

    def _single(self, ntime, prof, scal):
        fl, pre = prof[0], prof[1]
        nz = self.p.nz
        umax = math.sqrt(scal[0])
        flowrate = float(np.sum(fl)) / nz
        self._append("flowrate_time.dat", record(ntime, [flowrate, umax], 14, 6))
        self._pressure(ntime, pre)
        if self.ntime_profile and ntime % self.ntime_profile == 0:
            with open(os.path.join(self.dir, "profile", profile_name(ntime)), "w") as fh:
                for k in range(nz):
                    fh.write("".join(" " + fortran_e(v) for v in (k + 1.0, fl[k], pre[k] / (self.pore_z[k] + EPS))) + "\n")
        end = RUNNING
        if self.steady == 1:
            self.previous, self.current = self.current, flowrate
            rel = abs(self.current - self.previous) / (abs(self.current) + EPS)
            self._append("steady_monitor_flowrate_error.dat", record(ntime, [rel]))
            if rel < self.criteria and ntime > self.ntime_monitor:
                end = CONVERGED
        if math.isnan(flowrate) or umax > 0.5:
            end = FAILED
        return end

    def _multi(self, ntime, prof, scal):
        fl1, fl2, vol1, vol2, mass1, mass2, pre = prof
        p = self.p
        nz = p.nz
        sl = slice(self.n_in, nz - self.n_out)
        umax = math.sqrt(scal[0])
        ke1, ke2 = 0.5 * scal[1], 0.5 * scal[2]
        m1, m2, v1, v2 = mass1[sl].sum(), mass2[sl].sum(), vol1[sl].sum(), vol2[sl].sum()
        sat = v1 / (v1 + v2)
        self._append("saturation.dat", record(ntime, [sat, v1, v2, m1, m2]))
        t1, t2, t3, t4 = mass1.sum(), mass2.sum(), vol1.sum(), vol2.sum()
        sat_full = t3 / (t3 + t4)
        fl1w, fl2w = fl1.sum() / nz, fl2.sum() / nz
        nsamp = nz - self.n_out - self.n_in
        fl1a, fl2a = fl1[sl].sum() / nsamp, fl2[sl].sum() / nsamp
        ca = (fl1a + fl2a) / self.a_xy * p.la_nu1 / p.gamma
        self._append("Ca_number.dat", record(ntime, [ca, umax, ke1, ke2]))
        self._append("flowrate_time.dat", record(ntime, [fl1w + fl2w, fl1w, fl2w, fl1a + fl2a, fl1a, fl2a], 14, 6))
        self._append("saturation_full_domain.dat", record(ntime, [sat_full, t3, t4, t1, t2]))
        self._pressure(ntime, pre)
        if self.ntime_profile and ntime % self.ntime_profile == 0:
            with open(os.path.join(self.dir, "profile", profile_name(ntime)), "w") as fh:
                for k in range(nz):
                    vals = (k + 1.0, fl1[k], fl2[k], mass1[k] / (mass1[k] + mass2[k]), pre[k] / (self.pore_z[k] + EPS))
                    fh.write("".join(" " + fortran_e(v) for v in vals) + "\n")
        end = RUNNING
        if math.isnan(sat_full) or math.isnan(ca) or umax > 0.5:
            end = FAILED
        if self.steady == 3:
            self.previous, self.current = self.current, sat_full
            rel = abs(self.current - self.previous) / (abs(self.current) + EPS)
            self._append("steady_monitor_saturation_error.dat", record(ntime, [rel]))
            if rel < self.criteria and ntime > self.ntime_monitor:
                end = CONVERGED
        return end


def write_capillary_pressure(mf, ntime, out):
    """monitor_multiphase_steady_capillarypressure's record and end indicator
    (Monitor.F90:434-459) from Solver.steady_monitor(1)."""
    pc, pre_w, pre_nw, umax = out[0], out[1], out[2], out[3]
    mf.previous, mf.current = mf.current, pc
    temp = abs(mf.current - mf.previous) / (abs(mf.current) + EPS)
    mf._append("steady_monitor_capillary_pressure_error.dat", record(ntime, [temp, pc, pre_w, pre_nw, temp, umax]))
    if math.isnan(umax) or math.isnan(pc):
        return FAILED
    if umax >= 0.5:
        return FAILED
    return CONVERGED if (temp < mf.criteria and ntime > mf.ntime_monitor) else RUNNING


def write_phase_field_change(mf, ntime, out, ntime_relaxation=0):
    """monitor_multiphase_steady_phasefield's record and end indicator (Monitor.F90:340-360)
    from Solver.steady_monitor(2)."""
    d_phi, umax = out[0], out[1]
    if ntime <= ntime_relaxation:
        return RUNNING
    if math.isnan(umax) or math.isnan(d_phi):
        return FAILED
    mf._append("steady_monitor_max_phi_change.dat", record(ntime, [d_phi, umax]))
    if umax >= 0.5:
        return FAILED
    return CONVERGED if (d_phi < mf.criteria and ntime > mf.ntime_monitor) else RUNNING


def breakthrough(count):
    """monitor_breakthrough (Monitor.F90:500-503): end once fluid 1 reaches z = nz - 1."""
    return CONVERGED if count >= 1 else RUNNING
