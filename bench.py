#!/usr/bin/env python3
"""Benchmark: singlephase D3Q19 permeability lattice update, MLUPS on one GB300.

Workload (one bench "step" = one LBM time step over the whole lattice):
  256^3 lattice of overlapping solid spheres (seeded; lognormal radii, mean 8, sd 2
  voxels) added until porosity 0.22, isolated pores removed; body force 1e-6 along z;
  tau = 1 (nu = 1/6); MRT preset 1; periodic in x, y, z; FP64 storage and collision
  (the plain drop-in form).  MLUPS counts fluid nodes only, as the reference's
  benchmark does (singlephase_3D/0.src/Main.F90:471).

  value : device-resident timed region (CUDA events), K steps.  The PDF state
          (2.5 GB) is far larger than L2, so no flush is needed between steps.
  e2e   : the same metric through the C ABI with host buffers: each timed round
          uploads the full state from pinned host memory, runs R steps, and reads the
          monitor result (per-slice flow rate) back to the host.
  --impl reference : the reference algorithm's CPU implementation (the C++
          restatement, all host threads) on the same workload, bounded sample.
Under torchrun (N>1) every rank runs an independent replica (the lattice is not
sharded); value = total fluid-node updates of all ranks / max time over ranks.  The
per-form measurements, the convergence study and the CPU baseline belong to the N=1 line
and are left out at N>1.

Other forms and workloads: --precision 0-4 (FP64, FP32, FP16 deviations, FP64 storage with
the double-word collision, double-word storage), --workload c1 (tube drainage), c3
(packing drainage; --c3-study for saturation and phi error against FP64), c4 (ensemble to
steady state), c5 (learned warm start), c5net (one training step of its network).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("mf-lbm_gb300", "oracle"):
    sys.path.insert(0, os.path.join(ROOT, sub))

import numpy as np  # noqa: E402

METRIC = "MLUPS (% HBM roofline); time-to-converged permeability, mixed vs FP64 plain"
BYTES_PER_LU = {0: 19 * 8 * 2 + 1, 1: 19 * 4 * 2 + 1, 2: 19 * 2 * 2 + 1, 3: 19 * 8 * 2 + 1, 4: 19 * 8 * 2 + 1}
# multiphase collision: 2x19 PDFs read and written, phi written, cn_x/y/z + c_norm + curv read, wall
BYTES_PER_LU_MP = {0: 2 * 19 * 8 * 2 + 8 + 5 * 8 + 1, 1: 2 * 19 * 4 * 2 + 4 + 4 * 4 + 1,
                   3: 2 * 19 * 8 * 2 + 8 + 5 * 8 + 1, 4: 2 * 19 * 8 * 2 + 8 + 5 * 8 + 1}
# 1: the FP32 collision computes the node's curvature from the normal records around it
# (the workloads here use the fluid-cell gradient lists), so it reads its own 16-byte
# record and no curv value; the neighbours' records are other nodes' own records
# 3: FP64 storage, collision in double-word (two-FP32) arithmetic on the FP32 pipe;
# 4: double-word storage (hi + lo FP32 pair, 8 bytes) and the double-word collision
DTYPE = {0: "f64", 1: "f32", 2: "f16", 3: "f64ff", 4: "ff"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c3", "c4", "c5", "c5net"],
                    help="c2: singlephase packing permeability (default); c1: multiphase tube drainage; "
                         "c3: multiphase packing drainage; c4: batched permeability ensemble to steady state; "
                         "c5: learned warm start (train the network, then A/B against runs from rest)")
    ap.add_argument("--samples", type=int, default=256, help="c4: ensemble size")
    ap.add_argument("--train", type=int, default=200, help="c5: training samples")
    ap.add_argument("--test", type=int, default=6, help="c5: held-out samples")
    ap.add_argument("--epochs", type=int, default=8, help="c5: training epochs")
    ap.add_argument("--n5", type=int, default=128, help="c5: sample edge")
    ap.add_argument("--c5-data-tol", type=float, default=1e-7, help="c5: convergence of the training solutions")
    ap.add_argument("--c3-study", action="store_true",
                    help="c3: FP64 and FP32 forms over --c3-steps steps, saturation every 500 steps, phi L1 error")
    ap.add_argument("--c3-steps", type=int, default=20000)
    ap.add_argument("--c3-ff", action="store_true", help="c3 study: also the double-word form (FP64 storage)")
    ap.add_argument("--c3-fp64-steps", type=int, default=0,
                    help="c3 study: steps of the FP64 run (0: --c3-steps); the phi L1 error is taken there")
    ap.add_argument("--c4-fp64", action="store_true", help="c4: also run the FP64 ensemble for per-sample k errors")
    ap.add_argument("--c4-ff", action="store_true",
                    help="c4: also run the double-word storage ensemble (FP64-grade k) on every sample")
    ap.add_argument("--c4-fp64-samples", type=int, default=0,
                    help="c4: run the FP64 reference on the first K samples only (0: all)")
    ap.add_argument("--n", type=int, default=256, help="lattice edge (c2) / cross-section (c3)")
    ap.add_argument("--porosity", type=float, default=0.22)
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="0 FP64, 1 FP32 (deviations for singlephase), 2 FP16 deviations, "
                         "3 FP64 storage with the double-word collision, 4 double-word storage and collision "
                         "(FP16 singlephase only)")
    ap.add_argument("--e2e-round", type=int, default=100, help="steps per e2e round")
    ap.add_argument("--cpu-sample-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="c2: skip the per-form measurement (FP64 storage + double-word collision, double-word "
                         "storage, FP32 and FP16 deviations) that the default line carries under `forms`")
    ap.add_argument("--no-convergence", action="store_true",
                    help="skip the time-to-steady permeability study (singlephase workload only)")
    ap.add_argument("--conv-tol", type=float, default=1e-7)
    ap.add_argument("--open-z", action="store_true",
                    help="c2: the packing between 16-layer inlet and outlet buffers with a velocity inlet "
                         "(mean 1e-4) and a convective outlet instead of periodic z with a body force "
                         "(skips the per-form and convergence studies)")
    ap.add_argument("--layout", type=int, default=0, choices=[0, 1, 2],
                    help="PDF storage: 0 auto, 1 dense planes, 2 fluid list (fluid nodes + link slots)")
    return ap.parse_args()


def max_over_ranks(x, dist=None, device="cpu"):
    """The largest of x over all ranks of the process group (x itself without one): the
    slowest rank's time is the job's time.  device: "cuda" under NCCL, "cpu" under gloo."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(nodes_per_rank, steps, world, seconds):
    """Fluid-node updates of all ranks (independent replicas of the same workload) per
    second of the slowest rank, in millions."""
    return world * nodes_per_rank * steps / seconds / 1e6


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(args, device=0):
    from mflbm import workloads
    if args.workload == "c1":
        case = workloads.tube_drainage(device=device, precision=args.precision)
        desc = ("multiphase colour-gradient drainage, 64x64x160 tube (r=30) with a sphere (r=14), phi=+1 for z<28, "
                f"tau=1, gamma=0.01, theta=45, inlet velocity 1e-4, convective outlet, {DTYPE[args.precision]}")
    elif args.workload == "c3":
        case = workloads.packing_drainage(nxy=args.n, nzp=args.n, buffer=32, device=device, precision=args.precision)
        desc = (f"multiphase drainage, {args.n}^2x{args.n} sphere packing porosity 0.22 + 32-layer buffers, "
                f"inlet velocity 5e-5, gamma=0.01, theta=30, {DTYPE[args.precision]}")
    elif args.open_z:
        case = workloads.packing_throughflow(n=args.n, porosity=args.porosity, precision=args.precision,
                                             device=device)
        desc = (f"singlephase through-flow, {args.n}^3 sphere packing porosity {args.porosity} between 16-layer "
                "inlet and outlet buffers, walls in x and y, velocity inlet 1e-4, convective outlet, tau=1, "
                "MRT preset 1")
    else:
        case = workloads.packing_permeability(n=args.n, porosity=args.porosity, precision=args.precision,
                                              device=device)
        desc = (f"singlephase permeability, {args.n}^3 sphere packing porosity {args.porosity} "
                "(seeded lognormal radii mean 8 sd 2, isolated pores removed), periodic xyz, F_z=1e-6, tau=1, "
                "MRT preset 1")
    case["params"].layout = args.layout
    return case, desc


def config_of(args, case, desc):
    """The workload description both arms print (the same dict for --impl ours and
    --impl reference): what was run, not what was measured."""
    p = case["params"]
    elt = 8 if args.precision in (0, 3, 4) else (4 if args.precision == 1 else 2)
    state_bytes = (2 if p.multiphase else 1) * 19 * elt * case["pore"]
    return {"workload": desc, "lattice": [p.nx, p.ny, p.nz], "fluid_nodes": case["pore"],
            "l2": f"PDF state of the fluid nodes {state_bytes / 1e9:.2f} GB vs 129 MB L2"
                  + (": no flush needed" if state_bytes > 4 * 129e6 else ": inputs smaller than L2")
                  + "; the library's fluid-list sweeps alternate direction, so each starts on the slots the "
                    "previous step left in L2 (as in every run of the library)"}


def setup(sim, case):
    sim.set_geometry(case["walls"], case.get("solid"), case.get("fluid"), case.get("w_in"))
    if case["params"].multiphase:
        sim.init_equilibrium(case["phi"])
        sim.color_gradient()
    else:
        sim.init_equilibrium()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(case, steps):
    """The CPU restatement of the reference (all host threads) on the same workload."""
    import pyoracle
    p, pore = case["params"], case["pore"]
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(p, variant="fast", threads=threads)
    setup(o, case)
    o.run(1, 2)  # first-touch and warm-up
    t0 = time.perf_counter()
    o.run(3, steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": pore * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the full {p.nx}x{p.ny}x{p.nz} workload ({pore} fluid nodes), "
                      f"C++ restatement -O3, OpenMP {threads} threads, {dt:.2f} s"}


def hbm_peak():
    """Measured copy bandwidth of the GB300s, else the stated fallback."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"


def stored_traffic(prec, layout, multiphase, pore):
    """DRAM bytes per launch of the collision sweep from the committed ncu captures
    (profiles/sp_collide_traffic.json, profiles/mp_collide_traffic.json: bytes per fluid
    node x the fluid nodes here)."""
    tf = os.path.join(ROOT, "profiles", "mp_collide_traffic.json" if multiphase else "sp_collide_traffic.json")
    if not os.path.exists(tf):
        return None
    try:
        t = json.load(open(tf))
    except Exception:
        return None
    # singlephase FP64 storage with the double-word collision moves the FP64 form's bytes
    key = f"{DTYPE[prec if multiphase or prec != 3 else 0]}_{layout}"
    return t[key] * pore if key in t else None


def roofline_of(prof, pore, prec, multiphase, layout, hbm, peak_src):
    """Roofline of the collision sweep: algorithmic bytes per launch / the average
    event-timed launch duration, against the measured copy peak."""
    avg_s = prof["collide_ms"] / max(1, prof["collide_launches"]) / 1e3
    bpl = BYTES_PER_LU_MP[prec] if multiphase else BYTES_PER_LU[prec]
    achieved = pore * bpl / avg_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": stored_traffic(prec, layout, multiphase, pore), "traffic_source": "ncu capture "
            f"(profiles/{'mp' if multiphase else 'sp'}_collide_traffic.json, bytes per fluid node x fluid nodes)", "bytes_per_lu": bpl,
            "peak_source": peak_src, "avg_launch_ms": avg_s * 1e3, "launches_timed": prof["collide_launches"]}


def measure_form(args, case, prec, hbm, peak_src):
    """One storage form of the singlephase workload on the same geometry, timed exactly
    like the headline: per-step launches with events around every collision sweep,
    --steps steps after --warmup, then graph replay of the same number of steps."""
    import copy
    from mflbm import Solver
    p = copy.copy(case["params"])
    p.precision = prec
    pore = case["pore"]
    with Solver(p) as sim:
        setup(sim, case)
        sim.run(1, max(args.warmup, 3))
        sim.synchronize()
        sim.set_profiling(True)
        sim.run(args.warmup + 1, args.steps)
        prof = sim.get_profile()
        sim.set_profiling(False)
        sim.run(args.warmup + 1 + args.steps, args.steps)
        gprof = sim.get_profile()
        layout = {1: "dense", 2: "list"}.get(sim.layout, "dense")
    total_s = prof["region_ms"] / 1e3
    roof = roofline_of(prof, pore, prec, False, layout, hbm, peak_src)
    return {"value": pore * args.steps / total_s / 1e6, "unit": "MLUPS", "ms_per_step": 1e3 * total_s / args.steps,
            "graph_replay_mlups": pore * args.steps / (gprof["region_ms"] / 1e3) / 1e6, "layout": layout,
            "gpu_launches": prof["kernel_launches"], "roofline": roof}


def convergence_study(args, case, device):
    """Time-to-steady permeability of each storage form on the same geometry.

    Every form starts from rest and runs until |du|/u < tol between checks 100 steps
    apart (the monitor_timer role); k = nu * u_mean / F_z.  Wall time is the host clock
    around the whole loop (graph-replayed steps plus the FP64 monitor reductions and
    their read-back).  Errors are relative to the FP64 form.  A form that stops at another
    step count than FP64 also reports its k after exactly FP64's step count
    (k_rel_err_at_fp64_steps): the error of its storage precision alone."""
    import copy
    from mflbm import Solver
    from mflbm.permeability import mean_velocity, permeability, run_to_steady
    out = {"tol": args.conv_tol, "check_every": 100, "forms": {}}
    base = None
    for prec in (0, 3, 4, 1, 2):
        p = copy.copy(case["params"])
        p.precision = prec
        with Solver(p) as sim:
            sim.set_geometry(case["walls"])
            sim.init_equilibrium()
            sim.run(1, 100)          # graph capture outside the clock
            sim.init_equilibrium()
            sim.synchronize()
            # FP16's 11-bit significand puts its noise floor above 1e-7: it runs to 1e-5
            tol = args.conv_tol if prec != 2 else max(args.conv_tol, 1e-5)
            r = run_to_steady(sim, p, check_every=100, tol=tol, max_steps=200000)
        form = {"k": r.k, "steps": r.steps, "seconds": r.seconds, "converged": r.converged, "status": r.status,
                "tol": tol}
        if prec == 0:
            base = r
        else:
            form["k_rel_err_vs_fp64"] = abs(r.k - base.k) / abs(base.k)
            form["wall_time_ratio_fp64_over_form"] = base.seconds / r.seconds
            if r.steps != base.steps and base.converged:
                # the storage precision alone: k after exactly the FP64 run's step count,
                # so that where the stopping rule fired does not enter the error
                with Solver(p) as sim:
                    sim.set_geometry(case["walls"])
                    sim.init_equilibrium()
                    sim.run(1, base.steps)
                    u, _ = mean_velocity(sim, p.nx, p.ny, p.nz)
                k_eq = permeability(u, p.la_nu1, p.force_z)
                form["k_rel_err_at_fp64_steps"] = abs(k_eq - base.k) / abs(base.k)
        out["forms"][DTYPE[prec]] = form
    return out


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    args.precision = 0
    case, desc = workload(args)
    p, pore = case["params"], case["pore"]
    steps = max(1, args.steps)
    import pyoracle
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(p, variant="fast", threads=threads)
    setup(o, case)
    o.run(1, max(1, args.warmup))
    t0 = time.perf_counter()
    o.run(1 + max(1, args.warmup), steps)
    dt = time.perf_counter() - t0
    o.close()
    v = pore * steps / dt / 1e6
    line = {"metric": METRIC, "value": v, "unit": "MLUPS", "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_of(args, case, desc),
            "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": threads, "kind": "port",
                             "sample": f"{steps} steps of the full workload after {max(1, args.warmup)} warm-up "
                                       f"steps, {dt:.2f} s; the Fortran reference cannot be built (no Fortran "
                                       "compiler or MPI), so its C++ restatement runs instead, OpenMP "
                                       f"{threads} threads"},
            "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def ensemble_study(args):
    """c4: every sample of the ensemble from rest to |du|/u < tol (checks every 100
    steps), converged samples leaving the sweep; value = fluid-node updates per second,
    samples/s in config.  With --c4-fp64 the FP64 ensemble of the same seeds gives the
    per-sample permeability error of the storage form; with --c4-ff the double-word storage
    ensemble (k within ~1e-10 of FP64 at 4-5x its rate) gives it for every sample, and its own
    error against FP64 on the FP64 subset."""
    from mflbm import workloads
    world, rank, local = dist_env()
    prec = args.precision if args.precision else 1
    t0 = time.perf_counter()
    case = workloads.packing_ensemble(n_samples=args.samples, precision=prec, device=local,
                                      workers=min(16, os.cpu_count() or 1))
    gen_s = time.perf_counter() - t0
    import torch
    from mflbm.ensemble import Ensemble, run_to_steady, tune_cached
    torch.cuda.set_device(local)
    res = {}
    k64 = args.c4_fp64_samples if args.c4_fp64_samples > 0 else args.samples
    for pr in [prec] + ([4] if args.c4_ff else []) + ([0] if args.c4_fp64 else []):
        case["params"].precision = pr
        samples, nf = (case["samples"][:k64], case["nf"][:k64]) if pr == 0 else (case["samples"], case["nf"])
        with Ensemble(case["params"], samples) as ens:
            tune = tune_cached(ens, None, steps=6)
            ens.init()
            torch.cuda.synchronize()
            with ClockSampler(local) as clk:
                r = run_to_steady(ens, nf, check_every=100, tol=args.conv_tol, max_steps=200000)
            res[pr] = (r, tune, clk.summary(), ens.info())
    r, tune, clocks, info = res[prec]
    line = {"metric": METRIC, "value": r.fluid_updates / r.seconds / 1e6, "unit": "MLUPS", "n_gpus": 1,
            "steps": int(r.steps.max()), "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[prec], "data": "synthetic",
            "config": {"workload": f"batched permeability ensemble: {args.samples} sphere packings, edges U[48,160], "
                                   "porosity U[0.15,0.35], F_z=1e-6, tau=1, MRT preset 1, periodic xyz, "
                                   f"to |du|/u<{args.conv_tol} every 100 steps",
                       "samples": args.samples, "samples_per_s": args.samples / r.seconds,
                       "wall_s": r.seconds, "converged": int(r.converged.sum()),
                       "total_nodes": int(sum(e ** 3 for e in case["edges"])), "fluid_nodes": int(case["nf"].sum()),
                       "fluid_updates": r.fluid_updates, "generate_s": gen_s, "launch": tune.get("chosen"),
                       "tuner": tune.get("candidates")},
            "clocks": clocks, "gpu_launches": None}
    per = []
    for i in range(args.samples):
        row = {"edge": int(case["edges"][i]), "porosity": float(case["porosity"][i]), "steps": int(r.steps[i]),
               "k": float(r.k[i])}
        if args.c4_fp64 and i < k64:
            row.update(steps_fp64=int(res[0][0].steps[i]), k_fp64=float(res[0][0].k[i]))
        if args.c4_ff:
            row.update(steps_ff=int(res[4][0].steps[i]), k_ff=float(res[4][0].k[i]))
        per.append(row)
    line["config"]["per_sample"] = per
    if args.c4_fp64:
        r64 = res[0][0]
        err = np.abs(r.k[:k64] - r64.k) / np.abs(r64.k)
        line["config"]["k_rel_err_vs_fp64"] = {"max": float(err.max()), "median": float(np.median(err)),
                                               "samples_compared": int(k64)}
        line["config"]["fp64_wall_s"] = r64.seconds
        line["config"]["fp64_samples_per_s"] = k64 / r64.seconds
    if args.c4_ff:
        rff = res[4][0]
        err = np.abs(r.k - rff.k) / np.abs(rff.k)
        line["config"]["k_rel_err_vs_ff"] = {"max": float(err.max()), "median": float(np.median(err)),
                                             "p99": float(np.quantile(err, 0.99)),
                                             "above_1e-3": int((err > 1e-3).sum()), "samples_compared": args.samples}
        line["config"]["ff_wall_s"] = rff.seconds
        line["config"]["ff_samples_per_s"] = args.samples / rff.seconds
        line["config"]["ff_converged"] = int(rff.converged.sum())
        line["config"]["ff_launch"] = res[4][1].get("chosen")
        if args.c4_fp64:
            e2 = np.abs(rff.k[:k64] - res[0][0].k) / np.abs(res[0][0].k)
            line["config"]["ff_k_rel_err_vs_fp64"] = {"max": float(e2.max()), "samples_compared": int(k64)}
    print(json.dumps(line), flush=True)
    return 0


def warmstart_study(args):
    """c5: train the warm-start network on LBM solutions the solver produces (FP32
    deviation form to |du|/u < --c5-data-tol), then on held-out samples compare runs to 1e-7 from
    rest and from the prediction (FP64 and FP32), wall time including inference.  "rest"
    is the reference's start (equilibrium at rest, BGK weights); the warm start places the
    predicted velocity and density on the rest state of the MRT collision with consistent
    bounce-back slots, and the "mrt_rest" rows (that rest state at the sample's mean
    density, no prediction) separate the two contributions."""
    from mflbm import warmstart as ws
    n = args.n5
    t0 = time.perf_counter()
    workers = min(16, os.cpu_count() or 1)
    train_s = ws.make_samples(n, args.train, seed=101, workers=workers)
    test_s = ws.make_samples(n, args.test, seed=202, workers=workers)
    gen_s = time.perf_counter() - t0
    import torch
    torch.cuda.set_device(0)
    nu, fz = 1.0 / 6.0, 1e-6
    xs, ys, ms = [], [], []
    t0 = time.perf_counter()
    data_lu = 0
    for wg, x in train_s:
        r, mac, _ = ws.solve(wg, precision=1, tol=args.c5_data_tol, nu=nu, fz=fz)
        data_lu += int((wg == 0).sum()) * r.steps
        xs.append(torch.from_numpy(x).cuda().to(torch.bfloat16))
        ys.append(torch.from_numpy(ws.target_from_macro(mac, nu, fz, ws.mean_density(wg))).cuda())
        ms.append(torch.from_numpy((wg == 0).reshape(-1).astype(np.float32)).cuda())
    data_s = time.perf_counter() - t0
    net = ws.Net(n, seed=7)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = ws.train(net, xs, ys, ms, epochs=args.epochs, lr=1e-3, lr_end=1e-4, seed=3)
    torch.cuda.synchronize()
    train_s_time = time.perf_counter() - t0
    rows = []
    for wg, x in test_s:
        ref = ws.solve(wg, precision=0, tol=args.conv_tol, nu=nu, fz=fz)[0]
        r32 = ws.solve(wg, precision=1, tol=args.conv_tol, nu=nu, fz=fz)[0]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        net.forward(torch.from_numpy(x).cuda().to(torch.bfloat16))
        out = net.out.cpu().numpy()
        u = ws.velocity_from_output(out, n, nu, fz, wg)
        rho = ws.density_from_output(out, n, wg, ws.mean_density(wg))
        infer = time.perf_counter() - t1
        w64, _, set64 = ws.solve(wg, precision=0, tol=args.conv_tol, init_u=u, init_rho=rho, nu=nu, fz=fz)
        w32, _, set32 = ws.solve(wg, precision=1, tol=args.conv_tol, init_u=u, init_rho=rho, nu=nu, fz=fz)
        # the double-word storage form: FP64-grade k (about 1e-10 of FP64) on the FP32 pipe
        rff = ws.solve(wg, precision=4, tol=args.conv_tol, nu=nu, fz=fz)[0]
        wff, _, setff = ws.solve(wg, precision=4, tol=args.conv_tol, init_u=u, init_rho=rho, nu=nu, fz=fz)
        # ablation: the MRT rest state without the predicted velocity
        b32, _, setb = ws.solve(wg, precision=1, tol=args.conv_tol, rest_base=True, nu=nu, fz=fz)
        k0 = nu * float(np.mean(u[2])) / fz
        rows.append({"porosity": float((wg == 0).mean()), "k_fp64_rest": ref.k, "steps_fp64_rest": ref.steps,
                     "s_fp64_rest": ref.seconds, "steps_fp32_rest": r32.steps, "s_fp32_rest": r32.seconds,
                     "k_err_fp32_rest": abs(r32.k - ref.k) / ref.k,
                     "steps_fp64_warm": w64.steps, "s_fp64_warm": w64.seconds + infer + set64,
                     "k_err_fp64_warm": abs(w64.k - ref.k) / ref.k,
                     "steps_fp32_warm": w32.steps, "s_fp32_warm": w32.seconds + infer + set32,
                     "k_err_fp32_warm": abs(w32.k - ref.k) / ref.k,
                     "steps_ff_rest": rff.steps, "s_ff_rest": rff.seconds, "k_err_ff_rest": abs(rff.k - ref.k) / ref.k,
                     "steps_ff_warm": wff.steps, "s_ff_warm": wff.seconds + infer + setff,
                     "k_err_ff_warm": abs(wff.k - ref.k) / ref.k,
                     "steps_fp32_mrt_rest": b32.steps, "s_fp32_mrt_rest": b32.seconds + setb,
                     "k_err_fp32_mrt_rest": abs(b32.k - ref.k) / ref.k,
                     "k_err_prediction_only": abs(k0 - ref.k) / ref.k, "inference_s": infer})
    def agg(key, f=np.mean):
        return float(f([r[key] for r in rows]))
    line = {"metric": METRIC, "value": agg("s_fp64_rest") / agg("s_fp32_warm"), "unit": "x wall-time speed-up "
            "(FP64 from rest / FP32 + warm start, to the same tolerance)", "n_gpus": 1, "steps": None, "warmup": 0,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32",
            "data": "synthetic",
            "config": {"workload": f"learned warm start: {n}^3 sphere packings, porosity U[0.15,0.35], F_z=1e-6, tau=1, "
                                   f"{args.train} training samples (FP32 LBM to {args.c5_data_tol}), {args.test} held-out samples, "
                                   f"convergence {args.conv_tol} every 100 steps",
                       "generate_s": gen_s, "training_data_s": data_s, "training_data_mlups": data_lu / data_s / 1e6,
                       "train_s": train_s_time, "epochs": args.epochs, "loss_per_epoch": hist,
                       "mean": {k: agg(k) for k in rows[0]}, "max_k_err_fp32_warm": agg("k_err_fp32_warm", np.max),
                       "max_k_err_fp64_warm": agg("k_err_fp64_warm", np.max),
                       "steps_ratio_fp64_rest_over_warm": agg("steps_fp64_rest") / agg("steps_fp64_warm"),
                       "steps_ratio_fp32_mrt_rest_over_fp32_warm": agg("steps_fp32_mrt_rest") / agg("steps_fp32_warm"),
                       "time_ratio_fp64_rest_over_fp64_warm": agg("s_fp64_rest") / agg("s_fp64_warm"),
                       "time_ratio_fp64_rest_over_fp32_rest": agg("s_fp64_rest") / agg("s_fp32_rest"),
                       "time_ratio_fp64_rest_over_ff_warm": agg("s_fp64_rest") / agg("s_ff_warm"),
                       "max_k_err_ff_warm": agg("k_err_ff_warm", np.max),
                       "samples": rows}}
    print(json.dumps(line), flush=True)
    return 0


def network_step_bench(args):
    """c5net: one training step of the warm-start network (forward, masked MSE, backward,
    Adam) on one --n5^3 sample, K steps timed with CUDA events on the network's stream.
    The roofline is that of the largest tcgen05 GEMM (the forward convolution of the last
    decoder level, n^3 x 1344 x 16), timed alone on the same stream: HBM-bound, its
    algorithmic bytes are the im2col matrix, the weights and the FP32 output."""
    import torch
    from mflbm import _capi, geometry
    from mflbm import warmstart as ws
    torch.cuda.set_device(0)
    n = args.n5
    wg = geometry.sphere_packing((n, n, n), 0.25, mean_r=8.0, sd_r=2.0, seed=11)
    x = torch.from_numpy(ws.features(wg)).cuda().to(torch.bfloat16)
    rng = np.random.default_rng(5)
    target = torch.from_numpy(0.1 * rng.normal(size=(n ** 3, ws.NTARGET)).astype(np.float32)).cuda()
    mask = torch.from_numpy((wg == 0).reshape(-1).astype(np.float32)).cuda()
    net = ws.Net(n, seed=7)
    stream = torch.cuda.current_stream()

    def step():
        net.forward(x)
        net.loss_grad(target, mask)
        net.backward()
        net.adam(lr=1e-4)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    c0 = net.calls
    step()
    calls_per_step = net.calls - c0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    net.check_err()
    # the largest forward GEMM alone
    name = "d1"
    cin, cout = next((s[1], s[2]) for s in net.specs if s[0] == name)
    kp, nv = ws._kp(cin), n ** 3
    L, p, s = net.lib, net._p, net.stream
    reps = 20
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(reps):
        rc = L.mflbm_nn_gemm_bf16(p(net.col[name]), kp, p(net.Wb[name]), kp, p(net.acc), cout, nv, cout, kp, 0,
                                  p(net.err), s)
        if rc:
            raise _capi.MflbmError(rc, "gemm")
    g1.record(stream)
    torch.cuda.synchronize()
    net.check_err()
    gemm_s = g0.elapsed_time(g1) / reps / 1e3
    gbytes = nv * kp * 2 + cout * kp * 2 + nv * cout * 4
    gflop = 2.0 * nv * kp * cout
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    splitk = len(net.specs)     # one split-K weight-gradient GEMM (two launches) per layer
    line = {"metric": "warm-start network training steps per second", "value": 1e3 / ms, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic",
            "config": {"workload": f"warm-start network training step, one {n}^3 sample, channels {net.c}, "
                                   f"forward + masked MSE + backward + Adam",
                       "l2": "activations and im2col matrices (GBs) far above the 129 MB L2: no flush needed"},
            "roofline": {"bound": "hbm", "kernel": f"k_gemm_bf16 ({nv} x {kp} x {cout}, layer {name} forward)",
                         "achieved": gbytes / gemm_s / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": gbytes / gemm_s / 1e9 / hbm, "traffic": None,
                         "tensor_tflops": gflop / gemm_s / 1e12, "tensor_frac": gflop / gemm_s / 1e12 / bf16,
                         "avg_launch_ms": gemm_s * 1e3, "peak_source": "measured (MEASURED_PEAKS.json)"},
            "gpu_launches": (calls_per_step + splitk) * args.steps, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def drainage_study(args):
    """c3 at scale: the FP64 form, the FP32 mixed form and (--c3-ff) the FP64-grade
    double-word form of the same drainage from the same initial state; saturation (FP64
    device sums) every 500 steps and, at the end, the phi-field L1 error of each form against
    FP64 over the interior nodes."""
    import copy
    import torch
    from mflbm import Solver, workloads
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    case = workloads.packing_drainage(nxy=args.n, nzp=args.n, buffer=32, precision=0, gpu_preprocess=True)
    gen_s = time.perf_counter() - t0
    res = {}
    every = 500
    n64 = args.c3_fp64_steps if args.c3_fp64_steps > 0 else args.c3_steps
    for prec in (0, 1) + ((3,) if args.c3_ff else ()):
        p = copy.copy(case["params"])
        p.precision = prec
        nsteps = n64 if prec in (0, 3) else args.c3_steps
        with Solver(p) as sim:
            setup(sim, case)
            sim.run(1, 2)
            setup(sim, case)
            sim.synchronize()
            sat = []
            run_s = 0.0
            done = 0
            phi_cmp = None
            while done < nsteps:
                k = min(every, nsteps - done, n64 - done if done < n64 else nsteps)
                t1 = time.perf_counter()
                sim.run(1 + done, k)
                sim.synchronize()
                run_s += time.perf_counter() - t1
                done += k
                v1, v2 = sim.saturation()
                sat.append((done, v1 / (v1 + v2)))
                if done == n64:
                    phi_cmp = sim.macro()["phi"][4:-4, 4:-4, 4:-4].copy()
        res[prec] = (sat, phi_cmp, run_s, nsteps)
    fluid = case["walls"][2:-2, 2:-2, 2:-2] == 0
    dphi = np.abs(res[1][1] - res[0][1])[fluid]
    s64 = np.array([x[1] for x in res[0][0]])
    s32 = np.array([x[1] for x in res[1][0]])
    m = min(len(s64), len(s32))
    pore = case["pore"]
    line = {"metric": METRIC, "value": pore * args.c3_steps / res[1][2] / 1e6, "unit": "MLUPS", "n_gpus": 1,
            "steps": args.c3_steps, "warmup": 2, "ms_per_step": 1e3 * res[1][2] / args.c3_steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"multiphase drainage, {args.n}^2x{args.n} sphere packing porosity 0.22 + 32-layer "
                                   "buffers, inlet velocity 5e-5, gamma=0.01, theta=30; FP32 mixed form vs FP64",
                       "lattice": [case["params"].nx, case["params"].ny, case["params"].nz], "fluid_nodes": pore,
                       "generate_s": gen_s, "fp64_mlups": pore * res[0][3] / res[0][2] / 1e6, "fp64_steps": res[0][3],
                       "phi_compared_at_step": n64,
                       "fp32_mlups": pore * args.c3_steps / res[1][2] / 1e6,
                       "wall_s": {"fp64": res[0][2], "fp32": res[1][2]},
                       "saturation_every_500": {"step": [x[0] for x in res[1][0]], "fp64": s64.tolist(),
                                                "fp32": s32.tolist()},
                       "max_abs_saturation_diff": float(np.abs(s64[:m] - s32[:m]).max()),
                       "phi_L1_fp32_vs_fp64": float(dphi.mean()), "phi_max_abs_diff": float(dphi.max()),
                       "timed": "host clock around graph-replayed runs of 500 steps, saturation sums outside"}}
    if 3 in res:
        dff = np.abs(res[3][1] - res[0][1])[fluid]
        sff = np.array([x[1] for x in res[3][0]])
        line["config"]["double_word"] = {
            "mlups": pore * res[3][3] / res[3][2] / 1e6, "wall_s": res[3][2], "steps": res[3][3],
            "saturation_every_500": sff.tolist(),
            "max_abs_saturation_diff": float(np.abs(s64[:len(sff)] - sff).max()),
            "phi_L1_vs_fp64": float(dff.mean()), "phi_max_abs_diff": float(dff.max())}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "c3" and args.c3_study:
        return drainage_study(args)
    if args.workload == "c4":
        return ensemble_study(args)
    if args.workload == "c5":
        return warmstart_study(args)
    if args.workload == "c5net":
        return network_step_bench(args)
    world, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from mflbm import Solver
    case, desc = workload(args, device=local)
    p, pore = case["params"], case["pore"]
    hbm, peak_src = hbm_peak()
    sim = Solver(p)
    setup(sim, case)
    # warm-up (graph capture, first touch)
    sim.run(1, max(args.warmup, 3))
    sim.synchronize()

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timed region: per-step launches with CUDA events around every
    # collision sweep (profiling mode), the region bracketed by events on the same stream.
    # The clock sampler runs from here to the end of the per-form measurements below.
    barrier()
    clk = ClockSampler(local).__enter__()
    sim.set_profiling(True)
    sim.run(args.warmup + 1, args.steps)
    prof = sim.get_profile()   # synchronises the context stream
    total_s = max_over_ranks(prof["region_ms"] / 1e3, dist, "cuda")
    value = whole_job_mlups(pore, args.steps, world, total_s)

    # ---- graph-replayed region (the production path, no per-kernel events)
    barrier()
    sim.set_profiling(False)
    sim.run(args.warmup + 1 + args.steps, args.steps)
    gprof = sim.get_profile()
    graph_mlups = pore * args.steps / (gprof["region_ms"] / 1e3) / 1e6

    # ---- e2e through the C ABI with host buffers
    e2e = None
    try:
        rs = args.e2e_round
        state = sim.download_state()
        pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in state.items()}
        barrier()
        t0 = time.perf_counter()
        nround = max(1, args.steps // rs)
        for r in range(nround):
            sim.upload_state(pinned["f"], pinned.get("g"), pinned.get("phi"), pinned.get("f_convec"),
                             pinned.get("g_convec"), pinned.get("phi_convec"))
            sim.run(1, rs)           # the uploaded state follows an even step
            prof_z, scal, status = sim.monitor()
        e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
        h2d = sum(v.nbytes for k, v in pinned.items() if k != "f_convec" or p.outlet_bc == 1)
        d2h = (7 if p.multiphase else 2) * p.nz * 8 + 3 * 8 + 4
        e2e = {"value": whole_job_mlups(pore, rs * nround, world, e2e_s), "unit": "MLUPS",
               "h2d_bytes_per_step": h2d / rs, "d2h_bytes_per_step": d2h / rs,
               "round": f"upload full state (pinned) + {rs} steps + monitor readback"}
    except Exception as exc:  # keep the device-timed number even if e2e fails
        e2e = {"value": None, "unit": "MLUPS", "error": str(exc)[:200]}

    layout = {1: "dense", 2: "list"}.get(sim.layout, "dense")
    sim.close()
    roof = roofline_of(prof, pore, args.precision, bool(p.multiphase), layout, hbm, peak_src)
    mp_kernel = {1: "k_mp_step (curvature fused in)", 3: "k_mp_step_ff", 4: "k_mp_step_ff"}.get(args.precision,
                                                                                              "k_mp_step")
    roof["kernel"] = mp_kernel if p.multiphase else ("k_sp_list" if layout == "list" else "k_sp_step")

    # ---- every other storage form of the singlephase workload, measured the same way
    forms = None
    if rank == 0 and world == 1 and args.workload == "c2" and not args.no_forms and not args.open_z:
        forms = {}
        for prec in (0, 3, 4, 1, 2):
            if prec == args.precision:
                continue
            try:
                forms[DTYPE[prec]] = measure_form(args, case, prec, hbm, peak_src)
            except Exception as exc:
                forms[DTYPE[prec]] = {"error": str(exc)[:200]}
    clk.__exit__(None, None, None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:   # the CPU baseline: N = 1 only
        try:
            cpu = cpu_baseline(case, args.cpu_sample_steps)
        except Exception as exc:
            cpu = {"value": None, "unit": "MLUPS", "error": str(exc)[:200]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.precision],
            "data": "synthetic",
            "config": config_of(args, case, desc),
            "detail": {"replicas": world, "layout": layout,
                       "timed_path": "per-step launches with events around each collision sweep",
                       "graph_replay_mlups": graph_mlups},
            "e2e": e2e,
            "gpu_launches": prof["kernel_launches"],
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        if forms is not None:
            line["forms"] = forms
    if rank == 0 and world == 1 and args.workload == "c2" and not args.no_convergence and not args.open_z:
        try:
            line["convergence"] = convergence_study(args, case, local)
        except Exception as exc:
            line["convergence"] = {"error": str(exc)[:200]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
