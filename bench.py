"""Benchmark: zone-updates/s of the FD WENO-CT MHD step on the 3D blast, 256^3, FP32.

One "step" is one time step of astronomix's finite-difference MHD scheme
(CFL dt, five SSPRK(5,4) stages of WENO fluxes in x, y, z + constrained
transport, positivity floors) over the whole 256^3 periodic grid, launched
through the C ABI.  The blast is synthetic: rho = 1, v = 0, p = 10 inside
r < 0.1 of the centre and 0.1 outside, B = (1, 1, 0)/sqrt 2 with face fields
from initialize_interface_fields, gamma 5/3, C_cfl 1.5 (no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: each timed step is bracketed by CUDA events on the launching stream;
the state (738 MB) and the step's workspace (3.4 GB) are far larger than the
L2 cache (129 MB), so no flush is needed between steps.  The line also
carries: the end-to-end number through the C ABI with pinned host buffers
(H2D + step + D2H per step); the per-kernel launch durations (CUDA events
after every launch) and the roofline of the dominant kernel, k_weno; the
FP64 throughput of the same kernels and the FP32-vs-FP64 relative L1
density error of a full run to t_end = 0.02; the CPU baseline (the oracle,
a NumPy restatement of the reference, on a bounded sample); and the
secondary workloads (Orszag-Tang 512^2 FV, the reference's published blast
workloads, the batched ensemble, the adjoint, self-gravity).

With N > 1 (torchrun), every rank runs an independent replica of the
workload (the step does not shard); value = sum of zone-updates / max time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_CELLS = 256
METRIC = "zone-updates/s on 1 GB300, FP32 fused vs plain FP64, at L1 err <=1e-5 vs FP64"
WORKLOAD = ("3D MHD blast, FD 5th-order WENO + constrained transport, SSPRK(5,4), 256^3 periodic unit cube, "
            "gamma 5/3, rho 1, p 10 (r < 0.1) / 0.1, B (1,1,0)/sqrt2, C_cfl 1.5")
OT_WORKLOAD = "Orszag-Tang 2D MHD, FV HLL + Pang-Wu split (constrained B), MINMOD, SSP-RK2, 512x512 periodic, gamma 5/3"


def workload_config(n, world=1):
    """The `config` of the JSON line, identical in both arms."""
    return {"workload": WORKLOAD.replace("256^3", "%d^3" % n), "grid": [n, n, n],
            "precision": "fp32 fields, fp64 dt/time/conservation sums",
            "l2": "not flushed: state 738 MB + workspace 3.4 GB per step, far above the 129 MB L2" if n >= 128
            else "state below the L2 size",
            "parallelism": "replicas" if world > 1 else "single"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=None,
                    help="cells per axis (default: %d for the headline; each --case has its own)" % N_CELLS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-arena", action="store_true", help="skip the 256^3 blast comparison")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 64-run batched ensemble")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the 128^3 adjoint workload")
    ap.add_argument("--no-gravity", action="store_true", help="skip the self-gravity collapse workload")
    ap.add_argument("--no-l1", action="store_true", help="skip the full FP32 and FP64 runs to t_end (L1 error)")
    ap.add_argument("--no-ot", action="store_true", help="skip the Orszag-Tang 512^2 FV workload")
    ap.add_argument("--cpu-fp32-l1", type=int, default=0, metavar="N",
                    help="print the FP32-vs-FP64 L1 of the CPU restatement on Orszag-Tang N^2 to t = 0.5 and exit")
    ap.add_argument("--case", default=None, choices=["fdblast", "fd", "fdsrc", "fv3d", "fv3dseams", "fvsplit", "ensemble",
                                                     "adjoint", "gravity"],
                    help="run one small case of a secondary workload and exit (for profilers)")
    return ap.parse_args()


def run_case(name, n=None):
    """Small, self-contained runs of the workloads for ncu captures:
    fdblast: the headline FD blast at --n^3 (default 256^3) FP32, 2 steps (one warm-up);
    fd: the reference's FD WENO-CT arena blast 128^3 FP32, 2 steps; fv3d: FV Lax-Friedrichs MHD
    blast (--n, default 192)^3 FP32, 2 steps (one launch); fv3dseams: the same blast, the RK2 hydro
    seam and the magnetic seam called twice each (four launches; ncu -s 2 -c 2 takes the second
    pair); fvsplit: the same blast with the
    split MUSCL-Hancock scheme and HLLC; ensemble: 8 turbulent 2D MHD
    runs (128^2..512^2, t_end / 8) in one batched launch; adjoint: the 3D
    density-perturbation problem at 96^3 to t = 0.01, forward and backward
    with the stored tape (a 4 GB tape budget: the case holds a few GB at
    most); gravity: Evrard's collapse at 128^3 FP32, 3 steps of the
    self-gravity step sequence; fdsrc: the FD blast at 128^3 FP32 with
    turbulent forcing and the stellar-wind source, 2 steps."""
    import torch
    from astronomix_gb300 import _native

    if name == "fdblast":
        from _cases import blast_fd
        from astronomix_gb300.time_integration import get_plan

        n = n or N_CELLS
        cfg, prm, rv, s = blast_fd(n=n, dtype=np.float32, t_end=1e9)
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s.astype(np.float32)).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        info = plan.run(dev.data_ptr(), _native.make_params(prm), 2, st)
        print(json.dumps({"case": name, "n": n, "steps": info.steps, "status": info.status}))
    elif name in ("fd", "fv3d", "fvsplit"):
        from astronomix_gb300.time_integration import get_plan

        cfg, prm, rv, s = arena_blast(n or (128 if name == "fd" else 192), "fv_split" if name == "fvsplit" else name[:2])
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        info = plan.run(dev.data_ptr(), _native.make_params(prm), 2, st)
        print(json.dumps({"case": name, "steps": info.steps, "status": info.status}))
    elif name == "fv3dseams":
        from astronomix_gb300.time_integration import get_plan

        cfg, prm, rv, s = arena_blast(n or 192, "fv")
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        p = _native.make_params(prm)
        for _ in range(2):
            plan.hydro_rk2(dev.data_ptr(), p, 1e-5, st)
            plan.magnetic_update(dev.data_ptr(), p, 2e-4, st)
        torch.cuda.synchronize()
        print(json.dumps({"case": name, "status": plan.status(), "finite": bool(torch.isfinite(dev).all())}))
    elif name == "fdsrc":
        from astronomix_gb300.time_integration import get_plan
        from astronomix_gb300.option_classes import (WindConfig, WindParams, TurbulentForcingConfig,
                                                     TurbulentForcingParams)

        cfg, prm, rv, s = arena_blast(128, "fd")
        cfg = cfg._replace(wind_config=WindConfig(stellar_wind=True, num_injection_cells=8),
                           turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True))
        prm = prm._replace(wind_params=WindParams(wind_mass_loss_rate=1.0, wind_final_velocity=10.0),
                           turbulent_forcing_params=TurbulentForcingParams(energy_injection_rate=0.2))
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        info = plan.run(dev.data_ptr(), _native.make_params(prm), 2, st)
        print(json.dumps({"case": name, "steps": info.steps, "status": info.status}))
    elif name == "gravity":
        from astronomix_gb300.time_integration import get_plan
        from astronomix_gb300.initial_conditions import evrard_collapse

        cfg, prm, rv, s = evrard_collapse(128)
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        info = plan.run(dev.data_ptr(), _native.make_params(prm), 3, st)
        print(json.dumps({"case": name, "steps": info.steps, "status": info.status}))
    elif name == "ensemble":
        from astronomix_gb300.ensemble import Ensemble, turbulent_ensemble_member

        ms = [turbulent_ensemble_member(seed) for seed in range(8)]
        prms = [m[1]._replace(t_end=m[1].t_end / 8) for m in ms]
        ens = Ensemble([m[0] for m in ms], prms, ms[0][2], [m[3].shape for m in ms], np.float32)
        dev = [torch.from_numpy(m[3]).cuda() for m in ms]
        ens.run(dev)
        infos, lock = ens.info()
        print(json.dumps({"case": name, "lock_steps": lock, "status": max(i.status for i in infos)}))
    else:
        from astronomix_gb300.adjoint import AdjointIntegrator, density_perturbation_problem

        cfg, prm, rv, s, target = density_perturbation_problem(96, t_end=0.01)
        integ = AdjointIntegrator(cfg, prm, rv, s.shape, np.float32, tape_budget=4 << 30)
        y = integ.forward(torch.from_numpy(s).cuda())
        L, g = _loss_grad(y, torch.from_numpy(target).cuda().double())
        grad = integ.backward(g)
        torch.cuda.synchronize()
        print(json.dumps({"case": name, "steps": len(integ.schedule()[0]), "stored": integ.stored_tape(),
                          "finite": bool(torch.isfinite(grad).all())}))


def dist_setup(args):
    rank, world = 0, 1
    if args.gpus > 1 or "WORLD_SIZE" in os.environ:
        import torch
        import torch.distributed as dist

        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        local = int(os.environ.get("LOCAL_RANK", "0"))
        if world > 1:
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples (every 20 ms) of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.samples = []
        self.proc = None
        self.device_index = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is running (nvidia-smi
            # takes a while to start), so that its samples fall inside it
            t0 = time.perf_counter()
            while not self.samples and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
            self.samples.clear()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# The reference's own published benchmark: 3D MHD blast (arena/arena_tests/mhd/
# blast_test1.py:1-160), rho = 1, p = 100 inside r0 = 0.125 with a linear ramp
# to p = 1 at r1 = 1.1 r0, B = 10 (1, 1, 0)/sqrt(2), FP32, on 1x H200:
# fd_mhd 0.771 s/step and fv_mhd 0.0564 s/step at 256^3 (arena/*.svg).
H200_S_PER_STEP = {"fd": 0.771, "fv": 0.0564}


def arena_blast(n, solver):
    from astronomix_gb300 import (SimulationConfig, SimulationParams, get_registered_variables, finalize_config,
                                  construct_primitive_state, initialize_interface_fields, FINITE_DIFFERENCE,
                                  FINITE_VOLUME, LAX_FRIEDRICHS, PERIODIC_ROLL, SINGLE_PRECISION)
    from _cases import PERIODIC_2D

    if solver == "fd":
        cfg = SimulationConfig(solver_mode=FINITE_DIFFERENCE, mhd=True, dimensionality=3, num_cells=n,
                               boundary_handling=PERIODIC_ROLL, boundary_settings=PERIODIC_2D)
        prm = SimulationParams(C_cfl=1.5, minimum_density=1e-3, minimum_pressure=1e-3, t_end=0.02)
    elif solver == "fv_split":
        # the same blast with the split MUSCL-Hancock scheme and HLLC
        from astronomix_gb300 import SPLIT, MUSCL, HLLC
        cfg = SimulationConfig(solver_mode=FINITE_VOLUME, numerical_precision=SINGLE_PRECISION, mhd=True,
                               dimensionality=3, num_cells=n, riemann_solver=HLLC, split=SPLIT,
                               time_integrator=MUSCL, boundary_handling=PERIODIC_ROLL,
                               boundary_settings=PERIODIC_2D)
        prm = SimulationParams(C_cfl=0.8, t_end=0.02)
    else:
        cfg = SimulationConfig(solver_mode=FINITE_VOLUME, numerical_precision=SINGLE_PRECISION, mhd=True,
                               dimensionality=3, num_cells=n, riemann_solver=LAX_FRIEDRICHS,
                               boundary_handling=PERIODIC_ROLL, boundary_settings=PERIODIC_2D)
        prm = SimulationParams(C_cfl=0.8, t_end=0.02)
    rv = get_registered_variables(cfg)
    x = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    r0, r1 = 0.125, 1.1 * 0.125
    P = np.where(r <= r0, 100.0, np.where(r <= r1, 1.0 + 99.0 * (r1 - r) / (r1 - r0), 1.0))
    z = np.zeros_like(r, dtype=np.float32)
    b = np.full_like(z, 10 / np.sqrt(2))
    kw = dict(density=np.ones_like(z), velocity_x=z, velocity_y=z, velocity_z=z, magnetic_field_x=b,
              magnetic_field_y=b, magnetic_field_z=z, gas_pressure=P)
    if solver == "fd":
        fx, fy, fz = initialize_interface_fields(b, b, z)
        kw.update(interface_magnetic_field_x=fx, interface_magnetic_field_y=fy, interface_magnetic_field_z=fz)
    s = construct_primitive_state(cfg, rv, **kw)
    cfg = finalize_config(cfg, s.shape)
    return cfg, prm, rv, s


def time_arena(solver, n=256, steps=3):
    """s/step of the reference's published blast benchmark on this GPU (state > L2)."""
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan

    cfg, prm, rv, s = arena_blast(n, solver)
    plan = get_plan(cfg, rv, s.shape, np.float32)
    p = _native.make_params(prm)
    st = torch.cuda.current_stream()
    dev = torch.from_numpy(s).cuda()
    plan.reset(st.cuda_stream)
    plan.run_async(dev.data_ptr(), p, 2, st.cuda_stream)
    torch.cuda.synchronize()
    before = plan.run(dev.data_ptr(), p, 0, st.cuda_stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    plan.run_async(dev.data_ptr(), p, steps, st.cuda_stream)
    b.record(st)
    torch.cuda.synchronize()
    info = plan.run(dev.data_ptr(), p, 0, st.cuda_stream)
    sps = a.elapsed_time(b) / 1e3 / steps
    ok = bool(torch.isfinite(dev).all()) and info.status == 0
    del dev
    out = {"grid": [n, n, n], "s_per_step": sps, "zone_updates_per_s": n ** 3 / sps, "finite": ok,
           "steps_timed": steps}
    if solver in H200_S_PER_STEP:
        out["h200_published_s_per_step"] = H200_S_PER_STEP[solver]
        out["speedup_vs_h200_published"] = H200_S_PER_STEP[solver] / sps
    if solver == "fv":
        # FV 3D MHD: 4 (57 + 19 (k + 1)) algorithmic bytes per zone-update, k
        # the fixed-point iterations per step of the timed steps
        k = (info.magnetic_iterations - before.magnetic_iterations) / max(1, info.steps - before.steps)
        bpz = 4 * (57 + 19 * (k + 1))
        peak, src = hbm_peak()
        gbs = bpz * n ** 3 / sps / 1e9
        out["magnetic_iterations_mean"] = k
        out["roofline"] = {"bound": "hbm", "kernel": "fv_run_kernel", "achieved": gbs, "peak": peak, "unit": "GB/s",
                           "frac": gbs / peak, "traffic": load_traffic("fv_run_kernel_blast256_fp32_step"),
                           "note": "algorithmic %.0f B/zone-update (k = %.2f), peak %s; traffic = DRAM bytes per "
                                   "step (ncu)" % (bpz, k, src)}
    return out


def time_fd_sources(n=256, steps=3):
    """The FD showcase combination on the 256^3 blast (FP32): turbulent
    forcing (energy injection rate 0.2) before every step and a stellar-wind
    EI source (8 injection cells) in every stage, against the same run
    without them."""
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.option_classes import (WindConfig, WindParams, TurbulentForcingConfig,
                                                 TurbulentForcingParams)
    from astronomix_gb300.time_integration import get_plan

    cfg, prm, rv, s = arena_blast(n, "fd")
    cfg = cfg._replace(wind_config=WindConfig(stellar_wind=True, num_injection_cells=8),
                       turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True))
    prm = prm._replace(wind_params=WindParams(wind_mass_loss_rate=1.0, wind_final_velocity=10.0),
                       turbulent_forcing_params=TurbulentForcingParams(energy_injection_rate=0.2))
    plan = get_plan(cfg, rv, s.shape, np.float32)
    p = _native.make_params(prm)
    st = torch.cuda.current_stream()
    dev = torch.from_numpy(s).cuda()
    plan.reset(st.cuda_stream)
    plan.run_async(dev.data_ptr(), p, 2, st.cuda_stream)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    plan.run_async(dev.data_ptr(), p, steps, st.cuda_stream)
    b.record(st)
    torch.cuda.synchronize()
    info = plan.run(dev.data_ptr(), p, 0, st.cuda_stream)
    sps = a.elapsed_time(b) / 1e3 / steps
    ok = bool(torch.isfinite(dev).all()) and info.status == 0
    del dev
    return {"workload": "FD WENO-CT blast %d^3 + turbulent forcing + stellar-wind EI source" % n,
            "s_per_step": sps, "zone_updates_per_s": n ** 3 / sps, "finite": ok, "steps_timed": steps}


def time_ensemble(num_runs=64, sequential=True):
    """The batched turbulent ensemble: num_runs 2D MHD runs (seeds 0..num_runs-1,
    grid sizes from {128, 192, 256, 384, 512}^2, t_end in [0.05, 0.2], FV HLLC,
    FP32), autotuned, advanced to their end times by one graph-replayed
    persistent launch.  Zone-updates = sum over runs of steps x cells.  With
    `sequential`, the same runs one after another through the single-run
    path, for comparison."""
    import torch
    from astronomix_gb300.ensemble import Ensemble, turbulent_ensemble_member
    from astronomix_gb300.time_integration import get_plan
    from astronomix_gb300 import _native

    ms = [turbulent_ensemble_member(seed) for seed in range(num_runs)]
    shapes = [m[3].shape for m in ms]
    ens = Ensemble([m[0] for m in ms], [m[1] for m in ms], ms[0][2], shapes, np.float32)
    host = [torch.from_numpy(m[3]) for m in ms]
    dev = [h.cuda() for h in host]
    t0 = time.perf_counter()
    tiling = ens.tune(dev, steps=3)
    tune_s = time.perf_counter() - t0
    ens.reset()
    stream = torch.cuda.current_stream()
    ens.run([d.clone() for d in dev], max_steps=2)  # builds and warms the graph path
    torch.cuda.synchronize()
    ens.reset()
    work = [d.clone() for d in dev]
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ens.run(work)
    b.record(stream)
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3
    infos, lock = ens.info()
    zu = sum(i.steps * s[-1] * s[-2] for i, s in zip(infos, shapes))
    iters = sum(i.magnetic_iterations for i in infos) / max(1, sum(i.steps for i in infos))
    ok = all(i.status == 0 for i in infos) and all(abs(i.t - m[1].t_end) < 1e-9 for i, m in zip(infos, ms))
    # algorithmic bytes: each run's own steps and fixed-point iterations in
    # the 2D formula, 4 (46 + 16 (k + 1)) bytes a zone-update
    nbytes = sum(4 * s[-1] * s[-2] * (46 * i.steps + 16 * (i.magnetic_iterations + i.steps))
                 for i, s in zip(infos, shapes))
    peak, peak_src = hbm_peak()
    out = {"runs": num_runs, "grids": sorted(set(s[-1] for s in shapes)), "cells_total": sum(s[-1] * s[-2] for s in shapes),
           "zone_updates": zu, "seconds": sec, "zone_updates_per_s": zu / sec, "lock_steps": lock,
           "magnetic_iterations_mean": iters, "tiling": tiling, "tune_s": tune_s, "graph": True, "ok": ok,
           "launches": 2,
           "roofline": {"bound": "hbm", "kernel": "fv_batch_kernel", "achieved": nbytes / sec / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": nbytes / sec / 1e9 / peak, "traffic": None,
                        "note": "algorithmic bytes summed over the runs with their own steps and fixed-point "
                                "iterations, 4 (46 + 16 (k + 1)) B a zone-update; peak %s" % peak_src}}
    if sequential:
        seq_s = 0.0
        for m, h in zip(ms, host):
            cfg, prm, rv, st = m
            plan = get_plan(cfg, rv, st.shape, np.float32)
            p = _native.make_params(prm)
            d = h.cuda()
            plan.reset(stream.cuda_stream)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            plan.run(d.data_ptr(), p, 1 << 40, stream.cuda_stream)
            seq_s += time.perf_counter() - t1
            del d
        out["sequential_single_run_seconds"] = seq_s
        out["speedup_vs_sequential"] = seq_s / sec
    del work, dev
    return out


def time_gravity(n=128, steps=20, warmup=3, cpu_n=16):
    """Self-gravity: Evrard's collapse at n^3 (FP32), `steps` steps of the
    device-driven step sequence timed with CUDA events after `warmup` steps;
    the open-boundary Poisson solve on the padded grid ((n + 4)^3, zero
    padded to (2n + 8)^3) timed alone; the oracle on cpu_n^3 for one step on
    one host core."""
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan, gravitational_potential
    from astronomix_gb300.initial_conditions import evrard_collapse

    cfg, prm, rv, s = evrard_collapse(n)
    plan = get_plan(cfg, rv, s.shape, np.float32)
    dev = torch.from_numpy(s).cuda()
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    p = _native.make_params(prm)
    plan.reset(st)
    info = plan.run(dev.data_ptr(), p, warmup, st)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    plan.run_async(dev.data_ptr(), p, steps, st)
    b.record(stream)
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3
    status = plan.status(stream=st)
    # the Poisson solve of one gas update, alone (same grid as the run's)
    m = n + 4
    rho = torch.rand((m, m, m), device="cuda", dtype=torch.float32) + 0.5
    for _ in range(3):
        gravitational_potential(rho, cfg._replace(num_cells=m), 1.0)
    torch.cuda.synchronize()
    a.record(stream)
    reps = 20
    for _ in range(reps):
        gravitational_potential(rho, cfg._replace(num_cells=m), 1.0)
    b.record(stream)
    torch.cuda.synchronize()
    poisson_ms = a.elapsed_time(b) / reps
    out = {"workload": "Evrard collapse %d^3, split MUSCL-Hancock HLLC, RIEMANN_SPLIT_UNSTABLE, reflective walls "
                       "(open Poisson solve, Hockney-Eastwood)" % n,
           "steps": steps, "ms_per_step": 1e3 * sec / steps, "zone_updates_per_s": n ** 3 * steps / sec,
           "poisson_solve_ms": poisson_ms, "poisson_grid": [2 * m] * 3,
           "poisson_share_of_step": poisson_ms / (1e3 * sec / steps), "status": int(status)}
    # the oracle (reference algorithm, NumPy) on a small grid, one step
    from oracle import driver as odriver

    cfg_c, prm_c, rv_c, s_c = evrard_collapse(cpu_n, dtype=np.float64)
    t0 = time.perf_counter()
    odriver.time_integration(s_c, cfg_c, prm_c, rv_c, max_steps=1)
    cpu_s = time.perf_counter() - t0
    out["cpu_oracle"] = {"grid": [cpu_n] * 3, "zone_updates_per_s": cpu_n ** 3 / cpu_s, "cores": 1}
    del dev
    return out


def _loss_grad(y, tgt):
    """mean((rho_T - rho*)^2) in FP64 and its gradient with respect to the final state."""
    import torch

    d = y[0].double() - tgt
    L = float((d * d).mean())
    g = torch.zeros_like(y)
    g[0] = (2.0 * d / d.numel()).to(y.dtype)
    return L, g


def _fd_check(integ, x, grad, tgt, directions, eps, rows, seed=2):
    """Central differences of the replayed program along random directions on
    `rows`, relative to the adjoint's directional derivative."""
    import torch

    rng = np.random.default_rng(seed)
    errs = []
    for _ in range(directions):
        d = torch.zeros_like(x)
        for r in rows:
            d[r] = torch.from_numpy(rng.standard_normal(tuple(x.shape[1:])).astype(np.float32)).to(x)
        Lp, _ = _loss_grad(integ.replay(x + eps * d), tgt)
        Lm, _ = _loss_grad(integ.replay(x - eps * d), tgt)
        fd = (Lp - Lm) / (2 * eps)
        ad = float((grad.double() * d.double()).sum())
        errs.append(abs(fd - ad) / abs(ad))
    return {"directions": directions, "eps": eps, "rel_err_max": max(errs), "rel_err_median": float(np.median(errs))}


def time_adjoint(n=128, directions=16, eps=1e-3, checkpoint_every=20, fp64=True):
    """The adjoint workload: 3D MHD density-perturbation inverse problem at
    n^3 (HLL, Pang-Wu split, adaptive steps to t = 0.1), loss =
    mean((rho_T - rho*)^2) accumulated in FP64, gradient with respect to the
    whole initial state by the discrete adjoint, FP32.  Two initial states:
    the problem as posed (v = 0, uniform p), which is an HLL equilibrium in
    v and p with no magnetic fixed-point iterations, and a smooth variant
    with velocity and pressure perturbed (0.1 x GRF), whose magnetic update
    iterates.  For each: the plain forward, and forward + backward with the
    tape stored by the forward and with checkpoints every
    `checkpoint_every` steps (one segment replayed at a time).  The
    gradient is checked against central finite differences of the replayed
    program and against the FP64 adjoint; the problem as posed sits at the
    kink of the MINMOD limiter in v and p (their slopes are exactly zero),
    where no finite difference reproduces a gradient, so its check uses the
    density and pressure rows only and the smooth variant's all gas rows."""
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.adjoint import AdjointIntegrator, density_perturbation_problem
    from astronomix_gb300.ensemble import create_turb_field
    from astronomix_gb300.time_integration import get_plan

    def ev():
        return torch.cuda.Event(enable_timing=True)

    stream = torch.cuda.current_stream()

    def timed(integ, x, tgt):
        y = integ.forward(x)  # warm-up
        integ.backward(_loss_grad(y, tgt)[1])
        torch.cuda.synchronize()
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        y = integ.forward(x)
        e1.record(stream)
        L, g = _loss_grad(y, tgt)
        grad = integ.backward(g)
        e2.record(stream)
        torch.cuda.synchronize()
        return L, grad, e0.elapsed_time(e1) / 1e3, e0.elapsed_time(e2) / 1e3

    def smooth(s, dtype):
        for k, sd in ((1, 11), (2, 12), (3, 13)):
            f = create_turb_field(n, 1.0, -1.5, 1.0, 0.7 * n / 2, seed=sd, dimensionality=3)
            s[k] = (0.1 * f / f.std()).astype(dtype)
        f = create_turb_field(n, 1.0, -1.5, 1.0, 0.7 * n / 2, seed=14, dimensionality=3)
        s[4] = (1.0 + 0.1 * f / f.std()).astype(dtype)
        return s

    cfg, prm, rv, s, target = density_perturbation_problem(n)
    tgt = torch.from_numpy(target).cuda().double()
    plan = get_plan(cfg, rv, s.shape, np.float32)
    p = _native.make_params(prm)

    def measure(s0, rows):
        x = torch.from_numpy(s0).cuda()
        res = {}
        # the plain forward: the ordinary plan, no tape, no checkpoints
        for _ in range(2):
            xp = x.clone()
            plan.reset(stream.cuda_stream)
            a, b = ev(), ev()
            a.record(stream)
            plan.run(xp.data_ptr(), p, 1 << 40, stream.cuda_stream)
            b.record(stream)
            torch.cuda.synchronize()
        plain_s = a.elapsed_time(b) / 1e3
        res["plain_forward_s"] = plain_s
        grad = None
        for mode, budget in (("stored_tape", "auto"), ("checkpoints", 0)):
            integ = AdjointIntegrator(cfg, prm, rv, s.shape, np.float32, checkpoint_every=checkpoint_every,
                                      tape_budget=budget)
            L, g, fwd_s, fb_s = timed(integ, x, tgt)
            dts, its = integ.schedule()
            res[mode] = {"stored": integ.stored_tape(), "forward_s": fwd_s, "forward_plus_backward_s": fb_s,
                         "ratio_over_plain_forward": fb_s / plain_s, "memory_bytes": integ.memory()}
            if mode == "checkpoints":
                res[mode]["checkpoint_every"] = checkpoint_every
                res["steps"] = len(dts)
                res["magnetic_iterations_mean"] = float(np.mean(its)) if its else 0.0
                res["loss"] = L
                res["fd_check"] = _fd_check(integ, x, g, tgt, directions, eps, rows=rows)
                grad = g
            del integ
        return res, grad

    out = {"grid": [n, n, n]}
    posed, grad = measure(s.copy(), rows=(0, 4))
    out.update(posed)
    s_smooth = smooth(s.copy(), np.float32)
    out["smooth_variant"], grad_s = measure(s_smooth, rows=(0, 1, 2, 3, 4))
    # FP32 vs FP64 adjoint on both initial states
    if fp64:
        cfg64, prm64, rv64, s64, _ = density_perturbation_problem(n, dtype=np.float64)
        for key, s_init, g32, rows in ((None, s64, grad, [0, 4]),
                                       ("smooth_variant", smooth(s64.copy(), np.float64), grad_s, [0, 1, 2, 3, 4])):
            integ64 = AdjointIntegrator(cfg64, prm64, rv64, s64.shape, np.float64, tape_budget="auto")
            y64 = integ64.forward(torch.from_numpy(s_init).cuda())
            g64 = integ64.backward(_loss_grad(y64, tgt)[1])
            err = float(torch.linalg.norm(g32[rows].double() - g64[rows]) / torch.linalg.norm(g64[rows]))
            (out if key is None else out[key])["fp64_grad_rel_l2_err"] = err
            del integ64, y64, g64
    return out


def algorithmic_bytes_per_zone_update(k_mean, elem=4):
    # FV 2D MHD: hydro RK2 half steps 2 x 20 words + magnetic 16 words per
    # fixed-point evaluation x (k + 1) + 6 words of write-back
    return elem * (46 + 16 * (k_mean + 1))


def load_traffic(name):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(name)
    except (OSError, ValueError):
        return None


CPU_SAMPLE_N = 64


def run_reference(args, rank, world):
    """--impl reference: the reference's algorithm on this host's cores.  The
    reference is Python/JAX and JAX is not installed on these machines, so
    this times the port of its FD step that the oracle keeps: the compiled
    restatement oracle/cpu/fd_step.cpp (C++17, OpenMP over every host core),
    which is bit-identical to the NumPy oracle and to the reference's own
    results on the committed fixtures, on a bounded sample of the workload,
    the same blast at 64^3; each of the --steps steps is one time step."""
    if rank != 0:
        return
    m = CPU_SAMPLE_N
    v, steps, dt, threads = cpu_fd_sample(m, budget_s=120.0, max_steps=max(1, args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(1, steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.n or N_CELLS, world),
        "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": threads, "kind": "port",
                         "sample": "compiled restatement of the reference's FD step, %d OpenMP threads, blast %d^3 "
                                   "FP32, %d steps in %.1f s (after one warm-up step)" % (threads, m, steps, dt)},
        "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def time_orszag_tang(n=512, K=100, t_cmp=0.5, flush_mb=512):
    """The FV workload (Orszag-Tang 512^2, FP32): zone-updates/s with one
    step per launch and the L2 flushed between steps (the state is 7.3 MB),
    end to end through the C ABI with pinned host buffers, the FP64 rate of
    the same kernels, the FP32-vs-FP64 relative L1 density error of full runs
    to t_cmp, and the roofline of fv_run_kernel (HBM, algorithmic bytes)."""
    import torch

    from _cases import orszag_tang
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan

    cfg, prm, rv, s = orszag_tang(n=n, t_end=1e9, dtype=np.float32)
    p = _native.make_params(prm)
    plan = get_plan(cfg, rv, s.shape, np.float32)
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    state = torch.from_numpy(s).cuda()
    flush = torch.empty(flush_mb * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    plan.reset(st)
    for _ in range(5):
        plan.run_async(state.data_ptr(), p, 1, st)
    torch.cuda.synchronize()
    it0 = plan.run(state.data_ptr(), p, 0, st)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    for i in range(K):
        flush.zero_()
        starts[i].record(stream)
        plan.run_async(state.data_ptr(), p, 1, st)
        ends[i].record(stream)
    torch.cuda.synchronize()
    total_s = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / 1e3
    it1 = plan.run(state.data_ptr(), p, 0, st)
    k_mean = (it1.magnetic_iterations - it0.magnetic_iterations) / max(1, it1.steps - it0.steps)
    value = n * n * K / total_s
    # end to end through the C ABI with host buffers (pinned)
    host = torch.from_numpy(s.copy()).pin_memory()
    host_out = torch.empty_like(host).pin_memory()
    dev2 = torch.empty_like(state)
    nbytes = host.numel() * host.element_size()
    Ke = 20
    es = [torch.cuda.Event(enable_timing=True) for _ in range(Ke)]
    ee = [torch.cuda.Event(enable_timing=True) for _ in range(Ke)]
    plan.reset(st)
    for i in range(Ke):
        flush.zero_()
        es[i].record(stream)
        dev2.copy_(host, non_blocking=True)
        plan.run_async(dev2.data_ptr(), p, 1, st)
        host_out.copy_(dev2, non_blocking=True)
        ee[i].record(stream)
    torch.cuda.synchronize()
    e2e = n * n * Ke / (sum(a.elapsed_time(b) for a, b in zip(es, ee)) / 1e3)
    # FP64, same kernels
    cfg64, prm64, rv64, s64 = orszag_tang(n=n, t_end=1e9, dtype=np.float64)
    plan64 = get_plan(cfg64, rv64, s64.shape, np.float64)
    st64 = torch.from_numpy(s64).cuda()
    plan64.reset(st)
    for _ in range(3):
        plan64.run_async(st64.data_ptr(), p, 1, st)
    K64 = 10
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    plan64.run_async(st64.data_ptr(), p, K64, st)
    b.record(stream)
    torch.cuda.synchronize()
    fp64_value = n * n * K64 / (a.elapsed_time(b) / 1e3)
    # FP32 vs FP64 at t_cmp from the same initial state
    res = {}
    steps = {}
    for name, dt in (("fp32", np.float32), ("fp64", np.float64)):
        c_, pr_, rv_, s_ = orszag_tang(n=n, t_end=t_cmp, dtype=dt)
        pl = get_plan(c_, rv_, s_.shape, dt)
        d_ = torch.from_numpy(s_.astype(dt)).cuda()
        pl.reset(st)
        info = pl.run(d_.data_ptr(), _native.make_params(pr_), 1 << 40, st)
        res[name] = d_[0].double()
        steps[name] = info.steps
    l1 = float((res["fp32"] - res["fp64"]).abs().sum() / res["fp64"].abs().sum())
    bpz = algorithmic_bytes_per_zone_update(k_mean)
    achieved = bpz * n * n / (total_s / K) / 1e9
    peak, peak_src = hbm_peak()
    return {"workload": OT_WORKLOAD, "value": value, "unit": "zone-updates/s", "ms_per_step": 1e3 * total_s / K,
            "steps": K, "l2": "flushed between timed steps (%d MB write); state 7.3 MB" % flush_mb,
            "e2e": {"value": e2e, "unit": "zone-updates/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "fp64_value": fp64_value, "fp32_over_fp64": value / fp64_value,
            "l1_err_vs_fp64": l1, "l1_t_end": t_cmp, "l1_steps": [steps["fp32"], steps["fp64"]],
            "magnetic_iterations_mean": k_mean,
            "roofline": {"bound": "hbm", "kernel": "fv_run_kernel", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": load_traffic("fv_run_kernel_ot512_fp32_step"),
                         "note": "algorithmic %.0f B/zone-update (k = %.2f fixed-point iterations), peak %s" % (
                             bpz, k_mean, peak_src)}}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# FD algorithmic figures (FP32).  A step reads and writes 11 words per cell per
# array pass, 16 array passes: 704 B per zone-update.  The z and y k_weno
# launches read the cell-centre state (8 words) and write their flux
# difference (7: B's own-axis row is zero) and two CT-corrected fluxes: 17
# words per cell each.  The x launch, which applies the stage, reads the state
# (8), the y and z differences (7 + 7) and the registers Q0, Q, QF (24) and
# writes Q, QF (16) and its two CT fluxes: 64 words; in the last stage of the
# step (no Q0, Q) 40.  Averaged over the 15 launches of a step: 31.1 words.
FD_STEP_BYTES_PER_ZU = 704
WENO_BYTES_PER_CELL = 4 * (4 * (17 + 17 + 64) + (17 + 17 + 40)) / 15.0


def cpu_fd_sample(n, budget_s, max_steps=1 << 30):
    """The oracle's compiled restatement of the reference's FD step
    (oracle/cpu/fd_step.cpp, bit-identical to the NumPy oracle and to the
    reference's own results on the committed fixtures) on the same blast at
    n^3, FP32, with every host core (OpenMP): one warm-up step, then steps
    until budget_s.  Returns (zone-updates/s, steps, seconds, threads)."""
    from _cases import blast_fd
    from oracle import cpu

    cfg, prm, rv, s = blast_fd(n=n, dtype=np.float32, t_end=10.0)
    P = np.ascontiguousarray(s.astype(np.float32))
    cpu.fd_run(P, cfg, prm, max_steps=1)
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s and steps < max_steps:
        cpu.fd_run(P, cfg, prm, max_steps=1)
        steps += 1
    dt = time.perf_counter() - t0
    return n ** 3 * steps / dt, steps, dt, cpu.threads()


def cpu_baseline_fd(budget_s=15.0, n=64):
    v, steps, dt, threads = cpu_fd_sample(n, budget_s)
    return {"value": v, "unit": "zone-updates/s", "cores": threads, "kind": "port",
            "sample": "compiled restatement of the reference's FD step (C++17, OpenMP, %d threads), "
                      "blast %d^3 FP32, %d steps in %.1f s" % (threads, n, steps, dt)}


def cpu_fv_sample(cfg, prm, s, budget_s):
    """The oracle's compiled restatement of the reference's unsplit FV step
    (oracle/cpu/fv_step.cpp, equal to the NumPy oracle on the CPU tests) on
    the state s (FP32), with every host core (OpenMP): one warm-up step, then
    steps until budget_s.  Returns the cpu_baseline record."""
    from oracle import cpu

    P = np.ascontiguousarray(s.astype(np.float32))
    prm = prm._replace(t_end=1e9)
    cpu.fv_run(P, cfg, prm, max_steps=1)
    steps, iters = 0, 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        iters += cpu.fv_run(P, cfg, prm, max_steps=1)[2]
        steps += 1
    dt = time.perf_counter() - t0
    zones = int(np.prod(s.shape[1:]))
    shape = "x".join(str(v) for v in s.shape[1:])
    out = {"value": zones * steps / dt, "unit": "zone-updates/s", "cores": cpu.threads(), "kind": "port",
           "sample": "compiled restatement of the reference's FV step (C++17, OpenMP, %d threads), %s FP32, "
                     "%d steps in %.1f s" % (cpu.threads(), shape, steps, dt)}
    if cfg.mhd:
        out["magnetic_iterations_mean"] = iters / max(1, steps)
    return out


def e2e_pipelined(plan, p, host, like, steps, stream):
    """Seconds for `steps` independent time steps of states held in pinned
    host memory, through the C ABI: step i copies `host` into device buffer
    i % 2, advances it one step (plan.run_async on `stream`) and copies it
    back into a pinned host buffer.  The copies run on a second stream,
    ordered by events: step i + 1's input goes in and step i - 1's result
    comes out while step i computes; a buffer is refilled only after its
    previous result has left.  CUDA events on `stream` bracket the whole."""
    import torch

    copy = torch.cuda.Stream()
    bufs = [torch.empty_like(like), torch.empty_like(like)]
    outs = [torch.empty_like(host).pin_memory(), torch.empty_like(host).pin_memory()]
    h2d = [torch.cuda.Event() for _ in range(steps)]
    done = [torch.cuda.Event() for _ in range(steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = stream.cuda_stream
    torch.cuda.synchronize()
    start.record(stream)
    copy.wait_stream(stream)

    def load(i):
        with torch.cuda.stream(copy):
            bufs[i % 2].copy_(host, non_blocking=True)
            h2d[i].record(copy)

    load(0)
    for i in range(steps):
        if i + 1 < steps:
            load(i + 1)
        stream.wait_event(h2d[i])
        plan.run_async(bufs[i % 2].data_ptr(), p, 1, st)
        done[i].record(stream)
        with torch.cuda.stream(copy):
            copy.wait_event(done[i])
            outs[i % 2].copy_(bufs[i % 2], non_blocking=True)
    stream.wait_stream(copy)
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / 1e3


def cpu_fp32_l1(n, t_end=0.5):
    """FP32-vs-FP64 relative L1 density error of the oracle's compiled
    restatement of the reference's FV step (IEEE arithmetic, no contraction)
    on Orszag-Tang n^2 to t_end: the accuracy of a faithful FP32 run of the
    scheme, against which the GPU's FP32 figure is read.  CPU only."""
    from _cases import orszag_tang
    from oracle import cpu

    out, res = {"workload": "Orszag-Tang %dx%d to t = %g, oracle/cpu/fv_step.cpp" % (n, n, t_end)}, {}
    for dt in (np.float32, np.float64):
        cfg, prm, rv, s = orszag_tang(n=n, t_end=t_end, dtype=dt)
        s = np.ascontiguousarray(s.astype(dt))
        t0 = time.perf_counter()
        t, steps, iters = cpu.fv_run(s, cfg, prm)
        res[dt.__name__] = s[0].astype(np.float64)
        out[dt.__name__] = {"t": t, "steps": steps, "magnetic_iterations": iters,
                            "seconds": time.perf_counter() - t0}
    out["rel_l1_density_fp32_vs_fp64"] = float(np.abs(res["float32"] - res["float64"]).sum() /
                                               np.abs(res["float64"]).sum())
    out["cores"] = cpu.threads()
    return out


def run_ours(args, rank, world):
    import torch

    from _cases import blast_fd
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan
    from astronomix_gb300.replicas import replica_throughput

    dev_index = torch.cuda.current_device()
    n = args.n or N_CELLS
    cfg, prm, rv, s = blast_fd(n=n, dtype=np.float32, t_end=1e9)
    s = s.astype(np.float32)
    p = _native.make_params(prm)
    plan = get_plan(cfg, rv, s.shape, np.float32)
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    state = torch.from_numpy(s).cuda()
    plan.reset(st)

    # warm-up: W steps
    for _ in range(max(args.warmup, 3)):
        plan.run_async(state.data_ptr(), p, 1, st)
    torch.cuda.synchronize()

    # timed: K steps, one CUDA-event pair per step; the plan also records an
    # event after every launch (per-kernel durations for the roofline)
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    plan.profile(True)
    plan.profile_read(reset=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev_index) as clk:
        for i in range(K):
            starts[i].record(stream)
            plan.run_async(state.data_ptr(), p, 1, st)
            ends[i].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    prof = plan.profile_read(reset=True)
    plan.profile(False)
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    info = plan.run(state.data_ptr(), p, 0, st)
    status = info.status
    value = replica_throughput(n ** 3 * K, total_s)
    total_s_max = max_over_ranks(total_s, world)
    launches = int(sum(v[1] for v in prof.values()))
    kernels = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1], "share": v[0] / max(1e-30, sum(
        w[0] for w in prof.values()))} for k, v in prof.items() if v[1]}

    # ---- roofline of the dominant kernel, k_weno (x, y, z launches together)
    weno_ms = sum(prof[k][0] for k in ("weno_x", "weno_y", "weno_z"))
    weno_launches = sum(prof[k][1] for k in ("weno_x", "weno_y", "weno_z"))
    weno_s = weno_ms / 1e3 / max(1, weno_launches)
    peak, peak_src = hbm_peak()
    achieved = WENO_BYTES_PER_CELL * n ** 3 / weno_s / 1e9
    weno_prof = load_traffic("k_weno_fd_blast256_fp32") or {}
    traffic = weno_prof.get("dram_bytes_per_launch")
    fp32_peak = _native.probe_fp32_fma(st)
    flop_per_cell = weno_prof.get("fp32_flop_per_cell")
    compute = None
    if flop_per_cell:
        tf = flop_per_cell * n ** 3 / weno_s / 1e12
        compute = {"achieved": tf, "peak": fp32_peak, "unit": "TFLOP/s", "frac": tf / fp32_peak,
                   "flop_per_cell_per_launch": flop_per_cell,
                   "note": "FP32 flops counted by ncu per k_weno launch / cells: fadd + fmul + 2 ffma + "
                           "2 (fadd2 + fmul2 + 2 ffma2), the paired instructions doing two operations; "
                           "peak = amx_probe_fp32_fma (register-only FMA chains on every SM)"}

    # ---- end to end through the C ABI with host buffers (pinned)
    host = torch.from_numpy(s.copy()).pin_memory()
    host_out = torch.empty_like(host).pin_memory()
    dev2 = torch.empty_like(state)
    nbytes = host.numel() * host.element_size()
    Ke = max(3, min(K, 10))
    es = [torch.cuda.Event(enable_timing=True) for _ in range(Ke)]
    ee = [torch.cuda.Event(enable_timing=True) for _ in range(Ke)]
    plan.reset(st)
    for i in range(Ke):
        es[i].record(stream)
        dev2.copy_(host, non_blocking=True)
        plan.run_async(dev2.data_ptr(), p, 1, st)
        host_out.copy_(dev2, non_blocking=True)
        ee[i].record(stream)
    torch.cuda.synchronize()
    e2e_serial_s = sum(a.elapsed_time(b) for a, b in zip(es, ee)) / 1e3
    e2e_serial = replica_throughput(n ** 3 * Ke, e2e_serial_s)
    del dev2, host_out
    # the same Ke steps with every step's copies overlapping the neighbouring
    # steps' compute: the headline e2e figure
    e2e_s = e2e_pipelined(plan, p, host, state, Ke, stream)
    e2e_value = replica_throughput(n ** 3 * Ke, e2e_s)
    del host

    # ---- FP64: the same kernels in double precision (a few steps)
    cfg64, prm64, rv64, s64 = blast_fd(n=n, dtype=np.float64, t_end=1e9)
    plan64 = get_plan(cfg64, rv64, s64.shape, np.float64)
    st64 = torch.from_numpy(s64.astype(np.float64)).cuda()
    plan64.reset(st)
    plan64.run_async(st64.data_ptr(), p, 1, st)
    K64 = 3
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    plan64.run_async(st64.data_ptr(), p, K64, st)
    b.record(stream)
    torch.cuda.synchronize()
    fp64_value = n ** 3 * K64 / (a.elapsed_time(b) / 1e3)
    del st64

    # ---- accuracy: full runs to t_end = 0.02 in FP32 and FP64 from the same state
    l1 = None
    if not args.no_l1:
        res, steps_l1 = {}, {}
        for name, dt in (("fp32", np.float32), ("fp64", np.float64)):
            c_, pr_, rv_, s_ = blast_fd(n=n, dtype=dt, t_end=0.02)
            pl = get_plan(c_, rv_, s_.shape, dt)
            d_ = torch.from_numpy(s_.astype(dt)).cuda()
            pl.reset(st)
            inf = pl.run(d_.data_ptr(), _native.make_params(pr_), 1 << 40, st)
            res[name] = d_[0].double()
            steps_l1[name] = [inf.steps, inf.t, inf.status]
            del d_
        l1 = {"rel_l1_density": float((res["fp32"] - res["fp64"]).abs().sum() / res["fp64"].abs().sum()),
              "t_end": 0.02, "runs": steps_l1}
        del res

    # ---- secondary workloads
    ot = None if args.no_ot else time_orszag_tang()
    arena = {}
    if not args.no_arena:
        arena = {"fd_blast_fp32": time_arena("fd"), "fv_lf_blast_fp32": time_arena("fv"),
                 "fd_blast_forcing_wind_fp32": time_fd_sources(), "fv_split_hllc_blast_fp32": time_arena("fv_split")}
        arena["fd_blast_forcing_wind_fp32"]["overhead_vs_plain"] = (
            arena["fd_blast_forcing_wind_fp32"]["s_per_step"] / arena["fd_blast_fp32"]["s_per_step"] - 1.0)
    ensemble = None if args.no_ensemble else time_ensemble()
    adjoint = None if args.no_adjoint else time_adjoint()
    gravity = None if args.no_gravity else time_gravity()

    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline else cpu_baseline_fd()
    if not args.no_cpu_baseline:
        from _cases import orszag_tang
        if ot is not None:
            cfg_, prm_, rv_, s_ = orszag_tang(n=256, dtype=np.float32)
            ot["cpu_baseline"] = cpu_fv_sample(cfg_, prm_, s_, 8.0)
        if "fv_lf_blast_fp32" in arena:
            cfg_, prm_, rv_, s_ = arena_blast(64, "fv")
            arena["fv_lf_blast_fp32"]["cpu_baseline"] = cpu_fv_sample(cfg_, prm_, s_, 8.0)
    config = workload_config(n, world)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "zone-updates/s",
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s_max / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config,
        "e2e": {"value": e2e_value, "unit": "zone-updates/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes,
                "note": "each step: pinned host state -> device, one time step through the C ABI, device -> "
                        "pinned host, on two device buffers: a step's copies run on a second stream while the "
                        "neighbouring step computes (every copy inside the timed region); serial: copy, step "
                        "and copy back one after another on one stream",
                "serial": {"value": e2e_serial, "unit": "zone-updates/s"}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_weno (x, y, z)", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "note": "algorithmic %.1f B/cell per launch, %.3f ms average launch, peak %s; the kernel "
                             "is bound by FP32 issue, see compute" % (WENO_BYTES_PER_CELL, 1e3 * weno_s, peak_src),
                     "compute": compute,
                     "step": {"algorithmic_bytes_per_zone_update": FD_STEP_BYTES_PER_ZU,
                              "achieved_gbs": FD_STEP_BYTES_PER_ZU * value / 1e9,
                              "frac": FD_STEP_BYTES_PER_ZU * value / 1e9 / peak}},
        "kernels": kernels,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "fp64_value": fp64_value,
        "fp32_over_fp64": value / fp64_value,
        "l1_err_vs_fp64": l1["rel_l1_density"] if l1 else None,
        "l1": l1,
        "fp32_fma_peak_tflops": fp32_peak,
        "fv_orszag_tang_512_fp32": ot,
        "reference_published_workloads": arena,
        "ensemble_fp32": ensemble,
        "adjoint_fp32": adjoint,
        "self_gravity_fp32": gravity,
        "status": status,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.cpu_fp32_l1:
        print(json.dumps(cpu_fp32_l1(args.cpu_fp32_l1)))
        return
    if args.case:
        run_case(args.case, args.n)
        return
    rank, world = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        import torch

        if not torch.cuda.is_available():
            print(json.dumps({"metric": METRIC, "error": "no CUDA device"}))
            sys.exit(1)
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
