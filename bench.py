"""Benchmark: zone-updates/s of the FV MHD step on the 2D Orszag-Tang vortex, 512^2, FP32.

One "step" is one time step of astronomix's finite-volume MHD scheme (CFL dt,
SSP-RK2 hydro half step, implicit-midpoint magnetic sub-step, hydro half step)
over the whole 512^2 grid, launched through the C ABI.  The Orszag-Tang state
is synthetic (its analytic initial condition, advanced by warm-up steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: each timed step is bracketed by CUDA events on the launching stream
and the L2 cache (129 MB; the state is 7.3 MB) is flushed between steps by
writing a 512 MB buffer, outside the events.  The line also carries the
end-to-end number through the C ABI with host buffers (H2D + step + D2H per
step), the FP64 throughput of the same kernels, the FP32-vs-FP64 L1 density
error at t = 0.05, the roofline of the kernel and the CPU baseline (the
oracle, a NumPy restatement of the reference, timed on this host).

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

N_CELLS = 512
METRIC = "zone-updates/s on 1 GB300, FP32 fused vs plain FP64, at L1 err <=1e-5 vs FP64"
WORKLOAD = "Orszag-Tang 2D MHD, FV HLL + Pang-Wu split (constrained B), MINMOD, SSP-RK2, 512x512 periodic, gamma 5/3"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_CELLS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-arena", action="store_true", help="skip the 256^3 blast comparison")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 64-run batched ensemble")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the 128^3 adjoint workload")
    ap.add_argument("--no-gravity", action="store_true", help="skip the self-gravity collapse workload")
    ap.add_argument("--case", default=None, choices=["fd", "fdsrc", "fv3d", "fvsplit", "ensemble", "adjoint",
                                                     "gravity"],
                    help="run one small case of a secondary workload and exit (for profilers)")
    return ap.parse_args()


def run_case(name):
    """Small, self-contained runs of the secondary workloads for ncu captures:
    fd: FD WENO-CT blast 128^3 FP32, 2 steps; fv3d: FV Lax-Friedrichs MHD
    blast 192^3 FP32, 2 steps (one launch); fvsplit: the same blast with the
    split MUSCL-Hancock scheme and HLLC; ensemble: 8 turbulent 2D MHD
    runs (128^2..512^2, t_end / 8) in one batched launch; adjoint: the 3D
    density-perturbation problem at 96^3 to t = 0.01, forward and backward
    with the stored tape (a 4 GB tape budget: the case holds a few GB at
    most); gravity: Evrard's collapse at 128^3 FP32, 3 steps of the
    self-gravity step sequence; fdsrc: the FD blast at 128^3 FP32 with
    turbulent forcing and the stellar-wind source, 2 steps."""
    import torch
    from astronomix_gb300 import _native

    if name in ("fd", "fv3d", "fvsplit"):
        from astronomix_gb300.time_integration import get_plan

        cfg, prm, rv, s = arena_blast(128 if name == "fd" else 192, "fv_split" if name == "fvsplit" else name[:2])
        plan = get_plan(cfg, rv, s.shape, np.float32)
        dev = torch.from_numpy(s).cuda()
        st = torch.cuda.current_stream().cuda_stream
        plan.reset(st)
        info = plan.run(dev.data_ptr(), _native.make_params(prm), 2, st)
        print(json.dumps({"case": name, "steps": info.steps, "status": info.status}))
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


def fd_precision(n=128, t_end=0.02, flop_per_zu=44e3):
    """FD WENO-CT on the MHD blast of the FD workload (periodic unit cube,
    rho = 1, p = 10 inside r < 0.1 and 0.1 outside, B = (1, 1, 0)/sqrt 2,
    C_cfl 1.5, SSPRK(5,4)) at n^3 to t_end in FP32 and FP64 with the same
    kernels: s/step of each, their ratio, and the relative L1 density error
    of FP32 against FP64.  The FD kernel's compute roof is the measured FP32
    FMA rate; `flop_per_zu` is the estimated arithmetic per zone-update of
    the scheme (eigensystem once per interface, 7 characteristic fields)."""
    import torch
    from _cases import blast_fd
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan

    st = torch.cuda.current_stream()
    out = {"grid": [n, n, n], "t_end": t_end}
    res = {}
    for name, dt in (("fp32", np.float32), ("fp64", np.float64)):
        cfg, prm, rv, s = blast_fd(n=n, dtype=dt, t_end=t_end)
        s = s.astype(dt)
        plan = get_plan(cfg, rv, s.shape, dt)
        p = _native.make_params(prm)
        dev = torch.from_numpy(s).cuda()
        plan.reset(st.cuda_stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        info = plan.run(dev.data_ptr(), p, 1 << 40, st.cuda_stream)
        b.record(st)
        torch.cuda.synchronize()
        res[name] = dev[0].double()
        out[name] = {"steps": info.steps, "s_per_step": a.elapsed_time(b) / 1e3 / max(1, info.steps),
                     "status": info.status}
        del dev
    out["fp32_over_fp64"] = out["fp64"]["s_per_step"] / out["fp32"]["s_per_step"]
    out["l1_err_vs_fp64"] = float((res["fp32"] - res["fp64"]).abs().sum() / res["fp64"].abs().sum())
    peak = _native.probe_fp32_fma(st.cuda_stream)
    zu_s = n ** 3 / out["fp32"]["s_per_step"]
    out["compute_roof"] = {"fp32_fma_tflops_measured": peak, "flop_per_zone_update_estimate": flop_per_zu,
                           "achieved_tflops_estimate": zu_s * flop_per_zu / 1e12,
                           "frac": zu_s * flop_per_zu / 1e12 / peak}
    return out


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
    out = {"runs": num_runs, "grids": sorted(set(s[-1] for s in shapes)), "cells_total": sum(s[-1] * s[-2] for s in shapes),
           "zone_updates": zu, "seconds": sec, "zone_updates_per_s": zu / sec, "lock_steps": lock,
           "magnetic_iterations_mean": iters, "tiling": tiling, "tune_s": tune_s, "graph": True, "ok": ok,
           "launches": 2}
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
    whole initial state by the discrete adjoint, FP32.  Times the plain
    forward, and forward + backward with the tape stored by the forward and
    with checkpoints every `checkpoint_every` steps; checks the gradient
    against central finite differences of the replayed program on the density
    and pressure rows and against the FP64 adjoint of the same problem.  The
    problem's initial state (v = 0, uniform p) stays at the kink of the
    MINMOD limiter in v and p (their slopes are exactly zero), where no
    finite difference reproduces a gradient; the same checks are repeated on
    a smooth variant with velocity and pressure perturbed (0.1 x GRF)."""
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
    x = torch.from_numpy(s).cuda()
    tgt = torch.from_numpy(target).cuda().double()
    out = {"grid": [n, n, n]}
    # the plain forward: the ordinary plan, no tape, no checkpoints
    plan = get_plan(cfg, rv, s.shape, np.float32)
    p = _native.make_params(prm)
    for _ in range(2):
        xp = x.clone()
        plan.reset(stream.cuda_stream)
        a, b = ev(), ev()
        a.record(stream)
        plan.run(xp.data_ptr(), p, 1 << 40, stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
    plain_s = a.elapsed_time(b) / 1e3
    out["plain_forward_s"] = plain_s
    for mode, budget in (("stored_tape", "auto"), ("checkpoints", 0)):
        integ = AdjointIntegrator(cfg, prm, rv, s.shape, np.float32, checkpoint_every=checkpoint_every,
                                  tape_budget=budget)
        L, grad, fwd_s, fb_s = timed(integ, x, tgt)
        dts, its = integ.schedule()
        out[mode] = {"stored": integ.stored_tape(), "forward_s": fwd_s, "forward_plus_backward_s": fb_s,
                     "ratio_over_plain_forward": fb_s / plain_s, "memory_bytes": integ.memory()}
        if mode == "checkpoints":
            out[mode]["checkpoint_every"] = checkpoint_every
            out["steps"] = len(dts)
            out["magnetic_iterations_mean"] = float(np.mean(its)) if its else 0.0
            out["loss"] = L
            out["fd_check"] = _fd_check(integ, x, grad, tgt, directions, eps, rows=(0, 4))
        del integ
    # FP32 vs FP64 adjoint, and the smooth variant
    if fp64:
        cfg64, prm64, rv64, s64, _ = density_perturbation_problem(n, dtype=np.float64)
        integ64 = AdjointIntegrator(cfg64, prm64, rv64, s64.shape, np.float64, tape_budget="auto")
        y64 = integ64.forward(torch.from_numpy(s64).cuda())
        g64 = integ64.backward(_loss_grad(y64, tgt)[1])
        rows = [0, 4]
        num = torch.linalg.norm(grad[rows].double() - g64[rows])
        out["fp64_grad_rel_l2_err"] = float(num / torch.linalg.norm(g64[rows]))
        del integ64, y64, g64
        xs = torch.from_numpy(smooth(s.copy(), np.float32)).cuda()
        integ = AdjointIntegrator(cfg, prm, rv, s.shape, np.float32, tape_budget="auto")
        ys = integ.forward(xs)
        gs = integ.backward(_loss_grad(ys, tgt)[1])
        fd = _fd_check(integ, xs, gs, tgt, max(4, directions // 2), eps, rows=(0, 1, 2, 3, 4))
        del integ
        integ64 = AdjointIntegrator(cfg64, prm64, rv64, s64.shape, np.float64, tape_budget="auto")
        y64 = integ64.forward(torch.from_numpy(smooth(s64.copy(), np.float64)).cuda())
        g64 = integ64.backward(_loss_grad(y64, tgt)[1])
        rows = [0, 1, 2, 3, 4]
        err = float(torch.linalg.norm(gs[rows].double() - g64[rows]) / torch.linalg.norm(g64[rows]))
        out["smooth_variant"] = {"fd_check": fd, "fp64_grad_rel_l2_err": err,
                                 "steps": len(integ64.schedule()[0])}
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


def cpu_baseline_oracle(budget_s=15.0, n=128):
    """The oracle (NumPy restatement of the reference) on a bounded sample: OT n^2, FP32."""
    from _cases import orszag_tang
    from oracle import driver

    cfg, prm, rv, s = orszag_tang(n=n, t_end=10.0, dtype=np.float32)
    P = s
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        P = driver.time_integration(P, cfg, prm, rv, max_steps=1)
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": n * n * steps / dt, "unit": "zone-updates/s", "cores": 1, "kind": "port",
            "sample": "oracle (NumPy restatement) OT %dx%d FP32, %d steps in %.1f s" % (n, n, steps, dt)}


def _reference_replica(job):
    """One host process of the reference arm: OT n^2 FP32 advanced by the
    oracle one step at a time, `steps` steps or `budget` seconds."""
    n, steps, budget = job
    from _cases import orszag_tang
    from oracle import driver

    cfg, prm, rv, s = orszag_tang(n=n, t_end=10.0, dtype=np.float32)
    P = driver.time_integration(s, cfg, prm, rv, max_steps=1)  # warm-up step
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        P = driver.time_integration(P, cfg, prm, rv, max_steps=1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    return done, time.perf_counter() - t0


def run_reference(args, rank, world):
    """--impl reference: the oracle port of the reference's CPU path on this
    host, one independent replica per host core (processes started with
    spawn, one NumPy thread each); value = the replicas' summed throughput."""
    if rank != 0:
        return
    import multiprocessing as mp

    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    budget = 60.0
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_reference_replica, [(args.n, args.steps, budget)] * cores)
    v = sum(args.n * args.n * d / t for d, t in res)
    steps = min(d for d, _ in res)
    ms = 1e3 * sum(t / d for d, t in res) / len(res)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [args.n, args.n], "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": cores, "kind": "port",
                         "sample": "%d replicas x %d steps of OT %dx%d (each bounded to %.0f s)" % (
                             cores, steps, args.n, args.n, budget)},
        "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args, rank, world):
    import torch

    from _cases import orszag_tang
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan

    dev_index = torch.cuda.current_device()
    n = args.n
    cfg, prm, rv, s = orszag_tang(n=n, t_end=1e9, dtype=np.float32)
    p = _native.make_params(prm)
    plan = get_plan(cfg, rv, s.shape, np.float32)
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    state = torch.from_numpy(s).cuda()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    plan.reset(st)

    # warm-up: W steps, one launch each
    for _ in range(max(args.warmup, 3)):
        plan.run_async(state.data_ptr(), p, 1, st)
    torch.cuda.synchronize()
    it0 = plan.run(state.data_ptr(), p, 0, st)

    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev_index) as clk:
        for i in range(K):
            flush.zero_()
            starts[i].record(stream)
            plan.run_async(state.data_ptr(), p, 1, st)
            ends[i].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    it1 = plan.run(state.data_ptr(), p, 0, st)
    k_mean = (it1.magnetic_iterations - it0.magnetic_iterations) / max(1, it1.steps - it0.steps)
    status = it1.status
    from astronomix_gb300.replicas import replica_throughput

    value = replica_throughput(n * n * K, total_s)
    total_s_max = max_over_ranks(total_s, world)

    # ---- fused multi-step throughput (K steps in one launch, L2-resident state)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan.run_async(state.data_ptr(), p, K, st)
    e1.record(stream)
    torch.cuda.synchronize()
    fused_ms = e0.elapsed_time(e1)

    # ---- end to end through the C ABI with host buffers (pinned)
    host = torch.from_numpy(s.copy()).pin_memory()
    host_out = torch.empty_like(host).pin_memory()
    dev2 = torch.empty_like(state)
    nbytes = host.numel() * host.element_size()
    Ke = max(10, min(K, 100))
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
    e2e_s = sum(a.elapsed_time(b) for a, b in zip(es, ee)) / 1e3
    e2e_value = replica_throughput(n * n * Ke, e2e_s)

    # ---- FP64: same kernels, plain double precision
    cfg64, prm64, rv64, s64 = orszag_tang(n=n, t_end=1e9, dtype=np.float64)
    plan64 = get_plan(cfg64, rv64, s64.shape, np.float64)
    st64 = torch.from_numpy(s64).cuda()
    plan64.reset(st)
    for _ in range(3):
        plan64.run_async(st64.data_ptr(), p, 1, st)
    K64 = max(5, K // 10)
    t64 = []
    for _ in range(K64):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        plan64.run_async(st64.data_ptr(), p, 1, st)
        b.record(stream)
        t64.append((a, b))
    torch.cuda.synchronize()
    fp64_s = sum(a.elapsed_time(b) for a, b in t64) / 1e3
    fp64_value = n * n * K64 / fp64_s

    # ---- accuracy: FP32 vs FP64 density at t = 0.05 from the same initial state
    t_cmp = 0.05
    cfgA, prmA, rvA, sA = orszag_tang(n=n, t_end=t_cmp, dtype=np.float32)
    cfgB, prmB, rvB, sB = orszag_tang(n=n, t_end=t_cmp, dtype=np.float64)
    a32 = torch.from_numpy(sA).cuda()
    a64 = torch.from_numpy(sB).cuda()
    pa, pb = _native.make_params(prmA), _native.make_params(prmB)
    planA = get_plan(cfgA, rvA, sA.shape, np.float32)
    planB = get_plan(cfgB, rvB, sB.shape, np.float64)
    planA.reset(st)
    planB.reset(st)
    infoA = planA.run(a32.data_ptr(), pa, 1 << 40, st)
    infoB = planB.run(a64.data_ptr(), pb, 1 << 40, st)
    r32 = a32[0].double()
    r64 = a64[0]
    l1 = float((r32 - r64).abs().sum() / r64.abs().sum())

    # ---- roofline of the dominant (only) kernel: fv_run_kernel
    bpz = algorithmic_bytes_per_zone_update(k_mean)
    launch_s = total_s / K
    achieved = bpz * n * n / launch_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    traffic = load_traffic("fv_run_kernel_ot512_fp32_step")

    arena = {}
    if not args.no_arena:
        arena = {"fd_blast_fp32": time_arena("fd"), "fv_lf_blast_fp32": time_arena("fv"),
                 "fd_blast_fp32_vs_fp64": fd_precision(), "fd_blast_forcing_wind_fp32": time_fd_sources(),
                 "fv_split_hllc_blast_fp32": time_arena("fv_split")}
        arena["fd_blast_forcing_wind_fp32"]["overhead_vs_plain"] = (
            arena["fd_blast_forcing_wind_fp32"]["s_per_step"] / arena["fd_blast_fp32"]["s_per_step"] - 1.0)
    ensemble = None if args.no_ensemble else time_ensemble()
    adjoint = None if args.no_adjoint else time_adjoint()
    gravity = None if args.no_gravity else time_gravity()

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline_oracle()
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
        "config": {"workload": WORKLOAD, "grid": [n, n], "precision": "fp32 fields, fp64 dt/time",
                   "l2": "flushed between timed steps (512 MB write); state 7.3 MB",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e_value, "unit": "zone-updates/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": K,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "note": "algorithmic %.0f B/zone-update (k=%.2f fixed-point iterations), peak %s" % (
                         bpz, k_mean, peak_src)},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "fp64_value": fp64_value,
        "fp32_over_fp64": value / fp64_value,
        "l1_err_vs_fp64": l1,
        "l1_t": t_cmp,
        "l1_steps": [infoA.steps, infoB.steps],
        "fused_multistep_value": n * n * K / (fused_ms / 1e3),
        "magnetic_iterations_mean": k_mean,
        "reference_published_workloads": arena,
        "ensemble_fp32": ensemble,
        "adjoint_fp32": adjoint,
        "self_gravity_fp32": gravity,
        "status": status,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.case:
        run_case(args.case)
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
