#!/usr/bin/env python
"""Benchmark of the PyMiniWeather time step on GB300.

Workload: the collision case on an 8192 x 4096 grid in FP64 (two cos^2
bubbles of +-20 K, 20 km x 10 km, cfl 1.5, max_speed 450).  One step is one
full time step: two directions x three RK stages = six fused direction-stage
kernel launches over the whole grid.  The state (1.07 GB per array) is far
larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The headline times K calls of the public step (evolve -> mw_step_f64, which
keeps the first RK stage's result of each direction as double-FP32 pairs); the
per-kernel figures of the roofline come from a second pass that issues the same
six launches stage by stage through mw_dirstage_f64 with an event after each.

Prints one JSON line (rank 0).  Under torchrun each rank advances its own
replica (the step has no exchange on one GPU); value = cell-steps of all ranks
per second of the slowest rank.

--impl reference times the CPU restatement of the reference's algorithm (the
oracle port; the reference itself is NumPy code that cannot travel here) on
all host cores, on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-steps/s FP64 vs FP32 at 8192x4096 at stated err; %HBM peak; adjoint/fwd"
UNIT = "cell-steps/s"
# Compulsory state traffic of one direction-stage in values per cell: stage 1
# reads 4 (init is the forcing) and writes 4; stages 2 and 3 read 8, write 4.
VALUES_PER_STAGE = (8, 12, 12)
STATE_VALUES_PER_CELL_STEP = 2 * sum(VALUES_PER_STAGE)  # 64


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nx", type=int, default=8192)
    ap.add_argument("--nz", type=int, default=4096)
    ap.add_argument("--ic", default="collision")
    ap.add_argument("--mode", default="fp64", choices=["fp64", "split", "native"])
    ap.add_argument("--no-extras", action="store_true", help="skip the FP32 / native-FP64 / e2e / CPU legs")
    ap.add_argument("--cpu-steps", type=int, default=2, help="time steps in the CPU-baseline sample")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_max(torch, ms, dist, device):
    """The slowest rank's time: every rank advances its own replica, so the job
    ends when the last one does."""
    if dist is None:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, cells, steps, ms):
    """Whole-job cell-steps/s: all ranks' cells over the slowest rank's time."""
    return world * cells * steps / (ms * 1e-3)


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic():
    """Per-kernel DRAM bytes per cell per launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, device_id: str):
        self.device_id = device_id
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="mw_clocks_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.device_id, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        with open(self.path) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(self.NAMES, parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def device_id_for_smi(torch, dev):
    try:
        return "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        return str(dev)


# ---------------------------------------------------------------------------
def make_params(args, dtype_name="fp64"):
    p = dict(nx=args.nx, nz=args.nz, xlen=2e4, zlen=1e4, hs=2, s=4, ic_type=args.ic, cfl=1.5, max_speed=450.0)
    p["dx"] = p["xlen"] / p["nx"]
    p["dz"] = p["zlen"] / p["nz"]
    p["dt"] = min(p["dx"], p["dz"]) * p["cfl"] / p["max_speed"]
    p["f64_mode"] = args.mode
    return p


class StageRunner:
    """Issues a time step stage by stage through the C ABI (the same six
    launches mw_step_* makes), recording CUDA events between launches."""

    def __init__(self, torch, native, p, f):
        self.torch, self.n, self.p, self.f = torch, native, p, f
        self.reverse = 0
        self.fp64 = f.dtype == torch.float64
        self.mode = native.F64_MODES[p["f64_mode"]]
        self.hb = [native.ptr(a) for a in f.backgrounds()]
        self.stream = native.stream_handle(f.device)
        self.S, self.T, self.A = native.ptr(f.state), native.ptr(f.state_tmp), native.ptr(f.scratch)

    def stage(self, init, forcing, out, dts, d):
        n, p, f = self.n, self.p, self.f
        args = (f.nx, f.nz, p["dx"], p["dz"], p["dt"], *self.hb, None, init, forcing, out, dts, d)
        if self.fp64:
            n.call("mw_dirstage_f64", *args, self.mode, n.MW_FLAG_WRITE_HALO, self.stream)
        else:
            n.call("mw_dirstage_f32", *args, n.MW_FLAG_WRITE_HALO, self.stream)

    def step(self, events=None):
        dt = self.p["dt"]
        dirs = (0, 1) if self.reverse else (1, 0)
        for d in dirs:
            for (init, forcing, out, dts) in ((self.S, self.S, self.A, dt / 3), (self.S, self.A, self.T, dt / 2),
                                              (self.S, self.T, self.S, dt / 1)):
                self.stage(init, forcing, out, dts, d)
                if events is not None:
                    e = self.torch.cuda.Event(enable_timing=True)
                    e.record()
                    events.append((d, e))
        self.reverse ^= 1


def timed_run(torch, native, p, f, steps, warmup, dist=None):
    """Warm up, then time exactly `steps` steps; returns (ms_total, per-kernel stats)."""
    r = StageRunner(torch, native, p, f)
    for _ in range(warmup):
        r.step()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e0.record()
    events = []
    for _ in range(steps):
        r.step(events)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(events[-1][1])
    per = {0: [], 1: []}
    prev = e0
    for d, e in events:
        per[d].append(prev.elapsed_time(e))
        prev = e
    return ms, per, 6 * steps


def step_run(torch, p, f, steps, warmup, dist=None):
    """Warm up, then time exactly `steps` calls of the public step (evolve ->
    mw_step_f64 / mw_step_f32, one time step each); returns ms_total."""
    from pyminiweather_gb300.solve import evolve, reset_direction
    reset_direction()
    for _ in range(warmup):
        evolve(p, f, None, dt=p["dt"], nsteps=1)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        evolve(p, f, None, dt=p["dt"], nsteps=1)
    e1.record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    return e0.elapsed_time(e1)


def kernel_names(fp64, mode):
    if not fp64:
        return {0: "k_stage_x<float,F32>", 1: "k_stage_z<float,F32>"}
    if mode == "split":
        return {0: "k_stage_x_split", 1: "k_stage_z_split"}
    if mode == "fp64":
        return {0: "k_stage_x_ieee", 1: "k_stage_z_ieee"}
    return {0: "k_stage_x<double,NATIVE64>", 1: "k_stage_z<double,NATIVE64>"}


def roofline(per, cells, bytes_per_value, peak, peak_kind, names, traffic_table):
    tot = {d: sum(v) for d, v in per.items()}
    d = max(tot, key=tot.get)
    avg_ms = tot[d] / len(per[d])
    algo = cells * bytes_per_value * sum(VALUES_PER_STAGE) / 3.0
    achieved = algo / (avg_ms * 1e-3) / 1e9
    name = names[d]
    tr = traffic_table.get(name)
    traffic = cells * tr["dram_bytes_per_cell"] if tr else None
    return {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo, "avg_launch_ms": round(avg_ms, 4),
            "share": round(tot[d] / sum(tot.values()), 3),
            "other_kernel": {"kernel": names[1 - d], "avg_launch_ms": round(tot[1 - d] / len(per[1 - d]), 4),
                             "frac": round(algo / (tot[1 - d] / len(per[1 - d]) * 1e-3) / 1e9 / peak, 4)}}


def e2e_run(torch, p, f, steps, warmup, dist=None):
    """Public API with host buffers: per step, evolve_host() copies the state in
    from pinned host memory, advances it and copies it back out (the FP64 split
    form overlaps the copies with the step by row bands).  Under torchrun the
    ranks start together and the caller takes the slowest rank's time."""
    from pyminiweather_gb300.solve import evolve_host, reset_direction
    h_in = torch.empty(f.state.shape, dtype=f.dtype, pin_memory=True)
    h_out = torch.empty(f.state.shape, dtype=f.dtype, pin_memory=True)
    h_in.copy_(f.state)
    reset_direction()
    for _ in range(warmup):
        evolve_host(p, f, h_in, h_out, dt=p["dt"])
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        evolve_host(p, f, h_in, h_out, dt=p["dt"])
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    nbytes = f.state.numel() * f.state.element_size()
    return ms, nbytes


def ensemble_run(torch, steps, warmup, dtype):
    """The batching form: 256 thermal members of uneven sizes (nx log-uniform in
    [64, 1024]), autotuned, two steps per CUDA-graph replay."""
    from pyminiweather_gb300.ensemble import Ensemble, thermal_ensemble
    ens = Ensemble(thermal_ensemble(256, seed=0), dtype=dtype)
    tuned = ens.autotune(steps=1)
    replay = ens.graph()
    for _ in range(max(1, (warmup + 1) // 2)):
        replay()
    torch.cuda.synchronize()
    reps = max(1, (steps + 1) // 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        replay()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    n = 2 * reps
    out = {"value": ens.cells() * n / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / n, "steps": n,
           "members": ens.n_members(), "cells": ens.cells(), "cuda_graph": True,
           "launches_per_step": 6.5 if dtype == torch.float64 else 6,  # FP64: + the row-constant table, once per replay of 2 steps
           "tuning": {k: tuned[k] for k in ("z_tile", "grid_x", "grid_z")}}
    del ens
    torch.cuda.empty_cache()
    return out


def adjoint_run(torch, mode):
    """The differentiation form: 512 x 256 thermal, 200 steps, checkpoints every
    20; forward (the rollout) and adjoint (checkpoint replay + reverse sweep)
    timed with CUDA events."""
    from pyminiweather_gb300.adjoint import RolloutContext, rollout, upper_half_rhot_misfit
    from pyminiweather_gb300.data import initialize_fields
    from pyminiweather_gb300.ics import init
    p = dict(nx=512, nz=256, xlen=2e4, zlen=1e4, hs=2, s=4, ic_type="thermal", cfl=1.5, max_speed=450.0)
    p["dx"], p["dz"] = p["xlen"] / 512, p["zlen"] / 256
    p["dt"] = min(p["dx"], p["dz"]) * 1.5 / 450.0
    p["f64_mode"] = mode
    f = initialize_fields(p)
    init(f, p)
    target = f.state.clone() * 1.001
    ctx = RolloutContext(params=p, fields=f, nsteps=200, ckpt_every=20)
    res = []
    for _ in range(2):  # the first pass warms up
        x0 = f.state.clone().requires_grad_(True)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        loss = upper_half_rhot_misfit(rollout(x0, ctx), target, 256)
        ev[1].record()
        (g,) = torch.autograd.grad(loss, x0)
        ev[2].record()
        ev[2].synchronize()
        res = [ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])]
    del f, g
    torch.cuda.empty_cache()
    return {"grid": "512x256", "steps": 200, "ckpt_every": 20, "f64_mode": mode, "forward_ms": res[0],
            "adjoint_ms": res[1], "ratio": res[1] / res[0]}


def cpu_baseline(args, steps):
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    p = O.make_params(args.nx, args.nz, args.ic)
    t0 = time.perf_counter()
    sim = O.OracleSim(p, threads=threads)
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    sim.evolve(steps)
    dt = time.perf_counter() - t0
    return {"value": args.nx * args.nz * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d full time steps of the %dx%d %s case (oracle C port, OpenMP, %d threads; init %.1f s "
                      "untimed)" % (steps, args.nx, args.nz, args.ic, threads, t_init),
            "seconds": round(dt, 3)}


def config_dict(args, extra=None):
    c = {"workload": "%s %dx%d, 20 km x 10 km, cfl 1.5, max_speed 450; 1 step = 2 directions x 3 RK stages"
                     % (args.ic, args.nx, args.nz),
         "nx": args.nx, "nz": args.nz, "ic_type": args.ic, "f64_mode": args.mode,
         "l2": "inputs larger than L2 (1.07 GB per FP64 state array vs 129 MB L2); no flush",
         "parallelism": "replicas (one independent grid per GPU)"}
    if extra:
        c.update(extra)
    return c


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    p = O.make_params(args.nx, args.nz, args.ic)
    sim = O.OracleSim(p, threads=threads)
    for _ in range(args.warmup):
        sim.evolve(1)
    t0 = time.perf_counter()
    sim.evolve(args.steps)
    sec = time.perf_counter() - t0
    value = args.nx * args.nz * args.steps / sec
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the reference's analytic collision initial condition)",
            "config": config_dict(args, {"f64_mode": "reference formulas, FP64 (C port of the NumPy code)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d full time steps of the %dx%d %s case after %d warm-up steps"
                                       % (args.steps, args.nx, args.nz, args.ic, args.warmup)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group(backend="nccl", device_id=torch.device("cuda", local))
        dist = tdist
    else:
        torch.cuda.set_device(0)
    from pyminiweather_gb300 import _native
    from pyminiweather_gb300.data import initialize_fields
    from pyminiweather_gb300.ics import init
    from pyminiweather_gb300.post import compute_stats

    dev = torch.cuda.current_device()
    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    cells = args.nx * args.nz
    p = make_params(args)
    f = initialize_fields(p, dtype=torch.float64)
    init(f, p)
    torch.cuda.synchronize()
    m0 = compute_stats(p, f)[0]

    clocks = ClockSampler(device_id_for_smi(torch, dev))
    clocks.start()
    ms = step_run(torch, p, f, args.steps, args.warmup, dist)
    clk = clocks.stop()
    ms = replica_max(torch, ms, dist, "cuda")
    m1 = compute_stats(p, f)[0]
    launches = 6 * args.steps
    value = job_value(world, cells, args.steps, ms)
    # per-kernel durations: the same six launches a step makes, issued stage by
    # stage through the C ABI with an event after each (every stage in FP64
    # storage there; the step keeps its first RK stage's result as pairs)
    init(f, p)
    _, per, _ = timed_run(torch, _native, p, f, args.steps, args.warmup, dist)
    rl = roofline(per, cells, 8, peak, peak_kind, kernel_names(True, args.mode), traffic)
    rl["kernel_timing"] = "stage-by-stage C-ABI pass, FP64 storage in every stage"
    step_gbs = cells * STATE_VALUES_PER_CELL_STEP * 8 / (ms / args.steps * 1e-3) / 1e9
    rl["public_step"] = {"achieved": round(step_gbs, 1), "frac": round(step_gbs / peak, 4),
                         "note": "512 algorithmic B per cell-step over the public step's time"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.mode == "native" else "f64 storage/update, f32x2 arithmetic",
            "data": "synthetic (the reference's analytic collision initial condition)",
            "config": config_dict(args), "roofline": rl, "clocks": clk, "gpu_launches": launches,
            "mass_drift": (m1 - m0) / m0,
            "bytes_per_cell_step": STATE_VALUES_PER_CELL_STEP * 8}

    if not args.no_extras and world > 1:
        # several GPUs: the end-to-end leg only (the other forms are single-GPU figures)
        init(f, p)
        ms_e, nbytes = e2e_run(torch, p, f, args.steps, 1, dist)
        ms_e = replica_max(torch, ms_e, dist, "cuda")
        line["e2e"] = {"value": job_value(world, cells, args.steps, ms_e), "unit": UNIT,
                       "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                       "ms_per_step": ms_e / args.steps, "api": "pyminiweather_gb300.solve.evolve_host",
                       "f64_mode": args.mode}
    elif not args.no_extras:
        # end to end through the public API with host buffers (first, on the headline's fields)
        init(f, p)
        ms_e, nbytes = e2e_run(torch, p, f, args.steps, 1)
        line["e2e"] = {"value": job_value(world, cells, args.steps, ms_e), "unit": UNIT,
                       "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                       "ms_per_step": ms_e / args.steps, "api": "pyminiweather_gb300.solve.evolve_host",
                       "f64_mode": args.mode}
        # FP32 precision form on the same workload
        del f
        torch.cuda.empty_cache()
        f32 = initialize_fields(p, dtype=torch.float32)
        init(f32, p)
        ms32 = step_run(torch, p, f32, args.steps, args.warmup, None)
        init(f32, p)
        _, per32, _ = timed_run(torch, _native, p, f32, args.steps, args.warmup, None)
        v32 = job_value(world, cells, args.steps, ms32)
        line["fp32"] = {"value": v32, "ms_per_step": ms32 / args.steps, "speedup_vs_fp64": v32 / value,
                        "roofline": roofline(per32, cells, 4, peak, peak_kind, kernel_names(False, "split"), traffic)}
        del f32
        torch.cuda.empty_cache()
        # the other FP64 form (a few steps)
        other = "native" if args.mode == "split" else "split"
        po = dict(p, f64_mode=other)
        fo = initialize_fields(po, dtype=torch.float64)
        init(fo, po)
        ks = max(1, min(args.steps, 3))
        mso = step_run(torch, po, fo, ks, 1, None)
        init(fo, po)
        _, pero, _ = timed_run(torch, _native, po, fo, ks, 1, None)
        line["fp64_" + other] = {"value": job_value(world, cells, ks, mso), "ms_per_step": mso / ks,
                                 "roofline": roofline(pero, cells, 8, peak, peak_kind, kernel_names(True, other),
                                                      traffic)}
        # the batching form (ensemble of uneven grids), FP64 split and FP32
        line["ensemble"] = {"fp64": ensemble_run(torch, args.steps, args.warmup, torch.float64),
                            "fp32": ensemble_run(torch, args.steps, args.warmup, torch.float32)}
        # the differentiation form: adjoint / forward cost
        line["adjoint"] = {"split": adjoint_run(torch, "split"), "native": adjoint_run(torch, "native")}
        del fo
        torch.cuda.empty_cache()
        line["cpu_baseline"] = cpu_baseline(args, args.cpu_steps)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
