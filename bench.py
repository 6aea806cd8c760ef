#!/usr/bin/env python
"""Benchmark of the PyMiniWeather time step on GB300.

Workload: the collision case on an 8192 x 4096 grid (two cos^2 bubbles of
+-20 K, 20 km x 10 km, cfl 1.5, max_speed 450).  One step is one full time
step: two directions x three RK stages = six fused direction-stage kernel
launches over the whole grid.  The state (1.07 GB per FP64 array) is far
larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The headline is the IEEE-FP64 form (f64_mode "fp64": every floating-point
operation an IEEE FP64 add, multiply or FMA), timed over K calls of the public
step (evolve -> mw_step_f64).  The per-kernel figures of the roofline come from
a second pass that issues the step's six launches one by one through
mw_dirstage_f64 (the same kernels on the same arrays) with an event after each.
The other forms are reported on the same line: "fp64_dw" (the split form:
FP64 storage, double-FP32 arithmetic of ~47 significant bits -- not IEEE
FP64), "fp64_native" (IEEE FP64 with the reference's formulas as written),
"fp32", the ensemble and adjoint forms, the host-buffer end-to-end step, the
error each form runs at against the oracle, and the CPU baselines.

Prints one JSON line (rank 0).  Under torchrun each rank advances its own
replica (the step has no exchange on one GPU); value = cell-steps of all ranks
per second of the slowest rank.

--impl reference times the CPU restatement of the reference's algorithm (the
oracle, a C port of the NumPy code) on all host cores, on the same workload.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import os
import platform
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
# FP64 operations the GB300 SM retires per clock (DFMA, DADD or DMUL; the
# profiler's peak_sustained for sm__sass_thread_inst_executed_op_dfma_pred_on).
FP64_OPS_PER_CLOCK_PER_SM = 2.0

DTYPES = {
    "fp32": "f32 perturbation fields (FP64 backgrounds, IC and reductions)",
    "fp64": "f64",
    "native": "f64",
    "split": "f64 storage and update, double-FP32 interior arithmetic (~47-bit significand, FP32 exponent range; "
             "not IEEE FP64)",
}
KERNELS = {
    "fp64": {0: "k_stage_x_ieee_w", 1: "k_stage_z_ieee"},
    "split": {0: "k_stage_x_split", 1: "k_stage_z_split"},
    "native": {0: "k_stage_x<double,NATIVE64>", 1: "k_stage_z<double,NATIVE64>"},
    "fp32": {0: "k_stage_x_f32_bulk", 1: "k_stage_z_f32_bulk"},
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nx", type=int, default=8192)
    ap.add_argument("--nz", type=int, default=4096)
    ap.add_argument("--ic", default="collision")
    ap.add_argument("--mode", default="fp64", choices=["fp64", "split", "native", "fp32"],
                    help="form of the headline: an FP64 form (default: fp64, IEEE FP64) or fp32 (the "
                         "precision form; for profiling)")
    ap.add_argument("--no-extras", action="store_true", help="headline only (no other forms, e2e or CPU legs)")
    ap.add_argument("--cpu-steps", type=int, default=2, help="time steps in the oracle CPU-baseline sample")
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


def load_profile_table():
    """Per-kernel DRAM bytes and FP64 operations per cell from the committed ncu summaries."""
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


ARM_PARTS = {"0xd4f": "Arm Neoverse V2", "0xd40": "Arm Neoverse V1", "0xd0c": "Arm Neoverse N1",
             "0xd8e": "Arm Neoverse N3", "0xd84": "Arm Neoverse V3"}


def cpu_model():
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu part")):
                    name = line.split(":", 1)[1].strip()
                    return "%s (%s, %s)" % (ARM_PARTS[name], name, platform.machine()) if name in ARM_PARTS else name
    except Exception:
        pass
    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
def make_params(nx, nz, ic, mode="fp64"):
    p = dict(nx=nx, nz=nz, xlen=2e4, zlen=1e4, hs=2, s=4, ic_type=ic, cfl=1.5, max_speed=450.0)
    p["dx"] = p["xlen"] / p["nx"]
    p["dz"] = p["zlen"] / p["nz"]
    p["dt"] = min(p["dx"], p["dz"]) * p["cfl"] / p["max_speed"]
    p["f64_mode"] = mode
    return p


class StageRunner:
    """Issues a time step stage by stage through the C ABI -- the six launches
    mw_step_* makes, with the same storage formats (the split form keeps its
    first RK stage's result as pairs: MW_FLAG_PAIRS_OUT / _IN) -- recording a
    CUDA event on the launching stream after each launch."""

    def __init__(self, torch, native, p, f):
        self.torch, self.n, self.p, self.f = torch, native, p, f
        self.reverse = 0
        self.fp64 = f.dtype == torch.float64
        self.mode = native.F64_MODES[p["f64_mode"]]
        self.hb = [native.ptr(a) for a in f.backgrounds()]
        self.stream = native.stream_handle(f.device)
        self.S, self.T, self.A = native.ptr(f.state), native.ptr(f.state_tmp), native.ptr(f.scratch)

    def stage(self, init, forcing, out, dts, d, k):
        n, p, f = self.n, self.p, self.f
        args = (f.nx, f.nz, p["dx"], p["dz"], p["dt"], *self.hb, None, init, forcing, out, dts, d)
        if self.fp64:
            flags = n.MW_FLAG_WRITE_HALO
            if self.mode == n.MW_F64_SPLIT:
                flags |= (n.MW_FLAG_PAIRS_OUT, n.MW_FLAG_PAIRS_IN, 0)[k]
            n.call("mw_dirstage_f64", *args, self.mode, flags, self.stream)
        else:
            n.call("mw_dirstage_f32", *args, n.MW_FLAG_WRITE_HALO, self.stream)

    def step(self, events=None):
        dt = self.p["dt"]
        dirs = (0, 1) if self.reverse else (1, 0)
        for d in dirs:
            for k, (init, forcing, out, dts) in enumerate(((self.S, self.S, self.A, dt / 3),
                                                           (self.S, self.A, self.T, dt / 2),
                                                           (self.S, self.T, self.S, dt / 1))):
                self.stage(init, forcing, out, dts, d, k)
                if events is not None:
                    e = self.torch.cuda.Event(enable_timing=True)
                    e.record()
                    events.append((d, e))
        self.reverse ^= 1


def stage_pass(torch, native, p, f, steps, warmup, dist=None):
    """Warm up, then time `steps` steps launch by launch; per direction the
    list of launch durations (ms)."""
    r = StageRunner(torch, native, p, f)
    for _ in range(warmup):
        r.step()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e0.record()
    events = []
    for _ in range(steps):
        r.step(events)
    torch.cuda.synchronize()
    per = {0: [], 1: []}
    prev = e0
    for d, e in events:
        per[d].append(prev.elapsed_time(e))
        prev = e
    return per


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


def roofline(per, cells, bytes_per_value, peak, peak_kind, names, table, sm_mhz=None):
    """HBM roofline of the dominant kernel (algorithmic bytes per launch over
    its average CUDA-event launch time), with the other direction's kernel and,
    where the profile table has its FP64 operation count, the FP64-pipe figure."""
    tot = {d: sum(v) for d, v in per.items()}
    d = max(tot, key=tot.get)
    algo = cells * bytes_per_value * sum(VALUES_PER_STAGE) / 3.0

    def one(dd):
        avg = tot[dd] / len(per[dd])
        name = names[dd]
        tr = table.get(name, {})
        out = {"kernel": name, "avg_launch_ms": round(avg, 4),
               "achieved": round(algo / (avg * 1e-3) / 1e9, 1), "frac": round(algo / (avg * 1e-3) / 1e9 / peak, 4)}
        if tr.get("dram_bytes_per_cell") is not None:
            out["traffic"] = cells * tr["dram_bytes_per_cell"] * bytes_per_value / 8
        if tr.get("fp64_ops_per_cell") is not None and sm_mhz:
            ops = tr["fp64_ops_per_cell"] * cells / (avg * 1e-3)
            pk = FP64_OPS_PER_CLOCK_PER_SM * 152 * sm_mhz * 1e6
            out["fp64_pipe"] = {"achieved_gops": round(ops / 1e9, 1), "peak_gops": round(pk / 1e9, 1),
                                "frac": round(ops / pk, 4), "ops_per_cell": tr["fp64_ops_per_cell"]}
        return out

    dom, other = one(d), one(1 - d)
    rl = {"bound": "hbm", "kernel": dom["kernel"], "achieved": dom["achieved"], "peak": peak, "unit": "GB/s",
          "frac": dom["frac"], "peak_kind": peak_kind, "traffic": dom.get("traffic"),
          "algorithmic_bytes_per_launch": algo, "avg_launch_ms": dom["avg_launch_ms"],
          "share": round(tot[d] / sum(tot.values()), 3), "other_kernel": other}
    if "fp64_pipe" in dom:
        rl["fp64_pipe"] = dom["fp64_pipe"]
    return rl


def fp64_probe(torch, native, dev, repeats=5):
    """FP64 pipe throughput of this GPU, measured: mw_fp64_throughput (8
    independent FMA chains per thread, 4 CTAs of 256 threads per SM), the
    median of `repeats` runs of ~75 ms each with the SM clock sampled meanwhile.
    The denominator of fp64_pipe.frac_of_measured."""
    import ctypes
    out = ctypes.c_double(0.0)
    clocks = ClockSampler(device_id_for_smi(torch, dev))
    clocks.start()
    vals = []
    for _ in range(repeats):
        native.call("mw_fp64_throughput", 4, 2000, ctypes.byref(out), native.stream_handle())
        vals.append(out.value / 1e9)
    clk = clocks.stop()
    return {"gops": round(statistics.median(vals), 1), "runs": [round(v, 1) for v in vals], "clocks": clk,
            "kernel": "mw_fp64_throughput: 4 x 152 CTAs x 256 threads, 8 independent FP64 FMA chains per thread"}


def with_measured_fp64(rl, probe):
    """Adds the fraction of the measured FP64 pipe throughput to every
    fp64_pipe block of a roofline dict."""
    for blk in (rl.get("fp64_pipe"), rl.get("other_kernel", {}).get("fp64_pipe")):
        if blk and probe and probe.get("gops"):
            blk["peak_measured_gops"] = probe["gops"]
            blk["frac_of_measured"] = round(blk["achieved_gops"] / probe["gops"], 4)
    return rl


def e2e_run(torch, p, f, steps, warmup, dist=None):
    """Public API with host buffers: per step, evolve_host() copies the state in
    from pinned host memory, advances it and copies it back out (the FP64 forms
    "fp64" and "split" overlap the copies with the step by row bands).  Under
    torchrun the ranks start together and the caller takes the slowest rank's
    time."""
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
    return ms, nbytes, host_link(torch, f.state, h_in, h_out)


def host_link(torch, dev, h_in, h_out, reps=3):
    """Pinned host <-> device copy rates of one state array (GB/s, best of
    `reps`, each direction alone): the floor under the host-buffer step, which
    differs between boxes."""
    out = {}
    for name, dst, src in (("h2d", dev, h_in), ("d2h", h_out, dev)):
        best = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = max(best, src.numel() * src.element_size() / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        out[name] = round(best, 1)
    return out


def form_leg(torch, native, args, mode, dtype, peak, peak_kind, table, sm_mhz, steps, warmup):
    """One more form on the same workload: public-step timing plus the
    launch-by-launch roofline pass."""
    from pyminiweather_gb300.data import initialize_fields
    from pyminiweather_gb300.ics import init
    cells = args.nx * args.nz
    p = make_params(args.nx, args.nz, args.ic, mode)
    f = initialize_fields(p, dtype=dtype)
    init(f, p)
    ms = step_run(torch, p, f, steps, warmup)
    init(f, p)
    per = stage_pass(torch, native, p, f, steps, warmup)
    fp64 = dtype == torch.float64
    names = KERNELS[mode if fp64 else "fp32"]
    out = {"value": job_value(1, cells, steps, ms), "ms_per_step": ms / steps, "steps": steps,
           "dtype": DTYPES[mode] if fp64 else "f32 perturbation fields (FP64 backgrounds, IC and reductions)",
           "roofline": roofline(per, cells, 8 if fp64 else 4, peak, peak_kind, names, table, sm_mhz)}
    out["roofline"]["public_step_frac"] = round(
        cells * STATE_VALUES_PER_CELL_STEP * (8 if fp64 else 4) / (ms / steps * 1e-3) / 1e9 / peak, 4)
    del f
    torch.cuda.empty_cache()
    return out


def ensemble_run(torch, steps, warmup, dtype, mode, peak, ops_per_cell_stage=None, probe=None):
    """The batching form: 256 thermal members of uneven sizes (nx log-uniform in
    [64, 1024]), autotuned, two steps per CUDA-graph replay.  For the IEEE-FP64
    form also the FP64-pipe rate, from the single-grid kernels' operation
    counts per cell-stage (the ensemble kernels run the same arithmetic)."""
    from pyminiweather_gb300.ensemble import Ensemble, thermal_ensemble
    ens = Ensemble(thermal_ensemble(256, seed=0), dtype=dtype, f64_mode=mode)
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
    value = ens.cells() * n / (ms * 1e-3)
    bpc = STATE_VALUES_PER_CELL_STEP * (8 if dtype == torch.float64 else 4)
    out = {"value": value, "unit": UNIT, "ms_per_step": ms / n, "steps": n, "members": ens.n_members(),
           "cells": ens.cells(), "cuda_graph": True,
           "dtype": DTYPES[mode] if dtype == torch.float64 else "f32",
           # FP64 forms: + the row-constant table, once per replay of 2 steps
           "launches_per_step": 6.5 if dtype == torch.float64 else 6,
           "roofline": {"bound": "hbm", "bytes_per_cell_step": bpc, "achieved": round(value * bpc / 1e9, 1),
                        "peak": peak, "unit": "GB/s", "frac": round(value * bpc / 1e9 / peak, 4)},
           "tuning": {k: tuned[k] for k in ("z_tile", "grid_x", "grid_z")}}
    if ops_per_cell_stage:
        gops = value * 6 * ops_per_cell_stage / 1e9
        out["roofline"]["fp64_pipe"] = {"achieved_gops": round(gops, 1), "ops_per_cell_stage": ops_per_cell_stage}
        if probe and probe.get("gops"):
            out["roofline"]["fp64_pipe"].update(peak_measured_gops=probe["gops"],
                                                frac_of_measured=round(gops / probe["gops"], 4))
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
    p = make_params(512, 256, "thermal", mode)
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


def gpu_states_for_err(torch, nx, nz, ic, steps):
    """GPU states of every form after `steps` steps of the same case (for the
    error leg, which compares them with the oracle)."""
    from pyminiweather_gb300.data import initialize_fields
    from pyminiweather_gb300.ics import init
    from pyminiweather_gb300.solve import evolve, reset_direction
    out = {}
    for key, mode, dtype in (("fp64", "fp64", torch.float64), ("fp64_native", "native", torch.float64),
                             ("fp64_dw", "split", torch.float64), ("fp32", "fp64", torch.float32)):
        p = make_params(nx, nz, ic, mode)
        f = initialize_fields(p, dtype=dtype)
        init(f, p)
        reset_direction()
        evolve(p, f, None, dt=p["dt"], nsteps=steps)
        out[key] = f.state.to(torch.float64).cpu().numpy()
        del f
    torch.cuda.empty_cache()
    return out


def cpu_baselines(args, steps, gpu_err_states, err_case):
    """The CPU legs, all on the host cores of this machine: (1) the oracle (C port
    of the reference's NumPy code, OpenMP on every core) timed on `steps` full
    time steps of the workload; (2) the oracle as the checker of every GPU form
    on a smaller case run 200 steps (the error the metric is stated at);
    (3) the reference's own NumPy path (evolve, pyminiweather/solve/step.py:85),
    single-threaded, if it is installed next to this file (baseline/_ref)."""
    import numpy as np

    from oracle import oracle as O
    threads = os.cpu_count() or 1
    p = O.make_params(args.nx, args.nz, args.ic)
    t0 = time.perf_counter()
    sim = O.OracleSim(p, threads=threads)
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    sim.evolve(steps)
    dt = time.perf_counter() - t0
    base = {"value": args.nx * args.nz * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d full time steps of the %dx%d %s case (oracle C port, OpenMP, %d threads; init %.1f s "
                      "untimed)" % (steps, args.nx, args.nz, args.ic, threads, t_init),
            "seconds": round(dt, 3)}
    del sim
    # (2) error of every form against the oracle
    nx, nz, ic, nst = err_case
    o = O.OracleSim(O.make_params(nx, nz, ic), threads=threads)
    o.evolve(nst)
    ref = o.state
    err = {"case": "%s %dx%d after %d steps, against the oracle (pinned to the reference's own outputs); "
                   "per-variable normwise max|a-b|/max|b| over the interior" % (ic, nx, nz, nst),
           "bar": {"fp64": 1e-10, "fp32_rel_l2": 1e-4}}
    for key, st in gpu_err_states.items():
        a, b = st[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]
        nw = [float(np.abs(a[v] - b[v]).max() / np.abs(b[v]).max()) for v in range(4)]
        if key == "fp32":
            l2 = [float(np.linalg.norm(a[v] - b[v]) / np.linalg.norm(b[v])) for v in (0, 3)]
            err[key] = {"rel_l2_dens": l2[0], "rel_l2_rhot": l2[1], "max_normwise": max(nw)}
        else:
            err[key] = {"max_normwise": max(nw), "per_variable": nw}
    return base, err, numpy_reference_baseline()


def numpy_reference_baseline():
    """The reference NumPy path itself, timed on this machine's host (one core: the
    path is single-threaded SciPy convolve and NumPy ufuncs)."""
    ref_root = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref_root, "pyminiweather")):
        return {"unavailable": "the reference package is not installed at baseline/_ref"}
    try:
        import numpy as np
        os.environ.pop("LEGATE_MAX_DIM", None)
        os.environ.pop("LEGATE_MAX_FIELDS", None)
        sys.path.insert(0, ref_root)
        with contextlib.redirect_stdout(sys.stderr):  # it prints its backend on import
            import pyminiweather  # noqa: F401
            from pyminiweather.data import initialize_fields
            from pyminiweather.ics import init
            from pyminiweather.mesh import MeshData
            from pyminiweather.solve import step as S
    except Exception as e:  # numpy / scipy missing on this host
        return {"unavailable": "the reference cannot be imported here: %s" % str(e).splitlines()[0]}
    out = {"kind": "reference", "cores": 1, "cores_present": os.cpu_count(), "cpu": cpu_model(),
           "impl": "pyminiweather (NumPy %s, SciPy convolve) evolve, pyminiweather/solve/step.py:85" % np.__version__}
    for key, (nx, nz, ic, nsteps) in (("config0", (100, 50, "thermal", 200)),
                                      ("collision_1024x512", (1024, 512, "collision", 2))):
        p = make_params(nx, nz, ic)
        p.pop("f64_mode")
        p.update(nsteps=nsteps, nwarmups=0, output_freq=-1)
        with contextlib.redirect_stdout(sys.stderr):
            f = initialize_fields(p)
            m = MeshData(p)
            init(f, p, m)
            S.reverse_direction = False
            t0 = time.perf_counter()
            for _ in range(nsteps):
                S.evolve(p, f, m, dt=p["dt"])
            sec = time.perf_counter() - t0
        out[key] = {"value": nx * nz * nsteps / sec, "unit": UNIT, "seconds": round(sec, 3),
                    "sample": "%s %dx%d, %d time steps" % (ic, nx, nz, nsteps)}
    return out


def config_dict(args):
    return {"workload": "%s %dx%d, 20 km x 10 km, cfl 1.5, max_speed 450; 1 step = 2 directions x 3 RK stages"
                        % (args.ic, args.nx, args.nz),
            "nx": args.nx, "nz": args.nz, "ic_type": args.ic,
            "l2": "inputs larger than L2 (1.07 GB per FP64 state array vs 129 MB L2); no flush",
            "parallelism": "replicas (one independent grid per GPU)"}


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
            "config": config_dict(args),
            "implementation": "the oracle: a C restatement of the reference's NumPy step in its operation order, "
                              "OpenMP over rows, %d threads on %s" % (threads, cpu_model()),
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
    table = load_profile_table()
    cells = args.nx * args.nz
    f32 = args.mode == "fp32"
    p = make_params(args.nx, args.nz, args.ic, "fp64" if f32 else args.mode)
    f = initialize_fields(p, dtype=torch.float32 if f32 else torch.float64)
    vbytes = 4 if f32 else 8
    init(f, p)
    torch.cuda.synchronize()
    m0 = compute_stats(p, f)[0]

    clocks = ClockSampler(device_id_for_smi(torch, dev))
    clocks.start()
    ms = step_run(torch, p, f, args.steps, args.warmup, dist)
    clk = clocks.stop()
    ms = replica_max(torch, ms, dist, "cuda")
    m1 = compute_stats(p, f)[0]
    value = job_value(world, cells, args.steps, ms)
    if f32 and not args.no_extras:
        raise SystemExit("--mode fp32 is a profiling headline: use it with --no-extras")
    if not args.no_extras:
        # end to end through the public API with host buffers (on the headline's fields)
        init(f, p)
        clocks_e = ClockSampler(device_id_for_smi(torch, dev))
        clocks_e.start()
        ms_e, nbytes, link = e2e_run(torch, p, f, args.steps, args.warmup, dist)
        clk_e = clocks_e.stop()
        ms_e = replica_max(torch, ms_e, dist, "cuda")
        e2e_line = {"value": job_value(world, cells, args.steps, ms_e), "unit": UNIT,
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "ms_per_step": ms_e / args.steps, "api": "pyminiweather_gb300.solve.evolve_host",
                    "f64_mode": args.mode, "clocks": clk_e, "host_link_gbs": link,
                    "copies_back_to_back_ms": round(nbytes / (link["h2d"] * 1e6) + nbytes / (link["d2h"] * 1e6), 3)
                    if link["h2d"] and link["d2h"] else None}
    # per-kernel durations: the step's six launches issued one by one through
    # the C ABI (same kernels, same arrays, same storage formats), an event after each
    init(f, p)
    per = stage_pass(torch, _native, p, f, args.steps, args.warmup, dist)
    rl = roofline(per, cells, vbytes, peak, peak_kind, KERNELS[args.mode], table, clk.get("sm_mhz"))
    rl["kernel_timing"] = "the public step's six launches issued one by one (mw_dirstage_f64), CUDA events on the " \
                          "launching stream"
    step_gbs = cells * STATE_VALUES_PER_CELL_STEP * vbytes / (ms / args.steps * 1e-3) / 1e9
    rl["public_step"] = {"achieved": round(step_gbs, 1), "frac": round(step_gbs / peak, 4),
                         "note": "%d algorithmic B per cell-step over the public step's time"
                                 % (STATE_VALUES_PER_CELL_STEP * vbytes)}
    probe = fp64_probe(torch, _native, dev) if rl.get("fp64_pipe") or not args.no_extras else None
    with_measured_fp64(rl, probe)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES[args.mode],
            "data": "synthetic (the reference's analytic collision initial condition)",
            "config": config_dict(args), "f64_mode": args.mode,
            "roofline": rl, "clocks": clk, "gpu_launches": 6 * args.steps,
            "mass_drift": (m1 - m0) / m0, "bytes_per_cell_step": STATE_VALUES_PER_CELL_STEP * vbytes}
    if probe:
        line["fp64_peak_measured"] = probe
    if rl.get("fp64_pipe"):
        line["limiter"] = ("FP64 pipe (dominant kernel at %.0f %% of its nominal peak, %.0f %% of the measured FMA "
                           "throughput; HBM %.0f %%)" % (100 * rl["fp64_pipe"]["frac"],
                                                        100 * rl["fp64_pipe"].get("frac_of_measured", 0),
                                                        100 * rl["frac"]))
    if not args.no_extras:
        line["e2e"] = e2e_line

    del f
    torch.cuda.empty_cache()
    if not args.no_extras and world == 1:
        sm_mhz = clk.get("sm_mhz")
        # the other FP64 forms and FP32 on the same workload
        legs = [("fp64_dw", "split", torch.float64, args.steps), ("fp64_native", "native", torch.float64, 2),
                ("fp64", "fp64", torch.float64, args.steps), ("fp32", "fp64", torch.float32, args.steps)]
        for key, mode, dtype, ks in legs:
            if dtype == torch.float64 and mode == args.mode:
                continue
            line[key] = form_leg(torch, _native, args, mode, dtype, peak, peak_kind, table, sm_mhz, ks,
                                 1 if ks < 3 else args.warmup)
            with_measured_fp64(line[key]["roofline"], probe)
        line["fp32"]["speedup_vs_fp64"] = line["fp32"]["value"] / (value if args.mode == "fp64"
                                                                   else line["fp64"]["value"])
        if "fp64_dw" in line:
            line["fp32"]["speedup_vs_fp64_dw"] = line["fp32"]["value"] / line["fp64_dw"]["value"]
        # the batching form (ensemble of uneven grids)
        ieee_ops = [table.get(KERNELS["fp64"][d], {}).get("fp64_ops_per_cell") for d in (0, 1)]
        ieee_ops = round(sum(ieee_ops) / 2, 2) if all(ieee_ops) else None
        line["ensemble"] = {"fp64": ensemble_run(torch, args.steps, args.warmup, torch.float64, "fp64", peak,
                                                 ieee_ops, probe),
                            "fp64_dw": ensemble_run(torch, args.steps, args.warmup, torch.float64, "split", peak),
                            "fp32": ensemble_run(torch, args.steps, args.warmup, torch.float32, "fp64", peak)}
        # the differentiation form: adjoint / forward cost
        line["adjoint"] = {"fp64": adjoint_run(torch, "fp64"), "fp64_dw": adjoint_run(torch, "split"),
                           "fp64_native": adjoint_run(torch, "native")}
        # CPU legs (oracle timing, the error leg's checker, the reference NumPy path)
        err_case = (1024, 512, args.ic, 200)
        states = gpu_states_for_err(torch, *err_case)
        line["cpu_baseline"], line["err"], line["cpu_baseline_numpy"] = cpu_baselines(args, args.cpu_steps, states,
                                                                                      err_case)
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
