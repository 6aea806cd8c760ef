"""Ensembles of uneven grids advanced together on one GPU.

No counterpart in the reference, which runs one grid per process: here many
members -- each a full simulation with its own nx, nz, dx, dz, dt and initial
bubbles -- share three flat state buffers and advance with one persistent
kernel launch per direction-stage (six per step) walking a work list over all
members (mw_ensemble_step_*).  `graph()` captures two steps (both direction
orders) in a CUDA graph; `autotune()` picks the z tile height and the
persistent grid sizes by timing candidates on the ensemble itself.

Each member runs the arithmetic of `solve.evolve` on its own grid (the same
tile code); FP64 members (f64_mode "fp64", IEEE FP64, the default, or
"split") agree with single-grid runs of the same form to rounding level, FP32
members to FP32 rounding.  Members take no forcing term (no gravity-wave case).
"""
from __future__ import annotations

import ctypes
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .ics.initial_conditions import ic_spec

_TUNING_CACHE: Dict[tuple, dict] = {}


def member_params(nx: int, nz: int, ic_type: str = "thermal", xlen: float = 2e4, zlen: float = 1e4,
                  cfl: float = 1.5, max_speed: float = 450.0) -> dict:
    p = dict(nx=int(nx), nz=int(nz), xlen=xlen, zlen=zlen, hs=2, s=4, ic_type=ic_type, cfl=cfl,
             max_speed=max_speed)
    p["dx"] = xlen / nx
    p["dz"] = zlen / nz
    p["dt"] = min(p["dx"], p["dz"]) * cfl / max_speed
    return p


def thermal_ensemble(n: int = 256, seed: int = 0, nx_range: Tuple[int, int] = (64, 1024)) -> List[tuple]:
    """Members of the uneven thermal-bubble ensemble: nx log-uniform in
    nx_range rounded to an even integer (nz = nx / 2), 20 km x 10 km, bubble
    amplitude U[1, 5] K at x0 = U[0.3, 0.7] xlen, z0 = U[1.5, 3] km, radius
    2 km.  Returns [(params, bubbles)]; numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(nx_range[0]), math.log(nx_range[1])
    out = []
    for _ in range(n):
        nx = int(2 * round(math.exp(rng.uniform(lo, hi)) / 2))
        nx = min(max(nx, nx_range[0]), nx_range[1])
        p = member_params(nx, nx // 2)
        amp = rng.uniform(1.0, 5.0)
        x0 = rng.uniform(0.3, 0.7) * p["xlen"]
        z0 = rng.uniform(1500.0, 3000.0)
        out.append((p, [(amp, x0, z0, 2000.0, 2000.0)]))
    return out


class Ensemble:
    """Members [(params, bubbles or None)] in shared flat buffers on one GPU."""

    def __init__(self, members: Sequence[tuple], dtype=torch.float64, f64_mode: str = "fp64", device=None,
                 z_tile: int = 64):
        if dtype not in (torch.float64, torch.float32):
            raise TypeError("dtype must be torch.float64 or torch.float32")
        if dtype == torch.float64 and f64_mode not in ("fp64", "split"):
            raise ValueError("ensembles with FP64 storage run f64_mode 'fp64' (IEEE FP64) or 'split'")
        self.f64_mode = f64_mode if dtype == torch.float64 else None
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise ValueError("ensembles live on a CUDA device")
        self.dtype = dtype
        self.params = [dict(m[0]) for m in members]
        self.bubbles = [m[1] if len(m) > 1 else None for m in members]
        for p in self.params:
            if p["ic_type"] == "gravity":
                raise ValueError("ensemble members take no forcing term (gravity-wave case)")
        n = len(self.params)
        specs = (_native.EnsMember * n)()
        so = co = io = 0
        for e, p in enumerate(self.params):
            nx, nz = p["nx"], p["nz"]
            specs[e] = _native.EnsMember(nx, nz, p["dx"], p["dz"], p["dt"], so, co, io)
            so += 4 * (nx + 4) * (nz + 4)
            co += nz + 4
            io += nz + 1
        self.specs = specs
        z = lambda k, dt: torch.zeros(k, dtype=dt, device=self.device)
        self.state, self.state_tmp, self.scratch = z(so, dtype), z(so, dtype), z(so, dtype)
        self.hy_dens_cell, self.hy_dens_theta_cell = z(co, torch.float64), z(co, torch.float64)
        self.hy_dens_int, self.hy_dens_theta_int, self.hy_pressure_int = (z(io, torch.float64) for _ in range(3))
        self.reverse = 0
        self.grid_x = self.grid_z = 0
        self._init_members()
        self._build_plan(z_tile)
        self._graph = None
        self._stats_ws = None

    # -- layout -------------------------------------------------------------------------------
    def n_members(self) -> int:
        return len(self.params)

    def cells(self) -> int:
        return int(sum(p["nx"] * p["nz"] for p in self.params))

    def _views(self, buf, e):
        s = self.specs[e]
        n = 4 * (s.nx + 4) * (s.nz + 4)
        return buf[s.state_off:s.state_off + n].view(4, s.nz + 4, s.nx + 4)

    def member_state(self, e: int) -> torch.Tensor:
        return self._views(self.state, e)

    def member_state_tmp(self, e: int) -> torch.Tensor:
        return self._views(self.state_tmp, e)

    def member_backgrounds(self, e: int):
        s = self.specs[e]
        c = slice(s.cell_off, s.cell_off + s.nz + 4)
        i = slice(s.int_off, s.int_off + s.nz + 1)
        return (self.hy_dens_cell[c], self.hy_dens_theta_cell[c], self.hy_dens_int[i], self.hy_dens_theta_int[i],
                self.hy_pressure_int[i])

    def backgrounds(self):
        return (self.hy_dens_cell, self.hy_dens_theta_cell, self.hy_dens_int, self.hy_dens_theta_int,
                self.hy_pressure_int)

    def _init_members(self):
        fn = "mw_init_f64" if self.dtype == torch.float64 else "mw_init_f32"
        stream = _native.stream_handle(self.device)
        for e, p in enumerate(self.params):
            spec = ic_spec(p["ic_type"], p["xlen"])
            bub = spec.bubbles if self.bubbles[e] is None else [tuple(float(v) for v in b) for b in self.bubbles[e]]
            host = np.ascontiguousarray(np.array(bub, dtype=np.float64).reshape(-1)) if bub else None
            hptr = host.ctypes.data_as(ctypes.c_void_p) if host is not None else None
            bg = [_native.ptr(a) for a in self.member_backgrounds(e)]
            _native.call(fn, p["nx"], p["nz"], float(p["xlen"]), float(p["zlen"]), spec.background, float(spec.u0),
                         len(bub), hptr, _native.ptr(self.member_state(e)), *bg, stream)
        self.state_tmp.copy_(self.state)

    def _build_plan(self, z_tile: int):
        info = _native.EnsPlanInfo()
        n = self.n_members()
        _native.call("mw_ensemble_plan_info", n, self.specs, int(z_tile), ctypes.byref(info))
        plan = torch.empty((info.bytes + 15) // 16 * 2, dtype=torch.float64, device=self.device)
        _native.call("mw_ensemble_plan", n, self.specs, int(z_tile), _native.ptr(plan), plan.numel() * 8,
                     ctypes.byref(info), _native.stream_handle(self.device))
        self.plan, self.info, self.z_tile = plan, info, int(z_tile)

    # -- stepping -----------------------------------------------------------------------------
    def step(self, nsteps: int = 1) -> None:
        """Advance every member by nsteps time steps of its own dt."""
        rv = ctypes.c_int(self.reverse)
        hb = [_native.ptr(a) for a in self.backgrounds()]
        args = [_native.ptr(self.plan), ctypes.byref(self.info), *hb, _native.ptr(self.state),
                _native.ptr(self.state_tmp), _native.ptr(self.scratch), int(nsteps), ctypes.byref(rv)]
        stream = _native.stream_handle(self.device)
        if self.dtype == torch.float64:
            _native.call("mw_ensemble_step_f64", *args, _native.F64_MODES[self.f64_mode], _native.MW_FLAG_WRITE_HALO,
                         self.grid_x, self.grid_z, stream)
        else:
            _native.call("mw_ensemble_step_f32", *args, _native.MW_FLAG_WRITE_HALO, self.grid_x, self.grid_z, stream)
        self.reverse = rv.value

    def _form(self) -> int:
        """The kernel form of mw_ensemble_occupancy: 0 FP64 split, 1 FP32, 2 IEEE FP64."""
        if self.dtype == torch.float32:
            return 1
        return 2 if self.f64_mode == "fp64" else 0

    def default_grids(self) -> Tuple[int, int]:
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        out = []
        for d in (_native.MW_DIR_X, _native.MW_DIR_Z):
            b = ctypes.c_int(0)
            _native.call("mw_ensemble_occupancy", self._form(), d, ctypes.byref(b))
            out.append(max(1, b.value) * sms)
        return out[0], out[1]

    def graph(self):
        """Capture two steps (both direction orders) in a CUDA graph; returns a
        callable that replays them (advancing two steps).  Valid while the
        step parity at replay equals the parity at capture."""
        if self.grid_x <= 0 or self.grid_z <= 0:
            self.grid_x, self.grid_z = self.default_grids()
        start = self.reverse
        snap = [self.state.clone(), self.state_tmp.clone()]
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):  # warm-up outside capture
            self.step(2)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(2)
        self.state.copy_(snap[0])
        self.state_tmp.copy_(snap[1])
        self.reverse = start
        torch.cuda.synchronize(self.device)
        self._graph = g

        def replay():
            if self.reverse != start:
                raise RuntimeError("graph captured at a different step parity")
            g.replay()
        return replay

    # -- tuning -------------------------------------------------------------------------------
    def autotune(self, z_tiles=(16, 32, 64), steps: int = 2, verbose: bool = False) -> dict:
        """Pick the z tile height and the persistent grid sizes by timing
        candidates on this ensemble (state restored afterwards)."""
        key = (self.dtype, self.f64_mode, tuple((p["nx"], p["nz"]) for p in self.params),
               torch.cuda.get_device_name(self.device))
        if key in _TUNING_CACHE:
            self._apply(_TUNING_CACHE[key])
            return _TUNING_CACHE[key]
        snap = [self.state.clone(), self.state_tmp.clone(), self.reverse]
        bx, bz = self.default_grids()
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        cands = []
        for zt in z_tiles:
            for gx in sorted({bx, max(sms, bx // 2), 2 * bx}):
                for gz in sorted({bz, max(sms, bz // 2), 2 * bz}):
                    cands.append(dict(z_tile=zt, grid_x=gx, grid_z=gz))
        best, best_ms = None, float("inf")
        results = []
        for c in cands:
            self._apply(c)
            self.step(1)
            torch.cuda.synchronize(self.device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.step(steps)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            results.append((ms, c))
            if ms < best_ms:
                best, best_ms = c, ms
        self.state.copy_(snap[0])
        self.state_tmp.copy_(snap[1])
        self.reverse = snap[2]
        best = dict(best, ms_per_step=best_ms, candidates=len(cands))
        if verbose:
            for ms, c in sorted(results, key=lambda r: r[0])[:5]:
                print("  %.3f ms  %s" % (ms, c))
        _TUNING_CACHE[key] = best
        self._apply(best)
        return best

    def _apply(self, c):
        if c["z_tile"] != self.z_tile:
            self._build_plan(c["z_tile"])
        self.grid_x, self.grid_z = int(c["grid_x"]), int(c["grid_z"])
        self._graph = None

    # -- diagnostics --------------------------------------------------------------------------
    def member_stats(self, e: int) -> Tuple[float, float]:
        p = self.params[e]
        need = int(_native.load().mw_stats_workspace_bytes(p["nx"], p["nz"]))
        if self._stats_ws is None or self._stats_ws.numel() * 8 < need + 16:
            self._stats_ws = torch.empty(max(need // 8 + 2, 2050), dtype=torch.float64, device=self.device)
        ws = self._stats_ws
        hb = self.member_backgrounds(e)
        fn = "mw_stats_f64" if self.dtype == torch.float64 else "mw_stats_f32"
        _native.call(fn, p["nx"], p["nz"], float(p["dx"]), float(p["dz"]), _native.ptr(hb[0]), _native.ptr(hb[1]),
                     _native.ptr(self.member_state(e)), _native.ptr(ws[2:]), (ws.numel() - 2) * 8,
                     _native.ptr(ws[:2]), _native.stream_handle(self.device))
        m, en = ws[:2].tolist()
        return m, en
