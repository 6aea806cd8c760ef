"""Time stepping: the GPU counterpart of pyminiweather/solve/step.py:18-143.

evolve() advances the state by whole time steps through mw_step_* (six fused
direction-stage launches per step).  discrete_step() runs one direction-stage
through mw_dirstage_*.  Both write the halo cells of each forcing array as
set_bc_x / set_bc_z do, so `fields.state` and `fields.state_tmp` hold, halo
included, what the reference leaves in them.

The direction order alternates from step to step through the module-global
flag `reverse_direction`, as in the reference (step.py:18,103-109,143): the
first step after import runs z then x.  reset_direction() restores that.

FP64 arithmetic mode (params["f64_mode"], default DEFAULT_F64_MODE):
  "fp64"   - IEEE FP64 arithmetic throughout, with the fewest FP64 operations
             (1/rho by a Newton step, the pressure perturbation by its
             binomial series, values scaled by 12 so that no cell divides);
  "native" - IEEE FP64 with the reference's formulas as written (a pow and
             three divides per interface);
  "split"  - NOT IEEE FP64: FP64 loads, stores and stage update, interior
             arithmetic in pairs of FP32 (about 47 significant bits, FP32
             exponent range).  GB300 retires FP64 at 1/64 of the FP32 rate, so
             this form is ~3.5x faster than "fp64"; its error after 200 steps
             at 8192 x 4096 is ~4e-13 normwise, but it is narrower arithmetic
             than the reference's, so it is never the default.
"""
from __future__ import annotations

import ctypes
from typing import Dict

import torch

from .. import _native
from ..ics.directions import Directions

reverse_direction: bool = False
DEFAULT_F64_MODE = "fp64"


def reset_direction(value: bool = False) -> None:
    """Set the direction flag (False: the next step runs z then x)."""
    global reverse_direction
    reverse_direction = bool(value)


def f64_mode(params: Dict) -> int:
    mode = params.get("f64_mode", DEFAULT_F64_MODE)
    if mode not in _native.F64_MODES:
        raise ValueError("f64_mode must be one of %s" % sorted(_native.F64_MODES))
    return _native.F64_MODES[mode]


def _check_state(fields, t, name):
    return _native.require_cuda(t, name, dtype=fields.dtype, shape=fields.shape)


def _dirstage(params, fields, init, forcing, out, dt, direction: int, flags: int):
    hb = [_native.ptr(a) for a in fields.backgrounds()]
    args = (fields.nx, fields.nz, float(params["dx"]), float(params["dz"]), float(params["dt"]), *hb,
            _native.ptr(fields.src_w), _native.ptr(init), _native.ptr(forcing), _native.ptr(out), float(dt), direction)
    if fields.dtype == torch.float64:
        _native.call("mw_dirstage_f64", *args, f64_mode(params), flags, _native.stream_handle(fields.device))
    else:
        _native.call("mw_dirstage_f32", *args, flags, _native.stream_handle(fields.device))


def discrete_step(params: Dict, fields, mesh, state_init, state_forcing, state_out, dt: float,
                  direction: Directions) -> None:
    """One direction-stage: state_out = state_init + dt * tend(state_forcing).

    Like the reference it writes the halo of state_forcing; state_out may be
    the same array as state_forcing (stage 2 of the reference's RK3) -- the
    kernel then writes fields.scratch and the interior is copied over.
    """
    for t, n in ((state_init, "state_init"), (state_forcing, "state_forcing"), (state_out, "state_out")):
        _check_state(fields, t, n)
    d = _native.MW_DIR_X if direction == Directions.X else _native.MW_DIR_Z
    if params.get("ic_type") == "injection":
        raise NotImplementedError("the injection case is flagged unsupported by the reference")
    flags = _native.MW_FLAG_WRITE_HALO
    if state_out.data_ptr() == state_forcing.data_ptr():
        tmp = fields.scratch
        if tmp.data_ptr() in (state_init.data_ptr(), state_forcing.data_ptr()):
            tmp = torch.empty_like(tmp)
        _dirstage(params, fields, state_init, state_forcing, tmp, dt, d, flags)
        h = fields.hs
        state_out[:, h:-h, h:-h].copy_(tmp[:, h:-h, h:-h])
    else:
        _dirstage(params, fields, state_init, state_forcing, state_out, dt, d, flags)


def evolve(params: Dict, fields, mesh=None, dt: float = 1e-4, nsteps: int = 1) -> None:
    """Advance fields.state by nsteps time steps of size dt (step.py:85-143).

    Hyperviscosity uses params["dt"], as in the reference.  With
    params["check_finite"] the state is checked for NaN / Inf after the steps
    (synchronising) and MiniWeatherError with status MW_ERR_NONFINITE is raised.
    """
    global reverse_direction
    _check_state(fields, fields.state, "fields.state")
    _check_state(fields, fields.state_tmp, "fields.state_tmp")
    _check_state(fields, fields.scratch, "fields.scratch")
    if params.get("ic_type") == "injection":
        raise NotImplementedError("the injection case is flagged unsupported by the reference")
    rv = ctypes.c_int(1 if reverse_direction else 0)
    hb = [_native.ptr(a) for a in fields.backgrounds()]
    args = [fields.nx, fields.nz, float(params["dx"]), float(params["dz"]), float(params["dt"]), float(dt), *hb,
            _native.ptr(fields.src_w), _native.ptr(fields.state), _native.ptr(fields.state_tmp),
            _native.ptr(fields.scratch), int(nsteps), ctypes.byref(rv)]
    flags = params.get("step_flags", _native.MW_FLAG_WRITE_HALO)
    if params.get("check_finite"):  # blocking: raises MiniWeatherError (status 7) on NaN / Inf
        flags |= _native.MW_FLAG_CHECK_FINITE
    if fields.dtype == torch.float64:
        _native.call("mw_step_f64", *args, f64_mode(params), flags, _native.stream_handle(fields.device))
    else:
        _native.call("mw_step_f32", *args, flags, _native.stream_handle(fields.device))
    reverse_direction = bool(rv.value)


# Row bands of the host-buffer step (GB300, 8192 x 4096 collision, measured):
# the x stages of a band run on a second stream beside the z stages of the
# others, so the short banded launches fill each other's tails, and both forms
# do best with 32 bands: the split form is bound by the copies (9.3 ms per
# step), the IEEE-FP64 form by its compute (20.4 ms against 19.4 ms for the
# step alone; 22.0 ms in 8 bands, 29.9 ms unbanded).
HOST_STEP_BANDS = {"split": 32, "fp64": 32}


def evolve_host(params: Dict, fields, h_in: torch.Tensor, h_out: torch.Tensor, dt: float = 1e-4,
                nbands: int = None) -> None:
    """One time step of a state held in host memory: h_in (a CPU tensor of the
    state's shape, ideally pinned) is copied into fields.state, the step runs as
    evolve() would run it, and the new state is copied into h_out (may be
    h_in).  The FP64 forms "fp64" and "split" overlap the copies with the step
    by row bands (mw_step_f64_host; nbands None: the form's default,
    HOST_STEP_BANDS); other forms copy, step and copy.  Returns once the work
    is enqueued on the current stream; synchronise before reading h_out."""
    global reverse_direction
    for name, h in (("h_in", h_in), ("h_out", h_out)):
        if not isinstance(h, torch.Tensor) or h.device.type != "cpu" or tuple(h.shape) != tuple(fields.shape) \
                or h.dtype != fields.dtype or not h.is_contiguous():
            raise ValueError("%s must be a contiguous CPU tensor of shape %s and dtype %s"
                             % (name, tuple(fields.shape), fields.dtype))
    if fields.dtype != torch.float64:
        fields.state.copy_(h_in, non_blocking=True)
        evolve(params, fields, None, dt=dt)
        h_out.copy_(fields.state, non_blocking=True)
        return
    _check_state(fields, fields.state, "fields.state")
    _check_state(fields, fields.state_tmp, "fields.state_tmp")
    _check_state(fields, fields.scratch, "fields.scratch")
    rv = ctypes.c_int(1 if reverse_direction else 0)
    hb = [_native.ptr(a) for a in fields.backgrounds()]
    flags = params.get("step_flags", _native.MW_FLAG_WRITE_HALO)
    if params.get("check_finite"):  # blocking: raises MiniWeatherError (status 7) on NaN / Inf
        flags |= _native.MW_FLAG_CHECK_FINITE
    if nbands is None:
        nbands = HOST_STEP_BANDS.get(params.get("f64_mode", DEFAULT_F64_MODE), 1)
    _native.call("mw_step_f64_host", fields.nx, fields.nz, float(params["dx"]), float(params["dz"]),
                 float(params["dt"]), float(dt), *hb, _native.ptr(fields.src_w), ctypes.c_void_p(h_in.data_ptr()),
                 ctypes.c_void_p(h_out.data_ptr()), _native.ptr(fields.state), _native.ptr(fields.state_tmp),
                 _native.ptr(fields.scratch), ctypes.byref(rv), f64_mode(params), flags, int(nbands),
                 _native.stream_handle(fields.device))
    reverse_direction = bool(rv.value)

