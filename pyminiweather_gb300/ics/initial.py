"""init(): initial state and hydrostatic backgrounds, pyminiweather/ics/initial.py:11-105.

One call of the mw_init_* kernel evaluates the 3x3 Gauss-Legendre cell
averages of the initial condition over every cell (halo included) and the
backgrounds at cell centres and interfaces, in FP64.
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np
import torch

from .. import _native
from .initial_conditions import ic_spec


def init(fields, params: Dict, Mesh=None, bubbles: Optional[Sequence[Sequence[float]]] = None) -> None:
    """Fill fields.state, fields.state_tmp and the backgrounds.

    bubbles, if given, replaces the ic_type's bubble list: rows of
    (amplitude K, x0 m, z0 m, xrad m, zrad m).
    """
    spec = ic_spec(params["ic_type"], params["xlen"])
    bub = spec.bubbles if bubbles is None else [tuple(float(v) for v in b) for b in bubbles]
    if len(bub) > _native.MW_MAX_BUBBLES:
        raise ValueError("at most %d bubbles" % _native.MW_MAX_BUBBLES)
    host = np.ascontiguousarray(np.array(bub, dtype=np.float64).reshape(-1)) if bub else None
    hptr = host.ctypes.data_as(_native.ctypes.c_void_p) if host is not None else None
    f = fields
    _native.require_cuda(f.state, "fields.state", shape=f.shape)
    fn = "mw_init_f64" if f.state.dtype == torch.float64 else "mw_init_f32"
    hb = [_native.ptr(a) for a in f.backgrounds()]
    _native.call(fn, f.nx, f.nz, float(params["xlen"]), float(params["zlen"]), spec.background, float(spec.u0),
                 len(bub), hptr, _native.ptr(f.state), *hb, _native.stream_handle(f.device))
    f.state_tmp.copy_(f.state)
    if params["ic_type"] == "gravity":
        f.src_w = torch.empty((f.nz, f.nx), dtype=torch.float64, device=f.device)
        _native.call("mw_gravity_source_f64", f.nx, f.nz, float(params["xlen"]), float(params["zlen"]),
                     _native.ptr(f.hy_dens_cell), _native.ptr(f.src_w), _native.stream_handle(f.device))
    else:
        f.src_w = None
