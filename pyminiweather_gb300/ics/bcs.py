"""Halo fill, pyminiweather/ics/bcs.py:8-148 (set_bc_x: periodic in x on the
interior rows; set_bc_z: solid wall in z on all columns).  The fused step
applies these rules on the fly and never needs them; they serve callers of
the unfused API."""
from __future__ import annotations

from typing import Dict

import torch

from .. import _native


def _bc(params, fields, state_forcing, ic_type, direction):
    if ic_type == "injection":
        raise NotImplementedError("the injection boundary condition is flagged unsupported by the reference")
    _native.require_cuda(state_forcing, "state_forcing", dtype=torch.float64, shape=fields.shape)
    _native.call("mw_set_bc_f64", fields.nx, fields.nz, _native.ptr(fields.hy_dens_cell),
                 _native.ptr(state_forcing), direction, _native.stream_handle(fields.device))


def set_bc_x(params: Dict, fields, state_forcing, ic_type: str) -> None:
    _bc(params, fields, state_forcing, ic_type, _native.MW_DIR_X)


def set_bc_z(params: Dict, fields, state_forcing, ic_type: str) -> None:
    _bc(params, fields, state_forcing, ic_type, _native.MW_DIR_Z)
