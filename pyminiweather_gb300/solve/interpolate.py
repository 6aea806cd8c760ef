"""Unfused pieces of a direction-stage, pyminiweather/solve/interpolate.py:10-250.

Each function launches one kernel that follows the reference's NumPy
expression operation by operation (FP64 fields only) and writes the same
intermediate arrays of `fields`.  The fused step does not use them.
"""
from __future__ import annotations

from typing import Dict

import torch

from .. import _native


def _f64(fields, t, name, shape):
    return _native.require_cuda(t, name, dtype=torch.float64, shape=shape)


def _interp(params, fields, state, direction, vals, d3):
    state = fields.state if state is None else state
    _f64(fields, state, "state", fields.shape)
    _native.call("mw_interpolate_f64", fields.nx, fields.nz, _native.ptr(state), _native.ptr(vals), _native.ptr(d3),
                 direction, _native.stream_handle(fields.device))


def interpolate_x(params: Dict, fields, state=None) -> None:
    """fields.vals_x, d3_vals_x (4, nz, nx+1) from the interior rows of state (:10-43)."""
    _interp(params, fields, state, _native.MW_DIR_X, fields.vals_x, fields.d3_vals_x)


def interpolate_z(params: Dict, fields, state=None) -> None:
    """fields.vals_z, d3_vals_z (4, nz+1, nx) from the interior columns of state (:46-79)."""
    _interp(params, fields, state, _native.MW_DIR_Z, fields.vals_z, fields.d3_vals_z)


def _flux(params, fields, direction, vals, d3):
    hb = [_native.ptr(a) for a in fields.backgrounds()]
    _native.call("mw_flux_f64", fields.nx, fields.nz, float(params["dx"]), float(params["dz"]), float(params["dt"]),
                 *hb, _native.ptr(vals), _native.ptr(d3), _native.ptr(fields.flux), direction,
                 _native.stream_handle(fields.device))


def compute_flux_x(params: Dict, fields) -> None:
    """fields.flux[:, 0:nz, 0:nx+1] (:82-129)."""
    _flux(params, fields, _native.MW_DIR_X, fields.vals_x, fields.d3_vals_x)


def compute_flux_z(params: Dict, fields) -> None:
    """fields.flux[:, 0:nz+1, 0:nx]; zeroes d3_vals_z[DENS] at the walls as the reference does (:132-186)."""
    _flux(params, fields, _native.MW_DIR_Z, fields.vals_z, fields.d3_vals_z)


def _tend(params, fields, state, direction):
    _f64(fields, state, "state", fields.shape)
    _native.call("mw_tend_f64", fields.nx, fields.nz, float(params["dx"]), float(params["dz"]),
                 _native.ptr(fields.flux), _native.ptr(state), None, _native.ptr(fields.tend), direction,
                 _native.stream_handle(fields.device))


def compute_tend_x(params: Dict, fields, state) -> None:
    """fields.tend = -(F[i+1] - F[i]) / dx (:189-215)."""
    _tend(params, fields, state, _native.MW_DIR_X)


def compute_tend_z(params: Dict, fields, state) -> None:
    """fields.tend = -(G[k+1] - G[k]) / dz, minus rho' g on w (:218-250)."""
    _tend(params, fields, state, _native.MW_DIR_Z)
