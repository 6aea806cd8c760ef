"""Diagnostics, pyminiweather/post/stats.py:8-69, on the GPU in FP64."""
from __future__ import annotations

from typing import Dict, Tuple

import torch

from .. import _native


def _workspace(fields):
    need = int(_native.load().mw_stats_workspace_bytes(fields.nx, fields.nz))
    ws = fields._stats_ws
    if ws is None or ws.numel() * 8 < need + 16:
        # 2 doubles of result + the per-block partials
        ws = torch.empty(need // 8 + 2, dtype=torch.float64, device=fields.device)
        fields._stats_ws = ws
    return ws, need


def compute_stats_device(params: Dict, fields, state=None) -> torch.Tensor:
    """(total mass, total energy) as a 2-element FP64 CUDA tensor, no host sync."""
    st = fields.state if state is None else state
    _native.require_cuda(st, "state", dtype=fields.dtype, shape=fields.shape)
    ws, need = _workspace(fields)
    out = ws[:2]
    part = ws[2:]
    fn = "mw_stats_f64" if fields.dtype == torch.float64 else "mw_stats_f32"
    _native.call(fn, fields.nx, fields.nz, float(params["dx"]), float(params["dz"]), _native.ptr(fields.hy_dens_cell),
                 _native.ptr(fields.hy_dens_theta_cell), _native.ptr(st), _native.ptr(part), need, _native.ptr(out),
                 _native.stream_handle(fields.device))
    return out


def compute_stats(params: Dict, fields) -> Tuple[float, float]:
    """Return the total mass and total energy (ke has no 1/2, as in the reference)."""
    m, e = compute_stats_device(params, fields).tolist()
    return m, e


def compute_solution_variables(params: Dict, fields) -> torch.Tensor:
    """(rho', u, w, theta') over the interior, (4, nz, nx) FP64."""
    st = fields.state
    if st.dtype != torch.float64:
        st = st.to(torch.float64)
    _native.require_cuda(st, "state", dtype=torch.float64, shape=fields.shape)
    out = torch.empty((4, fields.nz, fields.nx), dtype=torch.float64, device=fields.device)
    _native.call("mw_solution_variables_f64", fields.nx, fields.nz, _native.ptr(fields.hy_dens_cell),
                 _native.ptr(fields.hy_dens_theta_cell), _native.ptr(st), _native.ptr(out),
                 _native.stream_handle(fields.device))
    return out


def count_nonfinite(fields, state: torch.Tensor = None) -> int:
    """Number of NaN / Inf interior values of the state (or of `state`, an
    array of the state's shape and dtype); synchronises to read the count."""
    st = fields.state if state is None else state
    _native.require_cuda(st, "state", dtype=fields.dtype, shape=fields.shape)
    count = torch.zeros(1, dtype=torch.int64, device=st.device)
    fn = "mw_count_nonfinite_f64" if st.dtype == torch.float64 else "mw_count_nonfinite_f32"
    _native.call(fn, fields.nx, fields.nz, _native.ptr(st), _native.ptr(count), _native.stream_handle(st.device))
    return int(count.item())

