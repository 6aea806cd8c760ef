"""Source terms, pyminiweather/solve/source.py:53-75: only the gravity-wave
case has one; its forcing (fields.src_w) is built by init()."""
from __future__ import annotations

from typing import Dict

from .. import _native


def add_source_terms(params: Dict, mesh, fields) -> None:
    if params.get("ic_type") == "gravity":
        if fields.src_w is None:
            raise RuntimeError("fields.src_w is missing: call init() first")
        _native.call("mw_add_source_f64", fields.nx, fields.nz, _native.ptr(fields.src_w), _native.ptr(fields.tend),
                     _native.stream_handle(fields.device))
