"""Checkpoint / restart of a run: the state, the direction parity and the
step count (no counterpart in the reference, whose driver always starts from
the initial condition).  A restart continues bit for bit: the next step sees
the same state and the same direction order as the uninterrupted run."""
from __future__ import annotations

from typing import Dict

import numpy as np
import torch

from .solve import step as _step

_KEYS = ("nx", "nz", "xlen", "zlen", "dx", "dz", "dt", "ic_type")


def save_checkpoint(path: str, params: Dict, fields, step: int) -> None:
    """Write fields.state, the module direction flag and `step` to `path` (.npz)."""
    meta = {k: params[k] for k in _KEYS if k in params}
    np.savez(path, state=fields.state.detach().cpu().numpy(), step=np.int64(step),
             reverse_direction=np.bool_(_step.reverse_direction), dtype=str(fields.dtype).replace("torch.", ""),
             **{"param_" + k: np.asarray(v) for k, v in meta.items()})


def load_checkpoint(path: str, params: Dict, fields) -> int:
    """Restore fields.state and the direction flag from `path`; returns the step
    count stored with them.  The grid and the dtype must match."""
    with np.load(path) as z:
        st = z["state"]
        if tuple(st.shape) != tuple(fields.shape):
            raise ValueError("checkpoint state has shape %s, fields have %s" % (st.shape, tuple(fields.shape)))
        if str(z["dtype"]) != str(fields.dtype).replace("torch.", ""):
            raise ValueError("checkpoint dtype %s does not match fields dtype %s" % (z["dtype"], fields.dtype))
        for k in _KEYS:
            key = "param_" + k
            if key in z and k in params and np.asarray(params[k]).item() != z[key].item():
                raise ValueError("checkpoint %s = %r, run has %r" % (k, z[key].item(), params[k]))
        fields.state.copy_(torch.from_numpy(st))
        _step.reverse_direction = bool(z["reverse_direction"])
        return int(z["step"])
