"""Text output of the reference's driver (pyminiweather/__main__.py:218-233):
the state and the solution variables written as np.savetxt(outfile,
array.reshape(-1, last_dim), delimiter=",") would write them, byte for byte,
by the library's threaded host writer (mw_savetxt_f64)."""
from __future__ import annotations

from typing import Dict

import numpy as np
import torch

from .. import _native
from .stats import compute_solution_variables


def savetxt(path: str, array, append: bool = False, threads: int = 0) -> None:
    """np.savetxt(fh, array.reshape(-1, array.shape[-1]), delimiter=",") into
    `path` (created, or appended to).  array: a tensor (any device) or an ndarray."""
    if isinstance(array, torch.Tensor):
        host = array.detach().to("cpu", torch.float64).contiguous().numpy()
    else:
        host = np.ascontiguousarray(array, dtype=np.float64)
    cols = host.shape[-1] if host.ndim else 1
    rows = host.size // cols if cols else 0
    _native.call("mw_savetxt_f64", host.ctypes.data_as(_native.ctypes.c_void_p), rows, cols,
                 str(path).encode(), 1 if append else 0, int(threads))


def svars_filename(app_filename: str) -> str:
    """The solution-variable file of the reference: name.ext -> name_svars.ext
    (the reference splits on the single '.')."""
    fname, ext = app_filename.split(".")
    return fname + "_svars." + ext


def write_output(params: Dict, fields, append: bool) -> None:
    """One output of the reference's driver: the full state array (halo
    included) to params["app_filename"], the solution variables to its
    "_svars" companion."""
    name = params["app_filename"]
    savetxt(name, fields.state, append=append)
    savetxt(svars_filename(name), compute_solution_variables(params, fields), append=append)
