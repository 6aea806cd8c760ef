"""Simulation arrays, the GPU counterpart of pyminiweather/data/fields.py:7-123.

All arrays are CUDA tensors.  state / state_tmp keep the reference's layout
(4, nz+4, nx+4), C order, x fastest, variables DENS, UMOM, WMOM, RHOT.  The
perturbation fields are FP64 (default) or FP32 (the precision form); the
hydrostatic backgrounds are always FP64.

Differences from the reference's container:
- `scratch` is a third state-sized array: the fused direction-stage kernel
  cannot update the array it reads neighbours from, so the RK3 stages
  ping-pong through it;
- the unfused intermediates (vals_x, d3_vals_x, vals_z, d3_vals_z, flux, tend)
  are allocated on first use, since the fused path never touches them (at
  8192 x 4096 in FP64 they would take 6.4 GB);
- `src_w` holds the gravity-wave forcing when ic_type is "gravity".
"""
from __future__ import annotations

import torch

NVARIABLES = 4


def _default_device():
    if not torch.cuda.is_available():
        raise RuntimeError("pyminiweather_gb300 needs a CUDA device; no CPU path exists")
    return torch.device("cuda", torch.cuda.current_device())


class Fields:
    """Arrays of one simulation (same attribute names as the reference's Fields)."""

    _LAZY = {
        "vals_x": lambda f: (NVARIABLES, f.nz, f.nx + 1),
        "d3_vals_x": lambda f: (NVARIABLES, f.nz, f.nx + 1),
        "vals_z": lambda f: (NVARIABLES, f.nz + 1, f.nx),
        "d3_vals_z": lambda f: (NVARIABLES, f.nz + 1, f.nx),
        "flux": lambda f: (NVARIABLES, f.nz + 1, f.nx + 1),
        "tend": lambda f: (NVARIABLES, f.nz, f.nx),
    }

    def __init__(self, nx, nz, hs, s, dtype, device):
        self.nx, self.nz, self.hs, self.s = int(nx), int(nz), int(hs), int(s)
        self.nvariables = NVARIABLES
        self.dtype = dtype
        self.device = device
        self.shape = (NVARIABLES, self.nz + 2 * self.hs, self.nx + 2 * self.hs)
        z = lambda *shape, dt=dtype: torch.zeros(shape, dtype=dt, device=device)
        self.state = z(*self.shape)
        self.state_tmp = z(*self.shape)
        self.scratch = z(*self.shape)
        self.hy_dens_cell = z(self.nz + 2 * self.hs, dt=torch.float64)
        self.hy_dens_theta_cell = z(self.nz + 2 * self.hs, dt=torch.float64)
        self.hy_dens_int = z(self.nz + 1, dt=torch.float64)
        self.hy_dens_theta_int = z(self.nz + 1, dt=torch.float64)
        self.hy_pressure_int = z(self.nz + 1, dt=torch.float64)
        # interpolation kernels, data/fields.py:94-97 (convolution order)
        self.fourth_order_kernel = torch.tensor([-1.0 / 12, 7.0 / 12, 7.0 / 12, -1.0 / 12], dtype=torch.float64)
        self.first_order_kernel = torch.tensor([1.0, -3.0, 3.0, -1.0], dtype=torch.float64)
        self.src_w = None
        self._stats_ws = None
        self._lazy = {}

    def __getattr__(self, name):
        lazy = type(self)._LAZY
        if name in lazy:
            d = self.__dict__["_lazy"]
            if name not in d:
                d[name] = torch.zeros(lazy[name](self), dtype=torch.float64, device=self.__dict__["device"])
            return d[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in type(self)._LAZY:
            self.__dict__["_lazy"][name] = value
        else:
            object.__setattr__(self, name, value)

    def backgrounds(self):
        return (self.hy_dens_cell, self.hy_dens_theta_cell, self.hy_dens_int, self.hy_dens_theta_int,
                self.hy_pressure_int)


def initialize_fields(params, dtype=None, device=None) -> Fields:
    """Allocate the arrays of a simulation, pyminiweather/data/fields.py:58-123.

    dtype: torch.float64 (default, or params["dtype"]) or torch.float32.
    """
    nx, nz, hs, s = params["nx"], params["nz"], params["hs"], params["s"]
    assert hs * 2 - s == 0
    if dtype is None:
        dtype = params.get("dtype", torch.float64)
    if isinstance(dtype, str):
        dtype = {"float64": torch.float64, "fp64": torch.float64, "float32": torch.float32,
                 "fp32": torch.float32}[dtype]
    if dtype not in (torch.float64, torch.float32):
        raise TypeError("state dtype must be torch.float64 or torch.float32")
    device = torch.device(device) if device is not None else _default_device()
    if device.type != "cuda":
        raise ValueError("pyminiweather_gb300 keeps its arrays on a CUDA device")
    return Fields(nx, nz, hs, s, dtype, device)
