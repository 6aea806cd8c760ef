"""Mesh coordinates, the counterpart of pyminiweather/mesh.py:5-112.

Coordinates are built as numpy.linspace(start, stop, num, endpoint=False)
builds them (k * step + start, step = (stop - start) / num) and returned as
FP64 CUDA tensors.  The kernels compute the coordinates they need themselves;
this class serves callers of the reference's MeshData API.
"""
from __future__ import annotations

from typing import Dict, Tuple

import torch


def _linspace(start, stop, num, device):
    step = (stop - start) / num
    return torch.arange(num, dtype=torch.float64, device=device) * step + start


class MeshData:
    def __init__(self, params: Dict, device=None):
        self.params = params
        self.xlen = params["xlen"]
        self.zlen = params["zlen"]
        self.dx = params["dx"]
        self.dz = params["dz"]
        self.nx = params["nx"]
        self.nz = params["nz"]
        self.hs = params["hs"]
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.mesh_int_ext = None
        self.mesh_cell_centers = None
        self.mesh_vertical_cell_edges = None
        self.mesh_vertical_cell_centers_int_ext = None

    def get_mesh_int_ext(self) -> Tuple[torch.Tensor, torch.Tensor]:
        """Cell left edges including the halo, mesh.py:25-51."""
        if self.mesh_int_ext is None:
            x = _linspace(-self.hs * self.dx, (self.nx + self.hs) * self.dx, self.nx + 2 * self.hs, self.device)
            z = _linspace(-self.hs * self.dz, (self.nz + self.hs) * self.dz, self.nz + 2 * self.hs, self.device)
            zz, xx = torch.meshgrid(z, x, indexing="ij")
            self.mesh_int_ext = (xx, zz)
        return self.mesh_int_ext

    def get_mesh_cell_centers(self) -> Tuple[torch.Tensor, torch.Tensor]:
        """Interior cell centres, mesh.py:53-75."""
        if self.mesh_cell_centers is None:
            x = _linspace(self.dx / 2.0, self.xlen + self.dx / 2.0, self.nx, self.device)
            z = _linspace(self.dz / 2.0, self.zlen + self.dz / 2.0, self.nz, self.device)
            zz, xx = torch.meshgrid(z, x, indexing="ij")
            self.mesh_cell_centers = (xx, zz)
        return self.mesh_cell_centers

    def get_mesh_vertical_cell_edges(self) -> torch.Tensor:
        """z of the nz+1 interfaces, mesh.py:77-92."""
        if self.mesh_vertical_cell_edges is None:
            self.mesh_vertical_cell_edges = _linspace(0.0, (self.nz + 1) * self.dz, self.nz + 1, self.device)
        return self.mesh_vertical_cell_edges

    def get_mesh_vertical_cell_centers_int_ext(self) -> torch.Tensor:
        """z of the cell centres including the halo, mesh.py:94-112."""
        if self.mesh_vertical_cell_centers_int_ext is None:
            self.mesh_vertical_cell_centers_int_ext = _linspace(
                (-self.hs + 0.5) * self.dz, (self.nz + self.hs + 0.5) * self.dz, self.nz + 2 * self.hs, self.device)
        return self.mesh_vertical_cell_centers_int_ext
