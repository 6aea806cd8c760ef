"""sample_ellipse_cosine, pyminiweather/utils/utils.py:5-51, for tensors on
any device (a helper of the API; the initial-condition kernel evaluates the
same profile itself)."""
from __future__ import annotations

import torch

from ..data.constants import Constants


def sample_ellipse_cosine(x, z, amplitude, x0, z0, xrad, zrad):
    x = torch.as_tensor(x, dtype=torch.float64)
    z = torch.as_tensor(z, dtype=torch.float64, device=x.device)
    pi = Constants.pi.value
    dist = torch.sqrt(((x - x0) / xrad) ** 2 + ((z - z0) / zrad) ** 2) * pi / 2.0
    c = torch.cos(dist)
    return torch.where(dist <= pi / 2.0, amplitude * (c * c), torch.zeros_like(dist))
