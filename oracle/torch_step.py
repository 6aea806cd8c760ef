"""Pure-PyTorch FP64 copy of the reference time step (test infrastructure).

Autograd through this module is the second check of the hand-written adjoint
(the first is central finite differences).  It restates, with differentiable
tensor operations on the interior cells only:
  - halo rules: periodic x on the interior rows (pyminiweather/ics/bcs.py:35-39),
    wall z on the interior columns (bcs.py:92-148);
  - interpolation and third difference (solve/interpolate.py:33-43, 69-79);
  - fluxes with hyperviscosity (interpolate.py:82-186), w and d3[DENS] zeroed
    at the z walls (:167-173);
  - tendencies and gravity (interpolate.py:189-250), stage update (step.py:80-82);
  - RK3 with alternating direction order (step.py:85-143).
"""
from __future__ import annotations

import torch

HV_BETA = 0.05
C0 = 27.5629410929725921310572974482
GAMMA = 1.40027894002789400278940027894
GRAV = 9.8
K4 = (-1.0 / 12, 7.0 / 12, 7.0 / 12, -1.0 / 12)  # convolution kernel, data/fields.py:94-97
K3 = (1.0, -3.0, 3.0, -1.0)


def _taps(s, axis, n):
    """The four shifted views s[.., i + j] for interfaces i = 0..n along axis."""
    return [s.narrow(axis, j, n + 1) for j in range(4)]


def _interp(t):
    # scipy.signal.convolve(mode="same") accumulation order: ((s0*k3 + s1*k2) + s2*k1) + s3*k0
    vals = ((t[0] * K4[3] + t[1] * K4[2]) + t[2] * K4[1]) + t[3] * K4[0]
    d3 = ((t[0] * K3[3] + t[1] * K3[2]) + t[2] * K3[1]) + t[3] * K3[0]
    return vals, d3


def tendency_x(s, bg, dx, dt_full):
    """s: interior (4, nz, nx) -> tend (4, nz, nx)."""
    hyc, hytc = bg[0], bg[1]
    nz, nx = s.shape[1], s.shape[2]
    ext = torch.cat([s[..., nx - 2:], s, s[..., :2]], dim=-1)  # periodic halo
    vals, d3 = _interp(_taps(ext, 2, nx))
    hv = -HV_BETA * dx / (16 * dt_full)
    rho = vals[0] + hyc[2:nz + 2, None]
    u = vals[1] / rho
    w = vals[2] / rho
    t = (vals[3] + hytc[2:nz + 2, None]) / rho
    p = C0 * torch.pow(rho * t, GAMMA)
    F = torch.stack([rho * u - hv * d3[0], rho * u ** 2 + p - hv * d3[1], rho * u * w - hv * d3[2],
                     rho * u * t - hv * d3[3]])
    return -(F[..., 1:] - F[..., :-1]) / dx


def tendency_z(s, bg, dz, dt_full):
    hyc, hytc, hyi, hyti, hypi = bg
    nz, nx = s.shape[1], s.shape[2]
    top = s[:, :1]
    bot = s[:, nz - 1:nz]
    zero = torch.zeros_like(top[0:1])

    def halo(row, scales):
        d = row[0:1].expand(1, len(scales), nx)
        u = torch.cat([row[1:2] / hyc[idx_src] * hyc[i] for i, idx_src in scales], dim=1)
        w = zero.expand(1, len(scales), nx)
        t = row[3:4].expand(1, len(scales), nx)
        return torch.cat([d, u, w, t], dim=0)

    lo = halo(top, [(0, 2), (1, 2)])
    hi = halo(bot, [(nz + 2, nz + 1), (nz + 3, nz + 1)])
    ext = torch.cat([lo, s, hi], dim=1)  # (4, nz+4, nx)
    vals, d3 = _interp(_taps(ext, 1, nz))
    hv = -HV_BETA * dz / (16 * dt_full)
    rho = vals[0] + hyi[:, None]
    u = vals[1] / rho
    w = vals[2] / rho
    t = (vals[3] + hyti[:, None]) / rho
    p = C0 * torch.pow(rho * t, GAMMA) - hypi[:, None]
    wall = torch.zeros(nz + 1, 1, dtype=torch.bool, device=s.device)
    wall[0] = True
    wall[nz] = True
    w = torch.where(wall, torch.zeros_like(w), w)
    d3r = torch.where(wall, torch.zeros_like(d3[0]), d3[0])
    G = torch.stack([rho * w - hv * d3r, rho * w * u - hv * d3[1], rho * w ** 2 + p - hv * d3[2],
                     rho * w * t - hv * d3[3]])
    tend = -(G[:, 1:] - G[:, :-1]) / dz
    return torch.cat([tend[:2], (tend[2] - s[0] * GRAV)[None], tend[3:]], dim=0)


def evolve_interior(s, bg, params, nsteps, reverse=False):
    """Advance interior state s (4, nz, nx) by nsteps; returns (s, reverse)."""
    dx, dz, dt = params["dx"], params["dz"], params["dt"]
    for _ in range(nsteps):
        dirs = ("x", "z") if reverse else ("z", "x")
        for d in dirs:
            L = (lambda q: tendency_x(q, bg, dx, dt)) if d == "x" else (lambda q: tendency_z(q, bg, dz, dt))
            s1 = s + dt / 3 * L(s)
            s2 = s + dt / 2 * L(s1)
            s = s + dt / 1 * L(s2)
        reverse = not reverse
    return s, reverse
