"""Adjoint of the time step: gradients of a final-state misfit with respect to
the initial state (no counterpart in the reference, which has no derivatives).

`Rollout.apply(state0, ctx)` advances `state0` (a (4, nz+4, nx+4) FP64 CUDA
tensor) by ctx.nsteps steps and is differentiable: its backward pass replays
the forward from checkpoints stored every ctx.ckpt_every steps, keeps the six
stage states of each step of a segment, and runs the hand-written
vector-Jacobian product of each direction-stage (mw_dirstage_vjp_f64) in
reverse, in the arithmetic of the forward's f64_mode (FP64, or double-FP32
for the split form).  For one direction (RK3 of solve/step.py:112-141):

    s1 = S + dt/3 L(S),  s2 = S + dt/2 L(s1),  S' = S + dt L(s2)

    s2bar = VJP(s2; S'bar)            (dt)
    s1bar = VJP(s1; s2bar)            (dt/2)
    Sbar  = S'bar + s2bar + s1bar + VJP(S; s1bar)   (dt/3)

Halo cells of the initial state get zero gradient: they are overwritten
before they are read.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import torch

from . import _native
from .solve.step import f64_mode


@dataclass
class RolloutContext:
    """Everything a rollout needs besides the initial state."""
    params: Dict
    fields: object           # a data.Fields (backgrounds; its state arrays are not touched)
    nsteps: int
    ckpt_every: int = 20
    reverse: bool = False    # direction flag at the first step (False: z then x)
    stats: Dict = field(default_factory=dict)


class _Buffers:
    """Work arrays for one grid: the recorded stage states of a segment (six
    per step), three adjoint work arrays and the VJP workspace."""

    def __init__(self, f, steps):
        n = 4 * (f.nz + 4) * (f.nx + 4)
        self.n = n
        self.stages = torch.empty(6 * steps * n, dtype=torch.float64, device=f.device)
        self.outs = torch.empty((steps + 1) * n, dtype=torch.float64, device=f.device)
        self.gbuf = torch.empty(3 * n, dtype=torch.float64, device=f.device)
        need = int(_native.load().mw_dirstage_vjp_workspace_bytes(f.nx, f.nz))
        self.ws = torch.empty(need // 8 + 1, dtype=torch.float64, device=f.device)


def _common(p, f, dt):
    hb = [_native.ptr(a) for a in f.backgrounds()]
    return [f.nx, f.nz, float(p["dx"]), float(p["dz"]), float(p["dt"]), float(dt), *hb]


def _segment_forward(p, f, cur, tmp, scratch, nsteps, reverse):
    """nsteps steps of cur in place (mw_step_f64); returns the new direction flag."""
    rv = ctypes.c_int(1 if reverse else 0)
    _native.call("mw_step_f64", *_common(p, f, p["dt"]), _native.ptr(f.src_w), _native.ptr(cur), _native.ptr(tmp),
                 _native.ptr(scratch), int(nsteps), ctypes.byref(rv), f64_mode(p), 0, _native.stream_handle(f.device))
    return bool(rv.value)


class Rollout(torch.autograd.Function):
    """state0 -> state after ctx.nsteps steps, with a checkpointed hand-written adjoint."""

    @staticmethod
    def forward(autograd_ctx, state0, ctx: RolloutContext):
        p, f = ctx.params, ctx.fields
        _native.require_cuda(state0, "state0", dtype=torch.float64, shape=f.shape)
        cur = state0.detach().clone()
        tmp, scratch = torch.empty_like(cur), torch.empty_like(cur)
        ckpts = []
        rev = ctx.reverse
        k = 0
        while k < ctx.nsteps:
            n = min(ctx.ckpt_every, ctx.nsteps - k)
            ckpts.append((k, cur.clone(), rev))
            rev = _segment_forward(p, f, cur, tmp, scratch, n, rev)
            k += n
        autograd_ctx.ctx = ctx
        autograd_ctx.ckpts = ckpts
        return cur

    @staticmethod
    def backward(autograd_ctx, g_final):
        ctx = autograd_ctx.ctx
        p, f = ctx.params, ctx.fields
        buf = _Buffers(f, ctx.ckpt_every)
        N = buf.n
        g = g_final.detach().to(torch.float64).contiguous().clone()
        stream = _native.stream_handle(f.device)
        common = _common(p, f, p["dt"])
        for k0, state, rev0 in reversed(autograd_ctx.ckpts):
            n = min(ctx.ckpt_every, ctx.nsteps - k0)
            # replay the segment, recording the six stage states of every step
            buf.outs[:N].copy_(state.reshape(-1))
            rev = rev0
            revs = []
            for j in range(n):
                _native.call("mw_step_record_f64", *common, _native.ptr(f.src_w),
                             _native.ptr(buf.outs[j * N:]), _native.ptr(buf.stages[6 * j * N:]),
                             _native.ptr(buf.outs[(j + 1) * N:]), int(rev), f64_mode(p), stream)
                revs.append(rev)
                rev = not rev
            for j in reversed(range(n)):
                _native.call("mw_step_vjp_f64", *common, _native.ptr(buf.stages[6 * j * N:]), _native.ptr(g),
                             _native.ptr(g), _native.ptr(buf.gbuf), int(revs[j]), f64_mode(p), _native.ptr(buf.ws),
                             buf.ws.numel() * 8, stream)
        g[:, :2, :].zero_()
        g[:, -2:, :].zero_()
        g[:, :, :2].zero_()
        g[:, :, -2:].zero_()
        return g, None


def rollout(state0: torch.Tensor, ctx: RolloutContext) -> torch.Tensor:
    return Rollout.apply(state0, ctx)


def upper_half_rhot_misfit(state: torch.Tensor, target: torch.Tensor, nz: int) -> torch.Tensor:
    """Sum over interior rows k >= nz/2 of ((rho theta)' - target)^2."""
    h = 2
    rows = slice(h + nz // 2, h + nz)
    d = state[3, rows, h:-h] - target[3, rows, h:-h]
    return (d * d).sum()
