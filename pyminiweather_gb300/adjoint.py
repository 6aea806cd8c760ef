"""Adjoint of the time step: gradients of a final-state misfit with respect to
the initial state (no counterpart in the reference, which has no derivatives).

`Rollout.apply(state0, ctx)` advances `state0` (a (4, nz+4, nx+4) FP64 CUDA
tensor) by ctx.nsteps steps and is differentiable: its backward pass replays
the forward from checkpoints stored every ctx.ckpt_every steps, keeps the six
stage states of each step of a segment, and runs the hand-written
vector-Jacobian product of each direction-stage (mw_dirstage_vjp_f64) in
reverse.  For one direction (RK3 of solve/step.py:112-141):

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
    """Work arrays for one grid (state-shaped FP64)."""

    def __init__(self, f, n_stage_states):
        z = lambda: torch.empty(f.shape, dtype=torch.float64, device=f.device)
        self.f = f
        self.stages = [z() for _ in range(n_stage_states)]
        self.g = [z() for _ in range(4)]
        need = int(_native.load().mw_dirstage_vjp_workspace_bytes(f.nx, f.nz))
        self.ws = torch.empty(need // 8 + 1, dtype=torch.float64, device=f.device)


def _stage(p, f, init, forcing, out, dts, d):
    hb = [_native.ptr(a) for a in f.backgrounds()]
    _native.call("mw_dirstage_f64", f.nx, f.nz, float(p["dx"]), float(p["dz"]), float(p["dt"]), *hb,
                 _native.ptr(f.src_w), _native.ptr(init), _native.ptr(forcing), _native.ptr(out), float(dts), d,
                 f64_mode(p), 0, _native.stream_handle(f.device))


def _vjp(p, f, forcing, g_out, g_dst, dts, d, ws, base_a=None, base_b=None, add_g_out=False):
    hb = [_native.ptr(a) for a in f.backgrounds()]
    _native.call("mw_dirstage_vjp_f64", f.nx, f.nz, float(p["dx"]), float(p["dz"]), float(p["dt"]), *hb,
                 _native.ptr(forcing), _native.ptr(g_out), _native.ptr(base_a), _native.ptr(base_b),
                 int(add_g_out), _native.ptr(g_dst), float(dts), d, _native.ptr(ws), ws.numel() * 8,
                 _native.stream_handle(f.device))


def _directions(reverse):
    return (_native.MW_DIR_X, _native.MW_DIR_Z) if reverse else (_native.MW_DIR_Z, _native.MW_DIR_X)


def _forward_step(p, f, S, out, stage_states, reverse):
    """One time step S -> out through six direction-stages, keeping the stage
    forcing states in stage_states[0..5] (S, s1, s2 per direction)."""
    dt = p["dt"]
    cur = S
    for n, d in enumerate(_directions(reverse)):
        S_d, s1, s2 = stage_states[3 * n:3 * n + 3]
        if S_d.data_ptr() != cur.data_ptr():
            S_d.copy_(cur)
        _stage(p, f, S_d, S_d, s1, dt / 3, d)
        _stage(p, f, S_d, s1, s2, dt / 2, d)
        dst = out if n == 1 else stage_states[3]
        _stage(p, f, S_d, s2, dst, dt, d)
        cur = dst


def _backward_step(p, f, stage_states, g, reverse, buf):
    """g: adjoint of the step's output; returns the adjoint of its input (one of buf.g)."""
    dt = p["dt"]
    gA, gB, gC, gD = buf.g
    cur = g
    for n, d in reversed(list(enumerate(_directions(reverse)))):
        S_d, s1, s2 = stage_states[3 * n:3 * n + 3]
        s2b = gA if cur.data_ptr() != gA.data_ptr() else gD
        _vjp(p, f, s2, cur, s2b, dt, d, buf.ws)
        s1b = gB
        _vjp(p, f, s1, s2b, s1b, dt / 2, d, buf.ws)
        outg = gC if cur.data_ptr() != gC.data_ptr() else gD
        _vjp(p, f, S_d, s1b, outg, dt / 3, d, buf.ws, base_a=cur, base_b=s2b, add_g_out=True)
        cur = outg
    return cur


class Rollout(torch.autograd.Function):
    """state0 -> state after ctx.nsteps steps, with a checkpointed hand-written adjoint."""

    @staticmethod
    def forward(autograd_ctx, state0, ctx: RolloutContext):
        p, f = ctx.params, ctx.fields
        _native.require_cuda(state0, "state0", dtype=torch.float64, shape=f.shape)
        cur = state0.detach().clone()
        nxt = torch.empty_like(cur)
        stages = [torch.empty_like(cur) for _ in range(6)]
        ckpts = []
        rev = ctx.reverse
        for k in range(ctx.nsteps):
            if k % ctx.ckpt_every == 0:
                ckpts.append((k, cur.clone(), rev))
            _forward_step(p, f, cur, nxt, stages, rev)
            cur, nxt = nxt, cur
            rev = not rev
        autograd_ctx.ctx = ctx
        autograd_ctx.ckpts = ckpts
        return cur

    @staticmethod
    def backward(autograd_ctx, g_final):
        ctx = autograd_ctx.ctx
        p, f = ctx.params, ctx.fields
        E = ctx.ckpt_every
        buf = _Buffers(f, 6 * E)
        g = g_final.detach().to(torch.float64).contiguous().clone()
        out = torch.empty_like(g)
        for k0, state, rev0 in reversed(autograd_ctx.ckpts):
            n = min(E, ctx.nsteps - k0)
            # replay the segment, keeping the six stage states of every step
            cur = state
            rev = rev0
            revs = []
            for j in range(n):
                st = buf.stages[6 * j:6 * j + 6]
                st[0].copy_(cur)
                _forward_step(p, f, st[0], out, st, rev)
                revs.append(rev)
                cur = out
                rev = not rev
            for j in reversed(range(n)):
                res = _backward_step(p, f, buf.stages[6 * j:6 * j + 6], g, revs[j], buf)
                g.copy_(res)
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
