"""The hand-written adjoint (differentiation form), checked against autograd
through the pure-PyTorch copy of the step and against central finite
differences."""
import time

import numpy as np
import pytest
import torch

from oracle import torch_step as TS
from pyminiweather_gb300 import _native
from pyminiweather_gb300.adjoint import RolloutContext, rollout, upper_half_rhot_misfit
from pyminiweather_gb300.data import initialize_fields
from pyminiweather_gb300.ics import init
from pyminiweather_gb300.solve import evolve, reset_direction
from tests.helpers import make_params

pytestmark = pytest.mark.gpu


def _fields(nx, nz, ic="thermal", amp=None):
    p = make_params(nx, nz, ic)
    f = initialize_fields(p)
    bub = None if amp is None else [(amp, p["xlen"] / 2, 2000.0, 2000.0, 2000.0)]
    init(f, p, None, bubbles=bub)
    return p, f


def _bg(f):
    return [a for a in f.backgrounds()]


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("direction", [0, 1])
def test_stage_vjp_matches_autograd(direction, mode):
    """One direction-stage: g_forcing = dt (dL/dforcing)^T g_out, against
    torch autograd of the pure-PyTorch tendency, in FP64 with the reference's
    formulas (mode 0), double-FP32 (mode 1) and IEEE FP64 with the fewest
    operations (mode 2)."""
    torch.manual_seed(0)
    p, f = _fields(40, 24, "collision")
    evolve(dict(p, f64_mode="native"), f, None, dt=p["dt"], nsteps=3)  # a developed state
    s = f.state.clone()
    g = torch.zeros_like(s)
    g[:, 2:-2, 2:-2] = torch.randn(4, 24, 40, dtype=torch.float64, device=s.device)
    dts = p["dt"] / 2
    out = torch.empty_like(s)
    ws = torch.empty(int(_native.load().mw_dirstage_vjp_workspace_bytes(40, 24)) // 8 + 1, dtype=torch.float64,
                     device=s.device)
    hb = [_native.ptr(a) for a in f.backgrounds()]
    _native.call("mw_dirstage_vjp_f64", 40, 24, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(s), _native.ptr(g),
                 None, None, 0, _native.ptr(out), dts, direction, mode, _native.ptr(ws), ws.numel() * 8,
                 _native.stream_handle())
    x = s[:, 2:-2, 2:-2].clone().requires_grad_(True)
    L = TS.tendency_x(x, _bg(f), p["dx"], p["dt"]) if direction == 0 else TS.tendency_z(x, _bg(f), p["dz"], p["dt"])
    (ref,) = torch.autograd.grad((dts * L * g[:, 2:-2, 2:-2]).sum(), x)
    got = out[:, 2:-2, 2:-2]
    for v in range(4):
        err = float((got[v] - ref[v]).abs().max() / ref[v].abs().max().clamp_min(1e-300))
        assert err <= (1e-12 if mode == 0 else 1e-11), (direction, mode, v, err)
    assert float(out[:, :2].abs().max()) == 0.0 and float(out[:, -2:].abs().max()) == 0.0  # halo rows
    assert float(out[:, :, :2].abs().max()) == 0.0 and float(out[:, :, -2:].abs().max()) == 0.0  # halo columns


@pytest.mark.parametrize("nx,nz", [(2, 1), (3, 2), (29, 5), (30, 31), (61, 58), (130, 3)])
@pytest.mark.parametrize("direction", [0, 1])
def test_stage_vjp_split_matches_native(nx, nz, direction):
    """The double-FP32 and the fewest-operation IEEE-FP64 stage adjoints
    against the reference-formula FP64 one on ragged grids (segment edges,
    one-row and two-column grids, both walls in one segment), with bases and
    accumulation of g_out."""
    p, f = _fields(nx, nz, "collision")
    evolve(dict(p, f64_mode="native"), f, None, dt=p["dt"], nsteps=2)
    s = f.state.clone()
    gen = torch.Generator(device="cpu").manual_seed(nx * 100 + nz + direction)
    g, ba, bb = (torch.zeros_like(s) for _ in range(3))
    for a in (g, ba, bb):
        a[:, 2:-2, 2:-2] = torch.randn(4, nz, nx, generator=gen, dtype=torch.float64).to(s.device)
    ws = torch.empty(int(_native.load().mw_dirstage_vjp_workspace_bytes(nx, nz)) // 8 + 1, dtype=torch.float64,
                     device=s.device)
    hb = [_native.ptr(a) for a in f.backgrounds()]
    outs = []
    for mode in (0, 1, 2):
        out = torch.full_like(s, 7.0)
        _native.call("mw_dirstage_vjp_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(s), _native.ptr(g),
                     _native.ptr(ba), _native.ptr(bb), 1, _native.ptr(out), p["dt"] / 3, direction, mode,
                     _native.ptr(ws), ws.numel() * 8, _native.stream_handle())
        outs.append(out)
    torch.cuda.synchronize()
    ref = outs[0]
    inc_ref = ref[:, 2:-2, 2:-2] - (g + ba + bb)[:, 2:-2, 2:-2]
    for mode, got in ((1, outs[1]), (2, outs[2])):
        inc_got = got[:, 2:-2, 2:-2] - (g + ba + bb)[:, 2:-2, 2:-2]
        for v in range(4):
            err = float((inc_got[v] - inc_ref[v]).abs().max() / inc_ref[v].abs().max().clamp_min(1e-300))
            assert err <= (1e-11 if mode == 1 else 1e-13), (nx, nz, direction, mode, v, err)
        assert torch.equal(got[:, :2], torch.zeros_like(got[:, :2]))
        assert torch.equal(got[:, :, -2:], torch.zeros_like(got[:, :, -2:]))


@pytest.mark.parametrize("mode", ["native", "fp64", "split"])
def test_rollout_gradient_matches_autograd(mode):
    """Gradient of the upper-half (rho theta)' misfit after 12 steps w.r.t. all
    four initial fields: hand-written adjoint (checkpoints every 5 steps; FP64
    or double-FP32 forward and adjoint) against autograd through the
    pure-PyTorch step."""
    nx, nz, steps = 48, 24, 12
    p, f = _fields(nx, nz, amp=3.0)
    _, ft = _fields(nx, nz, amp=3.5)
    reset_direction()
    evolve(dict(p, f64_mode="native"), ft, None, dt=p["dt"], nsteps=steps)
    target = ft.state.clone()
    x0 = f.state.clone().requires_grad_(True)
    ctx = RolloutContext(params=dict(p, f64_mode=mode), fields=f, nsteps=steps, ckpt_every=5)
    loss = upper_half_rhot_misfit(rollout(x0, ctx), target, nz)
    (g,) = torch.autograd.grad(loss, x0)
    xi = f.state[:, 2:-2, 2:-2].clone().requires_grad_(True)
    s, _ = TS.evolve_interior(xi, _bg(f), p, steps)
    d = s[3, nz // 2:, :] - target[3, 2 + nz // 2:2 + nz, 2:-2]
    (gr,) = torch.autograd.grad((d * d).sum(), xi)
    assert abs(float(loss) - float((d * d).sum())) <= 1e-9 * abs(float(loss))
    for v in range(4):
        err = float((g[v, 2:-2, 2:-2] - gr[v]).abs().max() / gr[v].abs().max())
        print("field %d: adjoint vs autograd normwise %.2e" % (v, err))
        assert err <= 1e-9
    assert float(g[:, :2].abs().max()) == 0.0 and float(g[:, :, -2:].abs().max()) == 0.0


def _config4(mode):
    """The differentiation configuration: 512 x 256 thermal (amplitude 3 K),
    200 steps, checkpoints every 20; target from amplitude 3.5 K; loss = the
    upper-half (rho theta)' misfit.  Returns (p, f, target, x0, ctx)."""
    nx, nz, steps = 512, 256, 200
    p, f = _fields(nx, nz, amp=3.0)
    p["f64_mode"] = mode
    _, ft = _fields(nx, nz, amp=3.5)
    reset_direction()
    evolve(dict(p, f64_mode="native"), ft, None, dt=p["dt"], nsteps=steps)
    target = ft.state.clone()
    ctx = RolloutContext(params=p, fields=f, nsteps=steps, ckpt_every=20)
    return p, f, target, f.state.clone().requires_grad_(True), ctx


@pytest.mark.parametrize("mode", ["native", "fp64", "split"])
def test_adjoint_vs_autograd_512x256_200_steps(mode):
    """The differentiation configuration checked against autograd through the
    pure-PyTorch step at its own size: 512 x 256, 200 steps, gradient with
    respect to all four initial fields.  Autograd recomputes each 20-step
    segment (torch.utils.checkpoint) to bound its memory.  Bar: 1e-9
    normwise per field for the FP64 forms; the double-FP32 form's error is
    printed and held to 1e-7."""
    from torch.utils.checkpoint import checkpoint
    p, f, target, x0, ctx = _config4(mode)
    nx, nz, steps = f.nx, f.nz, ctx.nsteps
    loss = upper_half_rhot_misfit(rollout(x0, ctx), target, nz)
    (g,) = torch.autograd.grad(loss, x0)
    bg = _bg(f)

    def segment(s, rev, n):
        return TS.evolve_interior(s, bg, p, n, reverse=rev)[0]

    xi = f.state[:, 2:-2, 2:-2].clone().requires_grad_(True)
    s, rev = xi, False
    for k in range(0, steps, 20):
        s = checkpoint(segment, s, rev, 20, use_reentrant=False)
        rev = rev if 20 % 2 == 0 else not rev
    d = s[3, nz // 2:, :] - target[3, 2 + nz // 2:2 + nz, 2:-2]
    lr = (d * d).sum()
    (gr,) = torch.autograd.grad(lr, xi)
    print("%s: loss %.12e (hand-written forward) vs %.12e (PyTorch step)" % (mode, float(loss), float(lr)))
    bar = 1e-7 if mode == "split" else 1e-9
    for v in range(4):
        err = float((g[v, 2:-2, 2:-2] - gr[v]).abs().max() / gr[v].abs().max())
        print("%s field %d: adjoint vs autograd normwise %.2e" % (mode, v, err))
        assert err <= bar
    assert abs(float(loss) - float(lr)) <= 1e-8 * abs(float(lr))
    assert float(g[:, :2].abs().max()) == 0.0 and float(g[:, :, -2:].abs().max()) == 0.0


@pytest.mark.parametrize("mode", ["native", "fp64"])
def test_adjoint_vs_finite_differences_512x256(mode):
    """The differentiation configuration: 512 x 256 thermal, 200 steps,
    checkpoints every 20; target from amplitude 3.5 K; 16 seeded directions,
    central differences with eps = 1e-6, for both IEEE-FP64 forwards (the FD
    quotient needs FP64 rounding in the forward: the split form's 2^-47 noise
    divided by 2 eps would dominate it)."""
    p, f, target, x0, ctx = _config4(mode)
    nx, nz = f.nx, f.nz
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = upper_half_rhot_misfit(rollout(x0, ctx), target, nz)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    (g,) = torch.autograd.grad(loss, x0)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    print("%s 512x256, 200 steps: forward %.3f s, adjoint %.3f s (ratio %.2f)" % (
        mode, t1 - t0, t2 - t1, (t2 - t1) / (t1 - t0)))

    def L(x):
        with torch.no_grad():
            return float(upper_half_rhot_misfit(rollout(x, ctx), target, nz))

    gen = torch.Generator(device="cpu").manual_seed(1234)
    eps = 1e-6
    worst = 0.0
    for k in range(16):
        v = torch.zeros_like(x0)
        v[:, 2:-2, 2:-2] = torch.randn(4, nz, nx, generator=gen, dtype=torch.float64).to(x0.device)
        fd = (L(x0.detach() + eps * v) - L(x0.detach() - eps * v)) / (2 * eps)
        ad = float((g * v).sum())
        rel = abs(fd - ad) / abs(ad)
        worst = max(worst, rel)
        print("%s direction %2d: adjoint %.10e  central FD %.10e  rel %.2e" % (mode, k, ad, fd, rel))
    assert worst <= 1e-6
