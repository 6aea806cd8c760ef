"""Ensembles of uneven grids (the batching form): every member must evolve
exactly as a single-grid run with the same parameters, through one persistent
launch per direction-stage, eagerly or replayed from a CUDA graph."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyminiweather_gb300.data import initialize_fields
from pyminiweather_gb300.ensemble import Ensemble, member_params, thermal_ensemble
from pyminiweather_gb300.ics import init
from pyminiweather_gb300.solve import evolve, reset_direction
from tests.helpers import TOL_STEP, normwise, rel_l2

pytestmark = pytest.mark.gpu


def small_members(seed=1):
    rng = np.random.default_rng(seed)
    out = []
    for nx, nz in ((64, 32), (100, 50), (130, 66), (256, 128), (37, 13), (300, 150)):
        p = member_params(nx, nz)
        out.append((p, [(rng.uniform(1, 5), rng.uniform(0.3, 0.7) * 2e4, rng.uniform(1500, 3000), 2000.0, 2000.0)]))
    return out


def single_run(p, bubbles, steps, dtype=torch.float64, mode="fp64"):
    q = dict(p, f64_mode=mode)
    f = initialize_fields(q, dtype=dtype)
    init(f, q, None, bubbles=bubbles)
    reset_direction()
    evolve(q, f, None, dt=q["dt"], nsteps=steps)
    return f.state.to(torch.float64).cpu().numpy()


# FP64 members run the same arithmetic as a single-grid run (rounding-level
# agreement); FP32 members agree to FP32 rounding (the ensemble kernels inline
# the same tile code with different constants folded, so FMA contraction may
# differ).
MEMBER_TOL = {torch.float64: 1e-12, torch.float32: 1e-5}


@pytest.mark.parametrize("dtype,mode", [(torch.float64, "fp64"), (torch.float64, "split"), (torch.float32, "fp64")])
def test_members_match_single_grid_runs(dtype, mode):
    mem = small_members()
    ens = Ensemble(mem, dtype=dtype, f64_mode=mode)
    ens.step(10)
    for e, (p, bub) in enumerate(mem):
        got = ens.member_state(e).to(torch.float64).cpu().numpy()
        ref = single_run(p, bub, 10, dtype, mode)
        err = max(normwise(got, ref, interior=False))
        print("%s member %d %dx%d: max normwise vs single grid %.2e identical %s" % (
            mode, e, p["nx"], p["nz"], err, np.array_equal(got, ref)))
        assert err <= MEMBER_TOL[dtype]


@pytest.mark.parametrize("dtype,mode", [(torch.float64, "fp64"), (torch.float64, "split"), (torch.float32, "fp64")])
def test_tiny_members_match_single_grid_runs(dtype, mode):
    """Members of 2 to 7 columns and 1 to 4 rows (and one of 66 x 2) beside each
    other: each equals its single-grid run."""
    rng = np.random.default_rng(8)
    mem = [(member_params(nx, nz), [(rng.uniform(1, 5), rng.uniform(0.3, 0.7) * 2e4, 1000.0, 2000.0, 2000.0)])
           for nx, nz in ((2, 1), (3, 2), (5, 3), (7, 1), (4, 4), (66, 2))]
    ens = Ensemble(mem, dtype=dtype, f64_mode=mode)
    ens.step(5)
    for e, (p, bub) in enumerate(mem):
        got = ens.member_state(e).to(torch.float64).cpu().numpy()
        ref = single_run(p, bub, 5, dtype, mode)
        err = max(normwise(got, ref, interior=False))
        assert err <= MEMBER_TOL[dtype], (p["nx"], p["nz"], err)


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_members_vs_oracle(mode):
    mem = small_members(seed=2)[:3]
    ens = Ensemble(mem, f64_mode=mode)
    ens.step(100)
    for e, (p, bub) in enumerate(mem):
        o = O.OracleSim(O.make_params(p["nx"], p["nz"], "thermal"), bubbles=bub)
        o.evolve(100)
        err = normwise(ens.member_state(e).cpu().numpy(), o.state)
        print("%s member %d vs oracle after 100 steps: %s" % (mode, e, ["%.2e" % v for v in err]))
        assert max(err) <= TOL_STEP


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_graph_replay_equals_eager_steps(mode):
    mem = small_members(seed=3)
    a, b = Ensemble(mem, f64_mode=mode), Ensemble(mem, f64_mode=mode)
    replay = a.graph()
    for _ in range(3):
        replay()
    b.grid_x, b.grid_z = a.grid_x, a.grid_z
    b.step(6)
    torch.cuda.synchronize()
    assert torch.equal(a.state, b.state) and torch.equal(a.state_tmp, b.state_tmp)
    assert a.reverse == b.reverse == 0


@pytest.mark.parametrize("dtype,mode", [(torch.float64, "fp64"), (torch.float64, "split"), (torch.float32, "fp64")])
def test_results_do_not_depend_on_the_grid(dtype, mode):
    """The persistent warps / CTAs take work items from the plan's cursor as
    they become free: any grid (one CTA, a few, one wave, several waves) gives
    the same bits, and the cursor starts every one of the 18 launches of three
    steps from the head of its list."""
    mem = small_members(seed=5)
    ref = None
    for grids in ((0, 0), (1, 1), (3, 5), (-4, -4)):
        ens = Ensemble(mem, dtype=dtype, f64_mode=mode)
        bx, bz = ens.default_grids()
        ens.grid_x = grids[0] if grids[0] >= 0 else -grids[0] * bx
        ens.grid_z = grids[1] if grids[1] >= 0 else -grids[1] * bz
        ens.step(3)
        torch.cuda.synchronize()
        if ref is None:
            ref = (ens.state.clone(), ens.state_tmp.clone())
        else:
            assert torch.equal(ens.state, ref[0]) and torch.equal(ens.state_tmp, ref[1]), grids


@pytest.mark.parametrize("dtype,mode", [(torch.float64, "fp64"), (torch.float32, "fp64")])
def test_plan_lists_sorted_and_cursor_reset(dtype, mode):
    """The plan's work lists hold every item once, sorted by decreasing cost
    (x: row length; z: tile rows, then used columns; member order within a
    cost), and the work cursor at the plan's end is zero again after a step
    call (the last CTA of every launch resets it)."""
    mem = small_members(seed=7)
    ens = Ensemble(mem, dtype=dtype, f64_mode=mode)
    ens.step(2)
    torch.cuda.synchronize()
    raw = ens.plan.view(torch.uint8).cpu().numpy()
    info = ens.info
    xi = raw[info.x_items_off:info.x_items_off + 8 * info.n_x_items].view(np.int32).reshape(-1, 2)
    zi = raw[info.z_items_off:info.z_items_off + 8 * info.n_z_items].view(np.int32).reshape(-1, 2)
    nxs = [p["nx"] for p, _ in mem]
    nzs = [p["nz"] for p, _ in mem]
    assert sorted(map(tuple, xi)) == sorted((e, k) for e in range(len(mem)) for k in range(nzs[e]))
    keys = [(-nxs[e], e, k) for e, k in xi]
    assert keys == sorted(keys)
    zt, cols = ens.z_tile, 64

    def tile(e, y):
        ncb = (nxs[e] + cols - 1) // cols
        cb, t = y % ncb, y // ncb
        return (-min(zt, nzs[e] - t * zt), -min(cols, nxs[e] - cb * cols))
    expect = sorted(((e, cb + ((nxs[e] + cols - 1) // cols) * t)
                     for e in range(len(mem)) for t in range((nzs[e] + zt - 1) // zt)
                     for cb in range((nxs[e] + cols - 1) // cols)))
    assert sorted(map(tuple, zi)) == expect
    zkeys = [tile(e, y) for e, y in zi]
    assert zkeys == sorted(zkeys)
    cursor = raw[info.bytes - 16:info.bytes].view(np.uint32)
    assert cursor[0] == 0 and cursor[1] == 0


def test_fp32_members_at_any_float_offset():
    """Member blocks that start at any float offset (not 8- or 16-byte aligned,
    as a C caller may lay them out) and rows of any length mod 4: the results
    equal those of the packed layout bit for bit."""
    import ctypes

    from pyminiweather_gb300 import _native
    mem = small_members(seed=6)
    ref = Ensemble(mem, dtype=torch.float32)
    n = ref.n_members()
    specs = (_native.EnsMember * n)()
    blocks, so = [], 0
    for e in range(n):
        s = ref.specs[e]
        so += 1 + e % 3  # gaps of 1..3 floats between the blocks
        size = 4 * (s.nx + 4) * (s.nz + 4)
        specs[e] = _native.EnsMember(s.nx, s.nz, s.dx, s.dz, s.dt, so, s.cell_off, s.int_off)
        blocks.append((so, size))
        so += size
    bufs = [torch.zeros(so + 8, dtype=torch.float32, device="cuda") for _ in range(3)]
    for e, (o, size) in enumerate(blocks):
        bufs[0][o:o + size] = ref.member_state(e).reshape(-1)
        bufs[1][o:o + size] = ref.member_state_tmp(e).reshape(-1)
    stream = _native.stream_handle()
    info = _native.EnsPlanInfo()
    _native.call("mw_ensemble_plan_info", n, specs, ref.z_tile, ctypes.byref(info))
    plan = torch.empty((info.bytes + 15) // 16 * 2, dtype=torch.float64, device="cuda")
    _native.call("mw_ensemble_plan", n, specs, ref.z_tile, _native.ptr(plan), plan.numel() * 8, ctypes.byref(info),
                 stream)
    rv = ctypes.c_int(0)
    _native.call("mw_ensemble_step_f32", _native.ptr(plan), ctypes.byref(info),
                 *[_native.ptr(a) for a in ref.backgrounds()], *[_native.ptr(b) for b in bufs], 3, ctypes.byref(rv),
                 _native.MW_FLAG_WRITE_HALO, 0, 0, stream)
    ref.step(3)
    torch.cuda.synchronize()
    assert rv.value == ref.reverse
    for e, (o, size) in enumerate(blocks):
        assert torch.equal(bufs[0][o:o + size], ref.member_state(e).reshape(-1)), e
        assert torch.equal(bufs[1][o:o + size], ref.member_state_tmp(e).reshape(-1)), e


def test_autotune_does_not_change_results():
    mem = small_members(seed=4)
    a, b = Ensemble(mem), Ensemble(mem)
    tuned = a.autotune(steps=1)
    assert tuned["z_tile"] in (16, 32, 64) and tuned["grid_x"] > 0 and tuned["grid_z"] > 0
    a.step(4)
    b.step(4)
    assert torch.equal(a.state, b.state)


def test_uneven_thermal_ensemble_256():
    """The batching configuration: 256 thermal members, nx log-uniform in
    [64, 1024], 100 steps, FP64 (IEEE; and the split form) and FP32; three
    members are re-run alone."""
    mem = thermal_ensemble(256, seed=0)
    e64 = Ensemble(mem, dtype=torch.float64)
    e64s = Ensemble(mem, dtype=torch.float64, f64_mode="split")
    e32 = Ensemble(mem, dtype=torch.float32)
    m0 = [e64.member_stats(e)[0] for e in range(len(mem))]
    for ens in (e64, e64s, e32):
        ens.autotune(steps=1)
        replay = ens.graph()
        for _ in range(50):
            replay()
    torch.cuda.synchronize()
    drift = max(abs(e64.member_stats(e)[0] - m0[e]) / m0[e] for e in range(len(mem)))
    assert drift <= 1e-13
    worst32 = 0.0
    for e in range(len(mem)):
        a = e32.member_state(e).to(torch.float64).cpu().numpy()
        b = e64.member_state(e).cpu().numpy()
        worst32 = max(worst32, max(rel_l2(a, b)[v] for v in (0, 3)))
    print("256 members, %d cells: FP32 vs FP64 worst rel-L2 (dens, rhot) %.2e, FP64 mass drift %.1e" % (
        e64.cells(), worst32, drift))
    assert worst32 <= 1e-4
    for e in (0, 100, 255):
        p, bub = mem[e]
        for ens, mode in ((e64, "fp64"), (e64s, "split")):
            ref = single_run(p, bub, 100, mode=mode)
            assert max(normwise(ens.member_state(e).cpu().numpy(), ref)) <= MEMBER_TOL[torch.float64]
        # the two FP64 forms agree with each other to the benchmark's tolerance
        assert max(normwise(e64s.member_state(e).cpu().numpy(), e64.member_state(e).cpu().numpy())) <= TOL_STEP
