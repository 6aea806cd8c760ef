"""Memory safety of every kernel of the library without compute-sanitizer:
the bounds-checked library (MW_CHECK=1) diverts and counts every array index
outside its array.  A child process loads that library, checks that the
counter sees a planted out-of-range index (the self-test), then runs on
ragged grids: the three FP64 forms (IEEE "fp64", "split", "native") and FP32
through the steps, single stages, host-banded steps and the pair-format
stages, the FP32 passes fed by tensor copies; the ensembles of every form;
the stage adjoints of every mode; the
initial condition, gravity source, stats, solution variables, non-finite
count and every unfused piece; and the z launches split at 65535 row tiles
(grid.y's limit) on a two-column grid over four million rows.  It asserts
that no kernel indexed outside its arrays."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = textwrap.dedent("""
    import ctypes, torch
    from pyminiweather_gb300 import _native
    from pyminiweather_gb300.data import initialize_fields
    from pyminiweather_gb300.ics import init, set_bc_x, set_bc_z
    from pyminiweather_gb300.post import compute_stats, compute_solution_variables, count_nonfinite
    from pyminiweather_gb300.solve import (evolve, evolve_host, reset_direction, interpolate_x, interpolate_z,
                                           compute_flux_x, compute_flux_z, compute_tend_x, compute_tend_z,
                                           add_source_terms)
    from pyminiweather_gb300.ensemble import Ensemble, thermal_ensemble
    from tests.helpers import make_params
    L = _native.load()
    assert _native.library_path().endswith("_check.so"), _native.library_path()
    n = ctypes.c_ulonglong(0)
    S = _native.stream_handle()
    def count():
        torch.cuda.synchronize()
        _native.call("mw_debug_oob_count", ctypes.byref(n), 0)
        return n.value
    _native.call("mw_debug_oob_count", ctypes.byref(n), 1)
    _native.call("mw_debug_oob_selftest", S)
    torch.cuda.synchronize()
    _native.call("mw_debug_oob_count", ctypes.byref(n), 1)
    assert n.value == 1, n.value  # the planted index was caught (and diverted)
    for nx, nz, ic in [(2, 1, "collision"), (3, 2, "thermal"), (5, 3, "thermal"), (7, 1, "collision"),
                       (4, 4, "thermal"), (66, 2, "thermal"), (37, 13, "collision"), (31, 5, "gravity"),
                       (62, 17, "density-current"), (130, 70, "collision"), (257, 129, "gravity"),
                       (96, 320, "thermal"),  # 16 host-step bands, the end ones half as tall
                       (256, 40, "collision"), (260, 9, "gravity"), (132, 7, "thermal")]:  # FP32 passes fed by
        # tensor copies (nx % 4 == 0, nx >= 128): rows of one and of two chunks
        p = make_params(nx, nz, ic)
        hb = None
        for mode in ("fp64", "split", "native"):
            for flags in (1, 0):
                q = dict(p, f64_mode=mode, step_flags=flags)
                f = initialize_fields(q)
                init(f, q, None)
                reset_direction()
                evolve(q, f, None, dt=p["dt"], nsteps=2)
                evolve(dict(q, check_finite=True), f, None, dt=p["dt"], nsteps=1)
                if nz >= 32 and mode != "native":
                    h = f.state.cpu().pin_memory()
                    evolve_host(q, f, h, h, dt=p["dt"], nbands=16)
                    evolve_host(q, f, h, h, dt=p["dt"], nbands=3)
            hb = [_native.ptr(a) for a in f.backgrounds()]
            if mode == "split":  # the pair-format stages, launch by launch
                a, b = torch.empty_like(f.state), torch.empty_like(f.state)
                for d in (0, 1):
                    _native.call("mw_dirstage_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(f.src_w),
                                 _native.ptr(f.state), _native.ptr(f.state), _native.ptr(a), p["dt"] / 3, d, 1,
                                 _native.MW_FLAG_PAIRS_OUT | 1, S)
                    _native.call("mw_dirstage_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(f.src_w),
                                 _native.ptr(f.state), _native.ptr(a), _native.ptr(b), p["dt"] / 2, d, 1,
                                 _native.MW_FLAG_PAIRS_IN | 1, S)
        f32 = initialize_fields(p, dtype=torch.float32)
        init(f32, p, None)
        evolve(dict(p, check_finite=True), f32, None, dt=p["dt"], nsteps=2)
        compute_stats(p, f32)
        count_nonfinite(f32)
        compute_stats(p, f)
        compute_solution_variables(p, f)
        count_nonfinite(f)
        # the unfused pieces of one stage per direction
        st = f.state.clone()
        set_bc_x(p, f, st, ic)
        interpolate_x(p, f, st)
        compute_flux_x(p, f)
        compute_tend_x(p, f, st)
        add_source_terms(p, None, f)
        set_bc_z(p, f, st, ic)
        interpolate_z(p, f, st)
        compute_flux_z(p, f)
        compute_tend_z(p, f, st)
        out = torch.empty_like(st)
        _native.call("mw_update_f64", nx, nz, _native.ptr(st), _native.ptr(f.tend), _native.ptr(out), p["dt"], S)
        ws = torch.empty(int(L.mw_dirstage_vjp_workspace_bytes(nx, nz)) // 8 + 1, dtype=torch.float64, device="cuda")
        g = torch.randn_like(f.state)
        for mode in (0, 1, 2):
            for d in (0, 1):
                _native.call("mw_dirstage_vjp_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(f.state),
                             _native.ptr(g), _native.ptr(g), None, 1, _native.ptr(out), p["dt"] / 3, d, mode,
                             _native.ptr(ws), ws.numel() * 8, S)
        print(nx, nz, ic, "OOB so far", count(), flush=True)
    from pyminiweather_gb300.ensemble import member_params
    tiny = [(member_params(nx, nz), None) for nx, nz in ((2, 1), (3, 2), (5, 3), (7, 1), (4, 4), (66, 2))]
    for dtype, mode in ((torch.float64, "fp64"), (torch.float64, "split"), (torch.float32, "fp64")):
        ens = Ensemble(thermal_ensemble(5, seed=3), dtype=dtype, f64_mode=mode)
        ens.step(3)
        ens = Ensemble(tiny, dtype=dtype, f64_mode=mode)  # members of 2 to 7 columns, 1 to 4 rows
        ens.step(3)
    print("ensembles: OOB so far", count(), flush=True)
    # z launches split at 65535 row tiles: 2 columns, more than 65535 x 64 rows
    nx, nz = 2, 64 * 65535 + 100
    p = make_params(nx, nz, "thermal")
    f = initialize_fields(p)
    init(f, p, None)
    hb = [_native.ptr(a) for a in f.backgrounds()]
    for mode in (2, 0):
        _native.call("mw_dirstage_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, None, _native.ptr(f.state),
                     _native.ptr(f.state), _native.ptr(f.state_tmp), p["dt"] / 3, 1, mode, 1, S)
    print("OOB", count())
    assert n.value == 0, n.value
    t = ctypes.c_ulonglong(1)
    _native.call("mw_debug_wait_timeouts", ctypes.byref(t), 0)
    assert t.value == 0, t.value
""")


def test_every_kernel_stays_in_bounds():
    env = dict(os.environ, MW_LIBRARY_VARIANT="check",
               PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", DRIVER], cwd=ROOT, capture_output=True, text=True, timeout=1500, env=env)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "OOB 0" in r.stdout
