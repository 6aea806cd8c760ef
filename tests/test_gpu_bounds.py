"""Memory safety of the split-form kernels without compute-sanitizer: the
bounds-checked library (MW_CHECK=1) diverts and counts every array index
outside its array.  A child process loads that library, checks that the
counter sees a planted out-of-range index (the self-test), then runs the
split stages, steps (plain and host-banded), ensembles and adjoint stages on
ragged grids and asserts that no kernel indexed outside its arrays."""
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
    from pyminiweather_gb300.ics import init
    from pyminiweather_gb300.solve import evolve, evolve_host, reset_direction
    from pyminiweather_gb300.ensemble import Ensemble, thermal_ensemble
    from tests.helpers import make_params
    L = _native.load()
    assert _native.library_path().endswith("_check.so"), _native.library_path()
    n = ctypes.c_ulonglong(0)
    _native.call("mw_debug_oob_count", ctypes.byref(n), 1)
    _native.call("mw_debug_oob_selftest", _native.stream_handle())
    torch.cuda.synchronize()
    _native.call("mw_debug_oob_count", ctypes.byref(n), 1)
    assert n.value == 1, n.value  # the planted index was caught (and diverted)
    for nx, nz, ic in [(2, 1, "collision"), (3, 2, "thermal"), (37, 13, "collision"), (31, 5, "gravity"),
                       (62, 17, "density-current"), (130, 70, "collision"), (257, 129, "gravity"),
                       (96, 320, "thermal")]:  # 16 host-step bands, the end ones half as tall
        p = make_params(nx, nz, ic)
        for flags in (1, 0):
            f = initialize_fields(p)
            init(f, p, None)
            reset_direction()
            evolve(dict(p, step_flags=flags), f, None, dt=p["dt"], nsteps=2)
            if nz >= 32:
                h = f.state.cpu().pin_memory()
                evolve_host(dict(p, step_flags=flags), f, h, h, dt=p["dt"], nbands=16)
                evolve_host(dict(p, step_flags=flags), f, h, h, dt=p["dt"], nbands=3)
        ws = torch.empty(int(L.mw_dirstage_vjp_workspace_bytes(nx, nz)) // 8 + 1, dtype=torch.float64, device="cuda")
        g = torch.randn_like(f.state)
        out = torch.empty_like(f.state)
        hb = [_native.ptr(a) for a in f.backgrounds()]
        for d in (0, 1):
            _native.call("mw_dirstage_vjp_f64", nx, nz, p["dx"], p["dz"], p["dt"], *hb, _native.ptr(f.state),
                         _native.ptr(g), _native.ptr(g), None, 1, _native.ptr(out), p["dt"] / 3, d, 1,
                         _native.ptr(ws), ws.numel() * 8, _native.stream_handle())
    ens = Ensemble(thermal_ensemble(5, seed=3))
    ens.step(3)
    torch.cuda.synchronize()
    _native.call("mw_debug_oob_count", ctypes.byref(n), 0)
    print("OOB", n.value)
    assert n.value == 0, n.value
""")


def test_split_kernels_stay_in_bounds():
    env = dict(os.environ, MW_LIBRARY_VARIANT="check",
               PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", DRIVER], cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "OOB 0" in r.stdout
