"""The C-ABI library loads, exports every declared symbol, and rejects bad
arguments with its status codes before any launch (no GPU needed: every case
here fails validation, so no CUDA call is made)."""
import ctypes
import os
import re

import numpy as np

import pytest
import torch

from pyminiweather_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "miniweather_gb300.h")

OK, INVALID, SHAPE, ALIGN, ALIAS, CUDA, WORKSPACE = 0, 1, 2, 3, 4, 5, 6


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mw_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _native.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # every declared function is bound by the Python layer with a signature
    assert set(names) <= set(_native._SIGNATURES), set(names) - set(_native._SIGNATURES)


def test_status_strings_and_version():
    L = _native.load()
    assert L.mw_abi_version() == 4
    for code in range(8):
        assert L.mw_status_string(code)
    assert L.mw_status_string(99) == b"unknown status"


FAKE = 1 << 20  # a fake, 8-byte aligned "device address"; never dereferenced


def P(x):
    return ctypes.c_void_p(x)


def dirstage(nx=16, nz=8, dx=1.0, dz=1.0, dtf=0.1, bg=(FAKE,) * 5, init=FAKE * 10, forcing=FAKE * 20,
             out=FAKE * 30, dts=0.1, direction=0, mode=0):
    L = _native.load()
    return L.mw_dirstage_f64(nx, nz, dx, dz, dtf, *[P(b) for b in bg], None, P(init), P(forcing), P(out), dts,
                             direction, mode, 1, None)


def test_dirstage_validation():
    L = _native.load()
    assert dirstage(nx=1) == SHAPE
    assert dirstage(nz=0) == SHAPE
    assert dirstage(dx=0.0) == INVALID
    assert dirstage(dtf=float("nan")) == INVALID
    assert dirstage(bg=(FAKE, 0, FAKE, FAKE, FAKE)) == INVALID
    assert dirstage(init=0) == INVALID
    assert dirstage(direction=2) == INVALID
    assert dirstage(mode=5) == INVALID
    assert dirstage(mode=3) == INVALID
    L = _native.load()
    bg = [P(FAKE)] * 5
    # the pair-format flags: split form only, one at a time, PAIRS_OUT with init == forcing
    st = L.mw_dirstage_f64(16, 8, 1.0, 1.0, 0.1, *bg, None, P(FAKE * 10), P(FAKE * 20), P(FAKE * 30), 0.1, 0, 2, 8,
                           None)
    assert st == INVALID
    st = L.mw_dirstage_f64(16, 8, 1.0, 1.0, 0.1, *bg, None, P(FAKE * 10), P(FAKE * 20), P(FAKE * 30), 0.1, 0, 1, 8,
                           None)
    assert st == INVALID and b"init == forcing" in L.mw_last_error()
    st = L.mw_dirstage_f64(16, 8, 1.0, 1.0, 0.1, *bg, None, P(FAKE * 10), P(FAKE * 20), P(FAKE * 30), 0.1, 0, 1, 24,
                           None)
    assert st == INVALID
    assert dirstage(init=FAKE * 10 + 4) == ALIGN
    assert dirstage(out=FAKE * 20) == ALIAS  # out == forcing
    assert dirstage(out=FAKE * 20 + 64) == ALIAS  # out overlaps forcing
    assert dirstage(out=FAKE * 10 + 8) == ALIAS  # out partially overlaps init
    assert b"forcing" in L.mw_last_error() or b"init" in L.mw_last_error()


def test_step_validation():
    L = _native.load()
    rv = ctypes.c_int(0)
    bg = [P(FAKE)] * 5
    st = L.mw_step_f64(16, 8, 1.0, 1.0, 0.1, 0.1, *bg, None, P(FAKE * 10), P(FAKE * 10), P(FAKE * 30), 1,
                       ctypes.byref(rv), 0, 1, None)
    assert st == ALIAS
    st = L.mw_step_f64(16, 8, 1.0, 1.0, 0.1, 0.1, *bg, None, P(FAKE * 10), P(FAKE * 20), P(FAKE * 30), 1, None, 0,
                       1, None)
    assert st == INVALID
    st = L.mw_step_f64(16, 8, 1.0, 1.0, 0.1, -0.1, *bg, None, P(FAKE * 10), P(FAKE * 20), P(FAKE * 30), 1,
                       ctypes.byref(rv), 0, 1, None)
    assert st == INVALID
    st = L.mw_step_f32(16, 8, 1.0, 1.0, 0.1, 0.1, *bg, None, P(FAKE * 10 + 2), P(FAKE * 20), P(FAKE * 30), 1,
                       ctypes.byref(rv), 1, None)
    assert st == ALIGN
    assert rv.value == 0  # untouched on failure


def test_init_and_stats_validation():
    L = _native.load()
    bub = (ctypes.c_double * 10)(3.0, 1e4, 2e3, 2e3, 2e3, 1.0, 1.0, 1.0, 0.0, 1.0)
    bg = [P(FAKE * (i + 2)) for i in range(5)]
    assert L.mw_init_f64(16, 8, 2e4, 1e4, 0, 0.0, 9, bub, P(FAKE), *bg, None) == INVALID
    assert L.mw_init_f64(16, 8, 2e4, 1e4, 0, 0.0, 2, bub, P(FAKE), *bg, None) == INVALID  # zero radius
    assert L.mw_init_f64(16, 8, 2e4, 1e4, 7, 0.0, 1, bub, P(FAKE), *bg, None) == INVALID  # background
    assert L.mw_init_f64(16, 8, -1.0, 1e4, 0, 0.0, 1, bub, P(FAKE), *bg, None) == INVALID
    need = L.mw_stats_workspace_bytes(16, 8)
    assert need == 16 * 8
    assert L.mw_stats_f64(16, 8, 1.0, 1.0, P(FAKE), P(FAKE), P(FAKE), P(FAKE * 4), need - 8, P(FAKE * 8),
                          None) == WORKSPACE
    assert L.mw_stats_workspace_bytes(8192, 4096) == 16 * 1024


def test_no_cpu_path():
    """Without a CUDA device the package refuses to allocate (no CPU fallback)."""
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from pyminiweather_gb300.data import initialize_fields
    from tests.helpers import make_params
    with pytest.raises(RuntimeError):
        initialize_fields(make_params(16, 8, "thermal"))


def test_ic_table_matches_oracle_table():
    """The product's initial-condition table and the oracle's are written
    independently; they must agree (ics/initial_conditions.py:96-268)."""
    from oracle import oracle as O
    from pyminiweather_gb300.ics.initial_conditions import IC_TYPES, ic_spec
    for ic in IC_TYPES:
        bg, u0, bub = O.ic_table(ic, 2e4)
        s = ic_spec(ic, 2e4)
        assert (s.background, s.u0, [tuple(b) for b in s.bubbles]) == (bg, u0, [tuple(b) for b in bub])
    with pytest.raises(NotImplementedError):
        ic_spec("injection", 2e4)


def test_ensemble_plan_validation():
    """Ensemble plans are built and checked on the host."""
    L = _native.load()
    M = _native.EnsMember
    info = _native.EnsPlanInfo()
    mem = (M * 2)(M(64, 32, 312.5, 312.5, 0.1, 0, 0, 0), M(100, 50, 200.0, 200.0, 0.1, 4 * 68 * 36, 36, 33))
    assert L.mw_ensemble_plan_info(2, mem, 16, ctypes.byref(info)) == OK
    assert info.n_x_items == 32 + 50
    assert info.n_z_items == 1 * 2 + 2 * 4  # (64-column blocks) x (16-row tiles) per member
    assert info.bytes % 16 == 0 and info.z_items_off >= info.x_items_off + 8 * info.n_x_items
    # the FP64 forms' row-constant table: one 40-byte entry per cell-centre background value used
    assert info.n_xrows == max(0 + 32 + 4, 36 + 50 + 4)
    assert info.xrows_off >= info.z_items_off + 8 * info.n_z_items and info.xrows_off % 16 == 0
    # then the members' stage constants (6 x 88 bytes each, 16-byte aligned), then the 16-byte work cursor last
    consts = (info.xrows_off + 40 * info.n_xrows + 15) // 16 * 16
    assert info.bytes == (consts + 2 * 6 * 88 + 15) // 16 * 16 + 16
    bad = (M * 2)(M(64, 32, 312.5, 312.5, 0.1, 0, 0, 0), M(100, 50, 200.0, 200.0, 0.1, 100, 36, 33))
    assert L.mw_ensemble_plan_info(2, bad, 16, ctypes.byref(info)) == ALIAS
    assert L.mw_ensemble_plan_info(2, mem, 65, ctypes.byref(info)) == INVALID
    one = (M * 1)(M(1, 32, 1.0, 1.0, 0.1, 0, 0, 0))
    assert L.mw_ensemble_plan_info(1, one, 16, ctypes.byref(info)) == SHAPE


def test_thermal_ensemble_generator():
    from pyminiweather_gb300.ensemble import thermal_ensemble
    a, b = thermal_ensemble(256, seed=0), thermal_ensemble(256, seed=0)
    assert [m[0]["nx"] for m in a] == [m[0]["nx"] for m in b]
    nx = [m[0]["nx"] for m in a]
    assert min(nx) >= 64 and max(nx) <= 1024 and all(n % 2 == 0 for n in nx)
    assert all(m[0]["nz"] * 2 == m[0]["nx"] for m in a)
    amps = [m[1][0][0] for m in a]
    assert 1.0 <= min(amps) and max(amps) <= 5.0
    # log-uniform: about half the members below the geometric mean 256
    assert 0.35 < np.mean(np.array(nx) < 256) < 0.65
    cells = sum(m[0]["nx"] * m[0]["nz"] for m in a)
    assert 15e6 < cells < 35e6


def test_python_constants_match_the_header():
    """The flag, enum and limit constants of the Python binding are the header's."""
    import os
    import re
    text = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                             "miniweather_gb300.h")).read()
    found = {}
    for name, val in re.findall(r"#define\s+(MW_[A-Z0-9_]+)\s+(\d+)u?\b", text):
        found[name] = int(val)
    for name, val in re.findall(r"\b(MW_[A-Z0-9_]+)\s*=\s*(\d+)\s*[,}/]", text):
        found[name] = int(val)
    names = [n for n in dir(_native) if n.startswith("MW_") and isinstance(getattr(_native, n), int)]
    assert len(names) >= 14
    for n in names:
        assert n in found, n
        assert getattr(_native, n) == found[n], n
