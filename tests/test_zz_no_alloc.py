"""mw_step_f64_noalloc, the time step for callers that cannot allocate.

A host model that owns every buffer it hands over, a framework custom call
whose buffers are all pre-allocated, or a real-time loop that forbids
allocation once running cannot give mw_step_f64 its third state-sized array;
the no-allocation entry point uses a fixed array inside the library instead
(grids up to 512 x 256 cells).  These tests call it through the C ABI and
compare it with mw_step_f64 on the same inputs, two calls in a row.

This file is named to be collected last, so that a run stopping at its first
failure has already run every other test.  It sets up everything it uses and
passes alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from pyminiweather_gb300 import _native
from pyminiweather_gb300.data import initialize_fields
from pyminiweather_gb300.ics import init
from tests.helpers import TOL_STEP, make_params, normwise

pytestmark = pytest.mark.gpu


def _args(p, f):
    return [f.nx, f.nz, p["dx"], p["dz"], p["dt"], p["dt"], *[_native.ptr(a) for a in f.backgrounds()],
            _native.ptr(f.src_w)]


@pytest.mark.parametrize("mode", ["split", "native"])
@pytest.mark.parametrize("ic,nx,nz", [("collision", 256, 128), ("gravity", 48, 24), ("thermal", 512, 256)])
def test_noalloc_step_matches_regular_step(mode, ic, nx, nz):
    p = make_params(nx, nz, ic)
    ref = initialize_fields(p)  # the regular entry point gets a scratch array of ours
    init(ref, p)
    new = initialize_fields(p)
    init(new, p)
    new.scratch = None  # the no-allocation entry point never sees a third array
    m = _native.F64_MODES[mode]
    stream = _native.stream_handle()
    rv_ref, rv_new = ctypes.c_int(0), ctypes.c_int(0)
    for call in range(2):
        _native.call("mw_step_f64", *_args(p, ref), _native.ptr(ref.state), _native.ptr(ref.state_tmp),
                     _native.ptr(ref.scratch), 3, ctypes.byref(rv_ref), m, _native.MW_FLAG_WRITE_HALO, stream)
        _native.call("mw_step_f64_noalloc", *_args(p, new), _native.ptr(new.state), _native.ptr(new.state_tmp), 3,
                     ctypes.byref(rv_new), m, _native.MW_FLAG_WRITE_HALO, stream)
        torch.cuda.synchronize()
        a, b = new.state.cpu().numpy(), ref.state.cpu().numpy()
        at, bt = new.state_tmp.cpu().numpy(), ref.state_tmp.cpu().numpy()
        err = max(normwise(a, b, interior=False) + normwise(at, bt, interior=False))
        print("%s %s %dx%d call %d: max normwise %.2e, identical %s" % (mode, ic, nx, nz, call + 1, err,
                                                                      np.array_equal(a, b) and np.array_equal(at, bt)))
        assert err <= TOL_STEP
        assert rv_new.value == rv_ref.value == (call + 1) % 2


def test_noalloc_rejects_grids_beyond_its_array():
    L = _native.load()
    rv = ctypes.c_int(0)
    fake = ctypes.c_void_p(1 << 20)  # never dereferenced: the size check comes first
    st = L.mw_step_f64_noalloc(1024, 512, 1.0, 1.0, 0.1, 0.1, *([fake] * 5), None, fake, fake, 1, ctypes.byref(rv),
                               _native.MW_F64_SPLIT, _native.MW_FLAG_WRITE_HALO, None)
    assert st == 6  # MW_ERR_WORKSPACE
    assert b"512 x 256" in L.mw_last_error()
    assert rv.value == 0


@pytest.mark.parametrize("mode", ["split", "native"])
def test_noalloc_check_finite_flag(mode):
    """MW_FLAG_CHECK_FINITE is honoured without allocating: a NaN planted in the
    state on the host makes the call return MW_ERR_NONFINITE (7), a clean state
    MW_OK, as mw_step_f64 does."""
    p = make_params(64, 32, "thermal")
    f = initialize_fields(p)
    init(f, p)
    L = _native.load()
    m = _native.F64_MODES[mode]
    flags = _native.MW_FLAG_WRITE_HALO | _native.MW_FLAG_CHECK_FINITE
    stream = _native.stream_handle()
    rv = ctypes.c_int(0)
    st = L.mw_step_f64_noalloc(*_args(p, f), _native.ptr(f.state), _native.ptr(f.state_tmp), 1, ctypes.byref(rv), m,
                               flags, stream)
    assert st == 0, L.mw_last_error()
    f.state[3, 10, 20] = float("nan")  # planted on the host side of the API, not by a kernel fault
    st = L.mw_step_f64_noalloc(*_args(p, f), _native.ptr(f.state), _native.ptr(f.state_tmp), 1, ctypes.byref(rv), m,
                               flags, stream)
    torch.cuda.synchronize()
    assert st == 7, (st, L.mw_last_error())
    assert b"non-finite" in L.mw_last_error()
