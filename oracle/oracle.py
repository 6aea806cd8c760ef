"""NumPy/ctypes front end of the C oracle (test infrastructure only).

Restates the reference's parameter handling and initial-condition table
independently of the product package, so that the CUDA path is checked
against code that shares nothing with it:

- dt from the CFL rule, pyminiweather/__main__.py:190-195;
- ic_type -> background and bubbles, pyminiweather/ics/initial_conditions.py:96-268;
- the module-global direction flag of solve/step.py:18,103-109,143, kept here
  per simulation (``reverse``), starting as a fresh import does (False).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmw_oracle.so")
SRC = os.path.join(HERE, "mw_oracle.c")

HS = 2
DIR_X, DIR_Z = 0, 1
BG_CONST_THETA, BG_BVFREQ = 0, 1

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile mw_oracle.c with gcc (-ffp-contract=off keeps NumPy's rounding order)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "mw_oracle.h"))
    ):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd, cwd=HERE)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            d, i, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
            L.mwo_max_threads.restype = i
            L.mwo_set_threads.argtypes = [i]
            L.mwo_init.argtypes = [i, i, d, d, i, d, i, P, P, P, P, P, P, P]
            L.mwo_gravity_source.argtypes = [i, i, d, d, P, P]
            L.mwo_dirstage.argtypes = [i, i, d, d, d, P, P, P, P, P, P, P, P, P, d, i]
            L.mwo_evolve.argtypes = [i, i, d, d, d, P, P, P, P, P, P, P, P, i, ctypes.POINTER(i)]
            L.mwo_stats.argtypes = [i, i, d, d, P, P, P, P]
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def ic_table(ic_type: str, xlen: float):
    """(background, u0, bubbles) per ic_type, ics/initial_conditions.py:96-268.
    A bubble is (amplitude K, x0, z0, xrad, zrad)."""
    if ic_type == "thermal":
        return BG_CONST_THETA, 0.0, [(3.0, xlen / 2, 2000.0, 2000.0, 2000.0)]
    if ic_type == "collision":
        return BG_CONST_THETA, 0.0, [(20.0, xlen / 2, 2000.0, 2000.0, 2000.0),
                                     (-20.0, xlen / 2, 8000.0, 2000.0, 2000.0)]
    if ic_type == "density-current":
        return BG_CONST_THETA, 0.0, [(-20.0, xlen / 2, 5000.0, 4000.0, 2000.0)]
    if ic_type == "gravity":
        return BG_BVFREQ, 15.0, []
    raise ValueError("unsupported ic_type %r" % ic_type)


def make_params(nx, nz, ic_type="thermal", xlen=2e4, zlen=1e4, cfl=1.5, max_speed=450.0, dt=None):
    """The params dict of pyminiweather/__main__.py:160-195."""
    p = dict(nx=nx, nz=nz, xlen=xlen, zlen=zlen, hs=2, s=4, ic_type=ic_type, cfl=cfl, max_speed=max_speed)
    p["dx"] = p["xlen"] / p["nx"]
    p["dz"] = p["zlen"] / p["nz"]
    p["dt"] = dt if dt is not None else (min(p["dx"], p["dz"]) * cfl / max_speed)
    return p


class OracleSim:
    """State and backgrounds of one simulation, advanced by the C oracle."""

    def __init__(self, params, bubbles=None, threads: int = 0):
        self.p = dict(params)
        L = lib()
        if threads:
            L.mwo_set_threads(int(threads))
        nx, nz = self.p["nx"], self.p["nz"]
        bg, u0, bub = ic_table(self.p["ic_type"], self.p["xlen"])
        if bubbles is not None:
            bub = list(bubbles)
        self.bg, self.u0, self.bubbles = bg, u0, bub
        shape = (4, nz + 2 * HS, nx + 2 * HS)
        self.state = np.zeros(shape)
        self.hy_dens_cell = np.zeros(nz + 2 * HS)
        self.hy_dens_theta_cell = np.zeros(nz + 2 * HS)
        self.hy_dens_int = np.zeros(nz + 1)
        self.hy_dens_theta_int = np.zeros(nz + 1)
        self.hy_pressure_int = np.zeros(nz + 1)
        barr = np.ascontiguousarray(np.array(bub, dtype=np.float64).reshape(-1))
        L.mwo_init(nx, nz, self.p["xlen"], self.p["zlen"], bg, u0, len(bub), _p(barr) if len(bub) else None,
                   _p(self.state), _p(self.hy_dens_cell), _p(self.hy_dens_theta_cell), _p(self.hy_dens_int),
                   _p(self.hy_dens_theta_int), _p(self.hy_pressure_int))
        self.state_tmp = self.state.copy()
        self.src_w = None
        if self.p["ic_type"] == "gravity":
            self.src_w = np.zeros((nz, nx))
            L.mwo_gravity_source(nx, nz, self.p["xlen"], self.p["zlen"], _p(self.hy_dens_cell), _p(self.src_w))
        self.reverse = 0

    def backgrounds(self):
        return (self.hy_dens_cell, self.hy_dens_theta_cell, self.hy_dens_int, self.hy_dens_theta_int,
                self.hy_pressure_int)

    def dirstage(self, init, forcing, out, dt_stage, direction):
        p = self.p
        hb = [_p(a) for a in self.backgrounds()]
        lib().mwo_dirstage(p["nx"], p["nz"], p["dx"], p["dz"], p["dt"], *hb, _p(self.src_w), _p(init),
                           _p(forcing), _p(out), dt_stage, direction)

    def evolve(self, nsteps=1, dt=None):
        p = self.p
        dt = p["dt"] if dt is None else dt
        rv = ctypes.c_int(self.reverse)
        hb = [_p(a) for a in self.backgrounds()]
        lib().mwo_evolve(p["nx"], p["nz"], p["dx"], p["dz"], dt, *hb, _p(self.src_w), _p(self.state),
                         _p(self.state_tmp), int(nsteps), ctypes.byref(rv))
        self.reverse = rv.value

    def stats(self, state=None):
        p = self.p
        st = self.state if state is None else np.ascontiguousarray(state)
        out = np.zeros(2)
        lib().mwo_stats(p["nx"], p["nz"], p["dx"], p["dz"], _p(self.hy_dens_cell), _p(self.hy_dens_theta_cell),
                        _p(st), _p(out))
        return float(out[0]), float(out[1])


def normwise_error(a, b, hs=HS):
    """Per-variable max|a-b| / max|b| over the interior cells."""
    a = np.asarray(a)[:, hs:-hs, hs:-hs]
    b = np.asarray(b)[:, hs:-hs, hs:-hs]
    out = []
    for v in range(a.shape[0]):
        den = np.abs(b[v]).max()
        num = np.abs(a[v] - b[v]).max()
        out.append(float(num / den) if den > 0 else float(num))
    return out
