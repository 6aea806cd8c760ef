"""Pin the CPU oracle against outputs of the reference itself (tests/golden).

The oracle is the checker of every GPU parity test, so it is held to tighter
bounds than the GPU path: rounding-level agreement (the residual is the
reference machine's SVML pow, about 1 ulp away from libm's).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import BACKGROUNDS, CASES, TOL_STEP, golden, normwise


@pytest.mark.parametrize("name,ic,nx,nz", CASES)
def test_oracle_initial_condition(name, ic, nx, nz):
    g = golden(name)
    p = O.make_params(nx, nz, ic)
    assert p["dt"] == float(g["p_dt"])
    s = O.OracleSim(p)
    for k in BACKGROUNDS:
        b = g[k]
        assert np.abs(getattr(s, k) - b).max() <= 1e-15 * np.abs(b).max(), k
    # the initial condition covers the halo cells too (ics/initial.py:57-77)
    for v in range(4):
        b = g["state_0"][v]
        assert np.abs(s.state[v] - b).max() <= 1e-14 * max(np.abs(b).max(), 1e-300), v
    m, e = s.stats()
    np.testing.assert_allclose([m, e], g["stats_0"], rtol=1e-14)


@pytest.mark.parametrize("name,ic,nx,nz", CASES)
def test_oracle_time_steps(name, ic, nx, nz):
    g = golden(name)
    s = O.OracleSim(O.make_params(nx, nz, ic))
    done = 0
    tight = 1e-11 if ic != "gravity" else TOL_STEP  # gravity-case fields are tiny, so normwise is looser
    for c in g["checkpoints"]:
        c = int(c)
        s.evolve(c - done)
        done = c
        err = normwise(s.state, g["state_%d" % c])
        assert max(err) <= tight, (c, err)
        # halo included: the oracle writes halos as the reference does
        errh = normwise(s.state, g["state_%d" % c], interior=False)
        assert max(errh) <= tight, (c, errh)
        if "state_tmp_%d" % c in g:
            errt = normwise(s.state_tmp, g["state_tmp_%d" % c], interior=False)
            assert max(errt) <= tight, (c, errt)
        np.testing.assert_allclose(s.stats(), g["stats_%d" % c], rtol=1e-13)


def test_oracle_direction_toggle():
    """Two single steps equal one two-step call, and the flag toggles (step.py:143)."""
    p = O.make_params(24, 12, "collision")
    a, b = O.OracleSim(p), O.OracleSim(p)
    a.evolve(1)
    assert a.reverse == 1
    a.evolve(1)
    b.evolve(2)
    assert a.reverse == b.reverse == 0
    assert np.array_equal(a.state, b.state)


def test_oracle_stage_intermediates_consistent():
    """One x and one z direction-stage of the oracle reproduce the reference's
    outputs of discrete_step, halo writes included."""
    g = golden("stage_collision_24x12")
    p = O.make_params(24, 12, "collision")
    s = O.OracleSim(p)
    for k in BACKGROUNDS:
        getattr(s, k)[...] = g[k]
    for d, name in ((O.DIR_X, "x"), (O.DIR_Z, "z")):
        init = g["state_in"].copy()
        forcing = g["state_in"].copy()
        out = np.zeros_like(init)
        s.dirstage(init, forcing, out, p["dt"] / 3, d)
        np.testing.assert_allclose(forcing, g["forcing_after_" + name], rtol=0, atol=1e-12)
        ref = g["out_" + name]
        for v in range(4):
            assert np.abs(out[v, 2:-2, 2:-2] - ref[v, 2:-2, 2:-2]).max() <= 1e-14 * np.abs(ref[v]).max() + 1e-300
