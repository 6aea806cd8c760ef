"""The command-line driver end to end and checkpoint / restart, on the GPU.

The driver's text output is compared with the reference's run of the same
case (thermal 100 x 50, cfl 1.5, max speed 450: the golden fixture's
checkpoints at steps 1 and 2), and with np.savetxt of the driver's own
arrays byte for byte."""
import io
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from pyminiweather_gb300.checkpoint import load_checkpoint, save_checkpoint
from pyminiweather_gb300.data import initialize_fields
from pyminiweather_gb300.ics import init
from pyminiweather_gb300.solve import evolve, reset_direction
from tests.helpers import TOL_STEP, golden, make_params, normwise

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run_cli(args, cwd):
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "pyminiweather_gb300"] + args, cwd=cwd, capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    return r.stderr + r.stdout


def test_cli_output_matches_reference_run(tmp_path):
    g = golden("thermal_100x50")
    log = _run_cli(["--nx", "100", "--nz", "50", "--ic-type", "thermal", "--cfl", "1.5", "--max-speed", "450",
                    "--nsteps", "3", "--output-freq", "1", "--app-filename", "out.txt"], str(tmp_path))
    for needle in ("Elapsed time for initialization:", "Start: total_mass, total_energy:", "Step: 0, max(rho*t):",
                   "Step: 2, max(rho*t):", "Elapsed time for timestepping:", "End: total_mass, total_energy:",
                   "Relative change in total_mass, total_energy:"):
        assert needle in log, (needle, log)
    shape = (4, 54, 104)
    text = (tmp_path / "out.txt").read_bytes()
    states = np.loadtxt(io.BytesIO(text), delimiter=",").reshape(3, *shape)  # outputs before steps 0, 1, 2
    fh = io.BytesIO()
    for s in states:
        np.savetxt(fh, s.reshape(-1, shape[-1]), delimiter=",")
    assert fh.getvalue() == text  # the bytes np.savetxt writes for these arrays
    assert max(normwise(states[0], g["state_0"], interior=False)) <= 1e-13  # the initial condition
    for c in (1, 2):
        assert max(normwise(states[c], g["state_%d" % c])) <= TOL_STEP
    svars = np.loadtxt(tmp_path / "out_svars.txt", delimiter=",").reshape(3, 4, 50, 100)
    assert np.isfinite(svars).all()
    for c in range(3):  # rho' of the solution variables is the state's, exactly
        assert np.array_equal(svars[c][0], states[c][0, 2:-2, 2:-2])


def test_checkpoint_restart_is_bit_identical(tmp_path):
    p = make_params(64, 32, "collision")
    ref = initialize_fields(p)
    init(ref, p, None)
    reset_direction()
    evolve(p, ref, None, dt=p["dt"], nsteps=5)

    f = initialize_fields(p)
    init(f, p, None)
    reset_direction()
    evolve(p, f, None, dt=p["dt"], nsteps=3)
    ck = str(tmp_path / "ck.npz")
    save_checkpoint(ck, p, f, 3)
    g = initialize_fields(p)
    init(g, p, None)
    reset_direction()  # a fresh process: the flag is back at its initial value
    assert load_checkpoint(ck, p, g) == 3
    evolve(p, g, None, dt=p["dt"], nsteps=2)
    assert torch.equal(g.state, ref.state)
    with pytest.raises(ValueError):
        load_checkpoint(ck, make_params(64, 32, "thermal"), g)


def test_cli_restart_continues_the_run(tmp_path):
    common = ["--nx", "48", "--nz", "24", "--ic-type", "collision"]
    _run_cli(common + ["--nsteps", "4", "--checkpoint-file", "full.npz"], str(tmp_path))
    _run_cli(common + ["--nsteps", "2", "--checkpoint-file", "half.npz"], str(tmp_path))
    log = _run_cli(common + ["--nsteps", "2", "--restart-file", "half.npz", "--checkpoint-file", "resumed.npz"],
                   str(tmp_path))
    assert "Restart from half.npz at step 2" in log
    a, b = np.load(tmp_path / "full.npz"), np.load(tmp_path / "resumed.npz")
    assert int(a["step"]) == int(b["step"]) == 4
    assert np.array_equal(a["state"], b["state"]) and bool(a["reverse_direction"]) == bool(b["reverse_direction"])
