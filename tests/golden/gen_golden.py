"""Generate the golden fixtures in this folder by running the reference itself.

Run from the repository root, in a container that holds the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/gen_golden.py --ref <checkout of the reference>

The reference (shriram-jagan/pyminiweather) is imported with its NumPy/SciPy
backend.  Its module-global direction flag (pyminiweather/solve/step.py:18) is
reset before every run so each run starts as a fresh import does.  Outputs are
small .npz files; the GPU tests and the oracle tests read only these files.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(ref_root):
    os.environ.pop("LEGATE_MAX_DIM", None)
    os.environ.pop("LEGATE_MAX_FIELDS", None)
    sys.path.insert(0, ref_root)
    import pyminiweather  # noqa: F401
    from pyminiweather.data import initialize_fields
    from pyminiweather.ics import init
    from pyminiweather.mesh import MeshData
    from pyminiweather.post import compute_solution_variables, compute_stats
    from pyminiweather.solve import step as step_mod
    return dict(initialize_fields=initialize_fields, init=init, MeshData=MeshData, compute_stats=compute_stats,
                compute_solution_variables=compute_solution_variables, step=step_mod)


def params(nx, nz, ic_type, cfl=1.5, max_speed=450.0, xlen=2e4, zlen=1e4):
    p = dict(nx=nx, nz=nz, xlen=xlen, zlen=zlen, hs=2, s=4, ic_type=ic_type, cfl=cfl, max_speed=max_speed,
             nsteps=0, nwarmups=0, output_freq=-1)
    p["dx"] = p["xlen"] / p["nx"]
    p["dz"] = p["zlen"] / p["nz"]
    p["dt"] = np.minimum(p["dx"], p["dz"]) * p["cfl"] / p["max_speed"]
    return p


def setup(R, p):
    f = R["initialize_fields"](p)
    m = R["MeshData"](p)
    R["init"](f, p, m)
    R["step"].reverse_direction = False
    return f, m


def bg(f):
    return dict(hy_dens_cell=f.hy_dens_cell.copy(), hy_dens_theta_cell=f.hy_dens_theta_cell.copy(),
                hy_dens_int=f.hy_dens_int.copy(), hy_dens_theta_int=f.hy_dens_theta_int.copy(),
                hy_pressure_int=f.hy_pressure_int.copy())


def scalar_params(p):
    return {"p_" + k: np.array(v) for k, v in p.items() if isinstance(v, (int, float, np.floating, str))}


def run_case(R, name, nx, nz, ic_type, checkpoints, keep_tmp=True):
    p = params(nx, nz, ic_type)
    f, m = setup(R, p)
    out = dict(scalar_params(p))
    out.update(bg(f))
    out["state_0"] = f.state.copy()
    out["stats_0"] = np.array(R["compute_stats"](p, f))
    done = 0
    for c in checkpoints:
        while done < c:
            R["step"].evolve(p, f, m, dt=p["dt"])
            done += 1
        out["state_%d" % c] = f.state.copy()
        if keep_tmp:
            out["state_tmp_%d" % c] = f.state_tmp.copy()
        out["stats_%d" % c] = np.array(R["compute_stats"](p, f))
    out["svars_%d" % done] = R["compute_solution_variables"](p, f)
    out["checkpoints"] = np.array(checkpoints)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, {k: v.shape for k, v in out.items() if v.ndim > 0})


def run_stage_intermediates(R, name, nx, nz, ic_type, presteps):
    """One discrete_step per direction, recording the reference's intermediate
    arrays (vals, d3, flux, tend) and the halo it writes into the forcing array."""
    from pyminiweather.ics import Directions
    p = params(nx, nz, ic_type)
    f, m = setup(R, p)
    for _ in range(presteps):
        R["step"].evolve(p, f, m, dt=p["dt"])
    out = dict(scalar_params(p))
    out.update(bg(f))
    base = f.state.copy()
    out["state_in"] = base.copy()
    for dname, d in (("x", Directions.X), ("z", Directions.Z)):
        f.state[...] = base
        f.state_tmp[...] = base
        forcing = f.state.copy()
        out_arr = np.zeros_like(base)
        R["step"].discrete_step(p, f, m, f.state, forcing, out_arr, p["dt"] / 3, d)
        out["forcing_after_" + dname] = forcing
        out["out_" + dname] = out_arr
        if dname == "x":
            out["vals_x"], out["d3_vals_x"] = f.vals_x.copy(), f.d3_vals_x.copy()
        else:
            out["vals_z"], out["d3_vals_z"] = f.vals_z.copy(), f.d3_vals_z.copy()
        out["flux_" + dname] = f.flux.copy()
        out["tend_" + dname] = f.tend.copy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, {k: v.shape for k, v in out.items() if v.ndim > 0})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="path of the reference checkout")
    a = ap.parse_args()
    R = load_reference(a.ref)
    # configuration 0 of the benchmark: thermal 100x50, cfl 1.5, max_speed 450, 200 steps
    run_case(R, "thermal_100x50", 100, 50, "thermal", [1, 2, 200])
    # collision initial condition (the GPU-scale case) on a small grid
    run_case(R, "collision_64x32", 64, 32, "collision", [1, 20])
    # odd, tile-unfriendly sizes
    run_case(R, "collision_37x13", 37, 13, "collision", [3], keep_tmp=True)
    # the other initial conditions, including the gravity-wave forcing
    run_case(R, "gravity_48x24", 48, 24, "gravity", [5, 100])
    run_case(R, "density_current_40x20", 40, 20, "density-current", [5])
    # per-stage intermediates
    run_stage_intermediates(R, "stage_collision_24x12", 24, 12, "collision", presteps=3)


if __name__ == "__main__":
    main()
