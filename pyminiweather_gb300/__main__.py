"""Command-line driver, the counterpart of pyminiweather/__main__.py:28-248:
the same flags, warm-up steps, log lines and text output, with the time
stepping on the GPU.

    python -m pyminiweather_gb300 --nx 400 --nz 200 --nsteps 100 --ic-type collision

Flags beyond the reference's: --f64-mode (split | native), --fp32 (the FP32
precision form), --checkpoint-file / --checkpoint-freq (write the state, the
direction parity and the step count every k steps) and --restart-file (start
from such a checkpoint instead of the initial condition).
"""
from __future__ import annotations

import argparse
import logging
import sys
from pathlib import Path

import torch


def get_logger(filename=None):
    logger = logging.getLogger("pyminiweather")
    handler = logging.StreamHandler() if filename is None else logging.FileHandler(filename, mode="w")
    handler.setFormatter(logging.Formatter("%(message)s"))
    logger.addHandler(handler)
    logger.setLevel(logging.INFO)
    return logger


def get_parser():
    p = argparse.ArgumentParser(prog="python -m pyminiweather_gb300")
    p.add_argument("--nx", type=int, default=200, dest="nx", help="Number of points in x-direction (default: 200)")
    p.add_argument("--nz", type=int, default=100, dest="nz", help="Number of points in z-direction (default: 100)")
    p.add_argument("--xlen", type=float, default=2e4, dest="xlen", help="Length of domain in x-direction (default: 2e4)")
    p.add_argument("--zlen", type=float, default=1e4, dest="zlen", help="Length of domain in z-direction (default: 1e4)")
    p.add_argument("--nsteps", type=int, default=10, dest="nsteps", help="Number of time steps (default: 10)")
    p.add_argument("--dt", type=float, default=None, dest="dt", help="Time step size (if none, calculated using CFL)")
    p.add_argument("--nwarmups", type=int, default=0, dest="nwarmups", help="Number of warmup time steps (default: 0)")
    p.add_argument("--ic-type", type=str, default="thermal", dest="ic_type",
                   choices=["thermal", "collision", "gravity", "density-current", "injection"],
                   help="Type of initial condition. The default value is thermal.")
    p.add_argument("--hs", type=int, default=2, choices=[2], dest="hs", help="Stencil half width (fixed at 2)")
    p.add_argument("--s", type=int, default=4, choices=[4], dest="s", help="Interpolation kernel size (fixed at 4)")
    p.add_argument("--max-speed", type=float, default=500.0, dest="max_speed",
                   help="Assumed maximum speed used for the time step (default: 500)")
    p.add_argument("--cfl", type=float, default=1.00, dest="cfl", help="CFL number for the time step (default: 1.0)")
    p.add_argument("--verbose", action="store_true", default=False, dest="verbose",
                   help="Print the simulation parameters")
    p.add_argument("--output-freq", type=int, default=-1, dest="output_freq",
                   help="Write the state and solution variables every output-freq steps (default: -1, off)")
    p.add_argument("--app-filename", type=str, default="PyMiniWeatherData.txt", dest="app_filename",
                   help="Output file of the state (default: PyMiniWeatherData.txt)")
    p.add_argument("--app-log-file", action="store", type=Path, default=None, metavar="FILE",
                   help="Write messages from the application to a file")
    p.add_argument("--f64-mode", type=str, default="fp64", choices=["fp64", "native", "split"], dest="f64_mode",
                   help="FP64 arithmetic form: fp64 (IEEE FP64, fewest operations; default), native (IEEE FP64, "
                        "the reference's formulas) or split (double-FP32 interior, not IEEE FP64)")
    p.add_argument("--fp32", action="store_true", default=False, dest="fp32",
                   help="FP32 perturbation fields (the precision form)")
    p.add_argument("--checkpoint-file", type=str, default=None, dest="checkpoint_file",
                   help="Write a restart checkpoint (.npz) to this file")
    p.add_argument("--checkpoint-freq", type=int, default=-1, dest="checkpoint_freq",
                   help="Checkpoint every checkpoint-freq steps and at the end (default: -1, at the end only)")
    p.add_argument("--restart-file", type=str, default=None, dest="restart_file",
                   help="Start from this checkpoint instead of the initial condition")
    return p


def get_params_from_args(args):
    keys = ("nx", "nz", "xlen", "zlen", "dt", "nsteps", "nwarmups", "ic_type", "hs", "s", "max_speed", "cfl",
            "output_freq", "app_filename", "app_log_file", "verbose")
    params = {k: getattr(args, k) for k in keys}
    params["f64_mode"] = args.f64_mode
    params["dtype"] = torch.float32 if args.fp32 else torch.float64
    return params


def main(argv=None):
    from .checkpoint import load_checkpoint, save_checkpoint
    from .data import initialize_fields
    from .ics import init
    from .mesh import MeshData
    from .post import compute_stats
    from .post.output import write_output
    from .solve import evolve
    from .utils import TimedCodeBlock

    args, _ = get_parser().parse_known_args(argv)
    params = get_params_from_args(args)
    logger = get_logger(args.app_log_file)

    params["dx"] = params["xlen"] / params["nx"]
    params["dz"] = params["zlen"] / params["nz"]
    if params["dt"] is None:
        params["dt"] = min(params["dx"], params["dz"]) * params["cfl"] / params["max_speed"]
    if params["verbose"]:
        for k, v in params.items():
            logger.info(f"{k:25s} {v}")

    with TimedCodeBlock(label="Elapsed time for initialization"):
        fields = initialize_fields(params)
        mesh = MeshData(params)
        init(fields, params, mesh)
        first = 0
        if args.restart_file:
            first = load_checkpoint(args.restart_file, params, fields)
            logger.info(f"Restart from {args.restart_file} at step {first}")

    total_mass_start, total_energy_start = compute_stats(params, fields)
    logger.info(f"Start: total_mass, total_energy: {total_mass_start}, {total_energy_start}")

    if params["nwarmups"]:
        with TimedCodeBlock(label="Elapsed time for warmups"):
            for _ in range(params["nwarmups"]):
                evolve(params, fields, mesh, dt=params["dt"])

    file_touched = False
    with TimedCodeBlock(label="Elapsed time for timestepping"):
        for istep in range(params["nsteps"]):
            if params["output_freq"] > 0 and (istep + 1) % params["output_freq"] == 0:
                logger.info(f"Step: {istep}, max(rho*t): {float(fields.state[3].max())}")
                write_output(params, fields, append=file_touched)
                file_touched = True
            evolve(params, fields, mesh, dt=params["dt"])
            if args.checkpoint_file and args.checkpoint_freq > 0 and (istep + 1) % args.checkpoint_freq == 0:
                save_checkpoint(args.checkpoint_file, params, fields, first + params["nwarmups"] + istep + 1)
    if args.checkpoint_file:
        save_checkpoint(args.checkpoint_file, params, fields, first + params["nwarmups"] + params["nsteps"])

    total_mass_end, total_energy_end = compute_stats(params, fields)
    logger.info(f"End: total_mass, total_energy: {total_mass_end}, {total_energy_end}")
    total_mass_change = (total_mass_end - total_mass_start) / total_mass_start
    total_energy_change = (total_energy_end - total_energy_start) / total_energy_start
    logger.info(f"Relative change in total_mass, total_energy: {total_mass_change}, {total_energy_change}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
