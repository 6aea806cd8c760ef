"""Build libminiweather_gb300.so from csrc/*.cu for sm_103a, in-tree.

    python -m pyminiweather_gb300.build [--force] [--ptxas-info] [--check]

With --check (or MW_LIBRARY_VARIANT=check in the environment of the process
that loads the package) the bounds-checked debug library
libminiweather_gb300_check.so is built (MW_CHECK=1: every kernel counts
out-of-range indices instead of accessing memory there) and loaded.

Each translation unit is compiled by nvcc in parallel and linked into
pyminiweather_gb300/_lib/libminiweather_gb300.so (static CUDA runtime).  The
library is rebuilt only when a source or header is newer than it.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I" + INCLUDE]


def configure(variant: str) -> None:
    """Select the library variant: "" (the product) or "check" (bounds-checked)."""
    global VARIANT, BUILD_DIR, LIB_NAME, LIB_PATH, NVCC_FLAGS
    if variant not in ("", "check"):
        raise ValueError("unknown library variant %r (expected '' or 'check')" % variant)
    VARIANT = variant
    BUILD_DIR = os.path.join(PKG, "_build", variant) if variant else os.path.join(PKG, "_build")
    LIB_NAME = "libminiweather_gb300%s.so" % ("_" + variant if variant else "")
    LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)
    NVCC_FLAGS = BASE_FLAGS + (["-DMW_CHECK=1"] if variant == "check" else [])


configure(os.environ.get("MW_LIBRARY_VARIANT", ""))


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libminiweather_gb300")
    return cand


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) + [
        os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(src: str, ptxas_info: bool) -> tuple[str, str]:
    obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (os.path.basename(src), r.stdout, r.stderr))
    return obj, r.stderr


def build(force: bool = False, ptxas_info: bool = False, verbose: bool = False) -> str:
    if not force and not ptxas_info and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_info), srcs))
    if ptxas_info or verbose:
        for (_, log), src in zip(results, srcs):
            if log.strip():
                print("== %s\n%s" % (os.path.basename(src), log), file=sys.stderr)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    ap.add_argument("--check", action="store_true", help="build the bounds-checked debug library")
    a = ap.parse_args()
    if a.check:
        configure("check")
    print(build(force=a.force, ptxas_info=a.ptxas_info, verbose=True))
