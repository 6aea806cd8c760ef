"""Initial-condition table, pyminiweather/ics/initial_conditions.py:96-429.

Each ic_type of the reference is a background profile, a constant wind and a
list of cos^2 potential-temperature bubbles; the initial-condition kernel
(mw_init_*) evaluates them.  The injection case is rejected, as the reference
itself flags it unsupported.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

from .. import _native

IC_TYPES = ("thermal", "collision", "gravity", "density-current")


@dataclass
class ICSpec:
    background: int  # _native.MW_BG_CONST_THETA or _native.MW_BG_BVFREQ
    u0: float = 0.0
    bubbles: List[Tuple[float, float, float, float, float]] = field(default_factory=list)
    # (amplitude K, x0, z0, xrad, zrad)


def ic_spec(ic_type: str, xlen: float) -> ICSpec:
    if ic_type == "thermal":  # ThermalInterior, :166-199
        return ICSpec(_native.MW_BG_CONST_THETA, 0.0, [(3.0, xlen / 2, 2000.0, 2000.0, 2000.0)])
    if ic_type == "collision":  # CollisionInterior, :96-134
        return ICSpec(_native.MW_BG_CONST_THETA, 0.0, [(20.0, xlen / 2, 2000.0, 2000.0, 2000.0),
                                                       (-20.0, xlen / 2, 8000.0, 2000.0, 2000.0)])
    if ic_type == "density-current":  # DensityCurrentInterior, :236-268
        return ICSpec(_native.MW_BG_CONST_THETA, 0.0, [(-20.0, xlen / 2, 5000.0, 4000.0, 2000.0)])
    if ic_type == "gravity":  # GravityWavesInterior, :202-233 (constant N = 0.02, u = 15 m/s)
        return ICSpec(_native.MW_BG_BVFREQ, 15.0, [])
    if ic_type == "injection":
        raise NotImplementedError("the injection initial condition is flagged unsupported by the reference")
    raise ValueError("unknown ic_type %r" % (ic_type,))
