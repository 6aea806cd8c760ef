"""pyminiweather_gb300: the PyMiniWeather finite-volume time step on GB300 (sm_103a).

Drop-in for the solver path of shriram-jagan/pyminiweather: the same module
layout and entry points (data.initialize_fields, ics.init, solve.evolve,
solve.discrete_step, post.compute_stats, ...), with arrays held as CUDA
tensors and every computation done by the hand-written kernels of
libminiweather_gb300.so (C ABI in include/miniweather_gb300.h).  There is no
CPU path: without a CUDA device or the library, the entry points raise.
"""
from enum import IntEnum

__version__ = "0.1.0"
backend = "gb300"


class IDS(IntEnum):
    """Variable order of the state, pyminiweather/__init__.py:14-18."""

    DENS = 0
    UMOM = 1
    WMOM = 2
    RHOT = 3
