"""Timing, the counterpart of pyminiweather/utils/timing.py:15-36: wall clock
plus CUDA events on the current stream, logged on exit."""
from __future__ import annotations

import logging
import time

import torch


class TimedCodeBlock:
    def __init__(self, label: str = "", logger: str = "pyminiweather"):
        self.label = label
        self.logger = logging.getLogger(logger)
        self.elapsed_s = None
        self.device_ms = None

    def __enter__(self):
        self._e0 = torch.cuda.Event(enable_timing=True)
        self._e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        self._t0 = time.perf_counter()
        self._e0.record()
        return self

    def __exit__(self, *exc):
        self._e1.record()
        self._e1.synchronize()
        self.elapsed_s = time.perf_counter() - self._t0
        self.device_ms = self._e0.elapsed_time(self._e1)
        self.logger.info("%s: %s s", self.label, self.elapsed_s)
        return False
