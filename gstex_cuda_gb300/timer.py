"""Named section timer with the interface of the reference's
``gstex_cuda.timer.Timer`` (gstex_cuda/timer.py:4-75), used by training loops
(example.py:121-185 of the reference) to time preprocess / project / render.

``start(key)`` opens an interval for ``key`` (closing nothing: an interval
that was started and not stopped is dropped), ``stop()`` closes it.  Each
interval is measured twice: host wall-clock time, and CUDA events recorded on
the current stream (``cuda_support=True``), which time the GPU work queued in
between.  ``dump()`` synchronises the device and prints one ``key<TAB>ms``
line per key (event time when CUDA timing is on, else wall time) and a
``TOTAL`` line.
"""
from __future__ import annotations

import time
from typing import Dict, List, Optional, Tuple

import torch


class Timer:
    def __init__(self, cuda_support: bool = True, disabled: bool = False):
        self.cuda_support = bool(cuda_support) and torch.cuda.is_available()
        self.disabled = disabled
        self.laps = 0
        self.key: Optional[str] = None
        self.times: Dict[str, float] = {}  # key -> accumulated wall seconds
        self.intervals: Dict[str, List[Tuple[torch.cuda.Event, torch.cuda.Event]]] = {}
        self._t0 = 0.0
        self._open: Optional[torch.cuda.Event] = None

    def start(self, key: str) -> None:
        if self.disabled:
            return
        self.key = key
        self.times.setdefault(key, 0.0)
        self.intervals.setdefault(key, [])
        if self.cuda_support:
            self._open = torch.cuda.Event(enable_timing=True)
            self._open.record()
        self._t0 = time.time()

    def stop(self) -> None:
        if self.disabled or self.key is None:
            return
        self.times[self.key] += time.time() - self._t0
        if self.cuda_support:
            end = torch.cuda.Event(enable_timing=True)
            end.record()
            self.intervals[self.key].append((self._open, end))
        self.key = None
        self._open = None

    def lap(self) -> None:
        if not self.disabled:
            self.laps += 1

    def dump_key(self, key: str):
        """Prints and returns (wall ms, CUDA-event ms) of ``key`` (event ms is 0
        without CUDA timing)."""
        if self.disabled:
            return None
        wall = 1000.0 * self.times[key]
        event = sum(a.elapsed_time(b) for a, b in self.intervals[key]) if self.cuda_support else 0.0
        print(f"{key}\t{(event if self.cuda_support else wall):.3f}")
        return wall, event

    def dump(self) -> None:
        if self.disabled:
            return
        if self.cuda_support:
            torch.cuda.synchronize()
        total = 0.0
        for key in self.times:
            wall, event = self.dump_key(key)
            total += event if self.cuda_support else wall
        print(f"TOTAL\t{total:.3f}")
