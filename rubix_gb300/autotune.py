"""Autotuner for the work-item shape of the cube kernels.

The fused accumulate kernel and its adjoint process each spaxel in chunks of
``chunk`` particles and schedule large single-chunk spaxels first
(``rubix_cube_tuning_set``).  The best chunk depends on how particles spread over
spaxels (a 16x16 grid holding 1e6 particles wants different chunks from a
150x150 grid holding 1e6), so ``autotune`` times a few candidates on the caller's
own launch with CUDA events, keeps the fastest for the device and caches the choice
by a caller-supplied key (for example the batch layout).  Results differ between
chunk sizes only in the summation order of spaxels longer than one chunk.
"""

from __future__ import annotations

import ctypes
import threading
from typing import Callable, Dict, Hashable, Iterable, Optional, Tuple

import torch

from . import _lib

CANDIDATES: Tuple[Tuple[int, int], ...] = ((256, 64), (192, 64), (128, 64), (256, 16),
                                           (128, 16), (64, 16))

_cache: Dict[Hashable, Tuple[int, int]] = {}
_lock = threading.Lock()


class _Tuning(ctypes.Structure):
    _fields_ = [("chunk", ctypes.c_int32), ("big_item", ctypes.c_int32)]


def get_tuning(device: int = 0) -> Tuple[int, int]:
    t = _Tuning()
    _lib.call("rubix_cube_tuning_get", int(device), ctypes.addressof(t))
    return int(t.chunk), int(t.big_item)


def set_tuning(device: int = 0, chunk: Optional[int] = None, big_item: int = 64) -> None:
    """Set (or, with chunk=None, reset to the defaults) the device's tuning."""
    if chunk is None:
        _lib.call("rubix_cube_tuning_set", int(device), None)
        return
    t = _Tuning(int(chunk), int(big_item))
    _lib.call("rubix_cube_tuning_set", int(device), ctypes.addressof(t))


def autotune(run: Callable[[], object], key: Hashable, device: int = 0,
             candidates: Iterable[Tuple[int, int]] = CANDIDATES, repeats: int = 3) -> dict:
    """Time ``run()`` under each candidate (chunk, big_item), keep the fastest on
    ``device`` and cache it under ``key``.  Returns {"best", "times_ms", "cached"}."""
    with _lock:
        if key in _cache:
            best = _cache[key]
            set_tuning(device, *best)
            return {"best": best, "times_ms": {}, "cached": True}
    times = {}
    with torch.cuda.device(device):
        for cand in candidates:
            set_tuning(device, *cand)
            run()  # warm-up (workspace sizes follow the tuning)
            torch.cuda.synchronize()
            best_ms = float("inf")
            for _ in range(repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                run()
                e1.record()
                torch.cuda.synchronize()
                best_ms = min(best_ms, e0.elapsed_time(e1))
            times[cand] = best_ms
    best = min(times, key=times.get)
    set_tuning(device, *best)
    with _lock:
        _cache[key] = best
    return {"best": best, "times_ms": times, "cached": False}
