"""Tile autotuning by measurement.

The strided passes of 2D Fourier plans (the y pass of the right-hand side,
the filter and the operators) process ``tile_cols`` adjacent columns per CTA:
4, 8 or 16 (at most the plan's cap).  Wider tiles make longer TMA rows and
fewer, larger CTAs; narrower ones more CTAs for small grids and batches.  The
arithmetic of each pencil is the same for every width, so the choice changes
speed only.  ``tune_tile_cols`` builds the plan at each allowed width, times a
few device steps of the caller's state with CUDA events and keeps the
fastest; results are cached per (shape, lengths, batch, plan options).
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence, Tuple

import torch

from .engine import Plan

_CACHE: Dict[Tuple, Tuple[int, Dict[int, float]]] = {}


def tune_tile_cols(shape: Sequence[int], lengths: Sequence[float], U: torch.Tensor, nsolve: int = 1,
                   dt: float = 1e-4, steps: int = 4, candidates: Sequence[int] = (4, 8, 16),
                   **plan_kw) -> Tuple[int, Dict[int, float]]:
    """Fastest ``tile_cols`` for this plan configuration and the measured
    milliseconds per step of every allowed width.  ``U`` (nsolve states on
    the plan's device) is only read: each candidate steps a copy."""
    key = (tuple(int(n) for n in shape), tuple(float(x) for x in lengths), int(nsolve),
           tuple(sorted((k, repr(v)) for k, v in plan_kw.items())))
    if key in _CACHE:
        return _CACHE[key]
    if len(shape) != 2:
        raise ValueError("tile widths apply to 2D Fourier plans")
    times: Dict[int, float] = {}
    for T in candidates:
        try:
            plan = Plan(shape, lengths, nsolve=nsolve, tile_cols=T, **plan_kw)
        except RuntimeError:
            continue  # not allowed for this grid
        V = U.clone()
        plan.run_(V, 1, dt)  # warm-up (kernel attributes, lazy loading)
        stream = torch.cuda.current_stream(plan.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.run_(V, steps, dt)
        e1.record(stream)
        e1.synchronize()
        times[T] = e0.elapsed_time(e1) / steps
        plan.close()
    if not times:
        raise RuntimeError("no tile width was accepted")
    best = min(times, key=lambda T: (times[T], -T))
    _CACHE[key] = (best, times)
    return best, times
