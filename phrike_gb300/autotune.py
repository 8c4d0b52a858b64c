"""Tile autotuning by measurement.

* The strided passes of 2D Fourier plans (the y pass of the right-hand side,
  the filter and the operators) process ``tile_cols`` adjacent columns per
  CTA: 4, 8 or 16 (at most the plan's cap).  Wider tiles make longer TMA rows
  and fewer, larger CTAs; narrower ones more CTAs for small grids and
  batches.
* The tcgen05 contractions of LGL plans at split-BF16x3 compute 128 x NT
  output tiles, NT = 64, 128, 176 or 256 (``umma_n_tile``), with a TMA ring
  of 2-3 stages in 100-210 KB of shared memory: wider tiles re-read the D
  matrix less, narrower ones keep more stages of smaller loads in flight.

The arithmetic of every output value is the same for every choice, so it
changes speed only.  The tuners build the plan at each allowed value, time a
few device steps of the caller's state with CUDA events and keep the
fastest; results are cached per (shape, lengths, batch, plan options).
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence, Tuple

import torch

from .engine import Plan

_CACHE: Dict[Tuple, Tuple[int, Dict[int, float]]] = {}


def _tune(option: str, shape, lengths, U, nsolve, dt, steps, candidates, plan_kw):
    key = (option, tuple(int(n) for n in shape), tuple(float(x) for x in lengths), int(nsolve),
           tuple(sorted((k, repr(v)) for k, v in plan_kw.items())))
    if key in _CACHE:
        return _CACHE[key]
    times: Dict[int, float] = {}
    for T in candidates:
        try:
            plan = Plan(shape, lengths, nsolve=nsolve, **{option: T}, **plan_kw)
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
        raise RuntimeError(f"no {option} value was accepted")
    best = min(times, key=lambda T: (times[T], -T))
    _CACHE[key] = (best, times)
    return best, times


def tune_umma_n_tile(shape: Sequence[int], lengths: Sequence[float], U: torch.Tensor, nsolve: int = 1,
                     dt: float = 1e-5, steps: int = 4, candidates: Sequence[int] = (64, 128, 176, 256),
                     **plan_kw) -> Tuple[int, Dict[int, float]]:
    """Fastest N tile of the tcgen05 contractions for an LGL x LGL plan at
    split-BF16x3 and the measured milliseconds per step of every tile."""
    if len(shape) != 2:
        raise ValueError("the tensor-core contractions belong to 2D LGL plans")
    kw = dict(plan_kw, basis="legendre", gemm_precision="bf16x3")
    return _tune("umma_n_tile", shape, lengths, U, nsolve, dt, steps, candidates, kw)


def tune_tile_cols(shape: Sequence[int], lengths: Sequence[float], U: torch.Tensor, nsolve: int = 1,
                   dt: float = 1e-4, steps: int = 4, candidates: Sequence[int] = (4, 8, 16),
                   **plan_kw) -> Tuple[int, Dict[int, float]]:
    """Fastest ``tile_cols`` for this plan configuration and the measured
    milliseconds per step of every allowed width.  ``U`` (nsolve states on
    the plan's device) is only read: each candidate steps a copy."""
    if len(shape) != 2:
        raise ValueError("tile widths apply to 2D Fourier plans")
    return _tune("tile_cols", shape, lengths, U, nsolve, dt, steps, candidates, plan_kw)
