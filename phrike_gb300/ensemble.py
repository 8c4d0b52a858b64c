"""Ensembles of independent solves of uneven sizes on one GPU.

Solves are grouped by grid; each group is one batched plan (all its states in
one device tensor) advanced on its own CUDA stream with the device-side CFL
time loop (ps_run_cfl).  A chunk of K steps per group is captured once in a
CUDA graph and replayed until every solve of the group has reached its end
time, so the host issues one graph launch per K steps and reads the group's
times once per chunk.  Groups run concurrently, which fills the GPU when
the small grids alone cannot.

The reference advances independent solves one at a time, each with its own
Python run loop (phrike/solver.py:338-422, 706-812); the result of every
solve here is the same as running it alone (same kernels and arithmetic per
solve; see tests/test_gpu_batch.py).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from .engine import Plan


@dataclass
class SolveSpec:
    """One solve: spatial shape (array order), lengths, initial state, end time."""

    shape: Tuple[int, ...]
    lengths: Tuple[float, ...]
    U0: np.ndarray
    t_end: float
    t0: float = 0.0


@dataclass
class _Group:
    shape: Tuple[int, ...]
    lengths: Tuple[float, ...]
    index: List[int]
    plan: Plan
    U: torch.Tensor
    t: torch.Tensor
    tend: torch.Tensor
    stream: torch.cuda.Stream
    graph: Optional[torch.cuda.CUDAGraph] = None
    done: bool = False
    chunks: int = 0


class Ensemble:
    """Batched CFL-driven ensemble.  ``gamma``, ``cfl``, dealiasing and the
    filter are shared by all solves; grids may differ."""

    def __init__(self, specs: Sequence[SolveSpec], gamma: float = 1.4, cfl: float = 0.4, dealias: bool = True,
                 filter_params: Optional[Dict] = None, device: Optional[torch.device] = None,
                 autotune: bool = False):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.specs = list(specs)
        groups: Dict[Tuple, List[int]] = {}
        for i, s in enumerate(self.specs):
            groups.setdefault((tuple(s.shape), tuple(float(x) for x in s.lengths)), []).append(i)
        self.groups: List[_Group] = []
        self.tile_cols: Dict[Tuple, int] = {}
        t_tune = time.perf_counter()
        for (shape, lengths), idx in groups.items():
            U = torch.as_tensor(np.stack([self.specs[i].U0 for i in idx]), dtype=torch.float32,
                                device=self.device).contiguous()
            kw = dict(gamma=gamma, dealias=dealias, filter_params=filter_params, cfl=cfl, device=self.device)
            tc = None
            if autotune and len(shape) == 2:  # measured strided-pass tile width (autotune.py)
                from .autotune import tune_tile_cols
                tc, _ = tune_tile_cols(shape, lengths, U, nsolve=len(idx), **kw)
                self.tile_cols[(tuple(shape), tuple(lengths))] = tc
            plan = Plan(shape, lengths, nsolve=len(idx), tile_cols=tc, **kw)
            t = torch.as_tensor([self.specs[i].t0 for i in idx], dtype=torch.float64, device=self.device)
            te = torch.as_tensor([self.specs[i].t_end for i in idx], dtype=torch.float64, device=self.device)
            self.groups.append(_Group(shape, lengths, idx, plan, U, t, te, torch.cuda.Stream(self.device)))
        self.tune_seconds = time.perf_counter() - t_tune

    @property
    def cells(self) -> int:
        return sum(int(np.prod(s.shape)) for s in self.specs)

    def _capture(self, g: _Group, chunk: int) -> None:
        # warm the chunk once outside the capture (lazy module loads, map encoding)
        g.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g.graph, stream=g.stream):
            g.plan.run_cfl_(g.U, chunk, g.t, g.tend)

    def run(self, chunk: int = 50, use_graphs: bool = True, max_chunks: int = 1_000_000) -> Dict[str, float]:
        """Advance every solve to its end time; returns timing statistics."""
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        capture_s = 0.0
        if use_graphs:
            for g in self.groups:
                with torch.cuda.stream(g.stream):
                    g.plan.run_cfl_(g.U, 1, g.t, g.tend)  # first step outside capture (also warms up)
            for g in self.groups:
                g.stream.synchronize()
            # capture is one-time host work with the GPU idle: its wall time is
            # reported apart and left out of the solve time
            tc = time.perf_counter()
            for g in self.groups:
                self._capture(g, chunk)
            capture_s = time.perf_counter() - tc
        for _ in range(max_chunks):
            live = [g for g in self.groups if not g.done]
            if not live:
                break
            for g in live:
                with torch.cuda.stream(g.stream):
                    if use_graphs:
                        g.graph.replay()
                    else:
                        g.plan.run_cfl_(g.U, chunk, g.t, g.tend)
                g.chunks += 1
            for g in live:
                g.stream.synchronize()
                if bool(torch.all(g.t >= g.tend - 1e-12).item()):
                    g.done = True
        torch.cuda.synchronize(self.device)
        elapsed = time.perf_counter() - t0 - capture_s
        cell_steps = 0
        for g in self.groups:
            cells = int(np.prod(g.shape))
            cell_steps += cells * sum(g.plan.steps_done())
        return {"seconds": elapsed, "capture_seconds": capture_s, "solves": len(self.specs),
                "solves_per_s": len(self.specs) / elapsed,
                "cell_updates": cell_steps, "cell_updates_per_s": cell_steps / elapsed,
                "status": max(g.plan.status() for g in self.groups)}

    def state(self, i: int) -> torch.Tensor:
        """Current state of solve i (a view into its group's tensor)."""
        for g in self.groups:
            if i in g.index:
                return g.U[g.index.index(i)]
        raise IndexError(i)

    def time(self, i: int) -> float:
        for g in self.groups:
            if i in g.index:
                return float(g.t[g.index.index(i)].item())
        raise IndexError(i)
