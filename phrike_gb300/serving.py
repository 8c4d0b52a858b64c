"""Serving loop: continuous batching of independent solve requests on one GPU.

A request is one solve (problem family, grid, initial state, end time).
Requests are grouped by (family, grid); each group is one batched plan of C
slots (phrike_gb300.engine.Plan with nsolve = C) whose states stay resident
in HBM, advanced on the group's own CUDA stream by the device-side CFL loop
(ps_run_cfl) in chunks of K steps captured once in a CUDA graph.  A slot is
free when its time has reached its end time: the CFL kernels skip it, so the
captured chunk needs no change when slots are filled or freed.

The loop, on one host thread:
  * arrivals (their own clock) join a pending list;
  * admission: a pending request takes a free slot of its group, or a new
    group is created when the HBM budget allows it; its initial state is
    copied into the slot with t = 0 and its t_end (on the group stream, so
    it lands between two chunks);
  * every group with live slots and no chunk in flight launches a chunk;
    groups overlap on the device;
  * a group whose chunk has completed reads its slot times; finished slots
    are copied out and freed (retirement), and the request's latency is
    completion - arrival.

Each result equals the same solve run alone (same kernels and arithmetic per
slot; tests/test_gpu_serving.py), with two conditions the families here meet:
the filter cadence is 1 (the plan-wide step counter sets the cadence), and
MHD initial states are projected by a single-solve plan before admission
(the reference's run() projects U0, solver.py:1117-1118).

The reference has no serving layer: it runs one solve per process through
BaseProblem.run (phrike/problems/base.py:1024-1181).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import problems
from .engine import Plan

TWO_PI = 2.0 * math.pi

# family -> plan options (gamma, lengths in array order, CFL, filter, equations, basis)
FAMILIES: Dict[str, dict] = {
    "sod1d": dict(ndim=1, gamma=1.4, cfl=0.4, filter={"enabled": True, "p": 8, "alpha": 36.0}),
    "khi2d": dict(ndim=2, gamma=1.4, cfl=0.4, filter=None),
    "ot2d": dict(ndim=2, gamma=5.0 / 3.0, cfl=0.3, filter={"enabled": True, "p": 8, "alpha": 36.0},
                 equations="mhd"),
    "tgv3d": dict(ndim=3, gamma=1.4, cfl=0.25, filter=None),
    "lgl2d": dict(ndim=2, gamma=1.4, cfl=0.3, filter=None, basis="legendre", gemm_precision="bf16x3"),
    "lgl1d": dict(ndim=1, gamma=1.4, cfl=0.3, filter=None, basis="legendre", gemm_precision="fp32"),
}


def family_lengths(family: str, n: int) -> Tuple[float, ...]:
    if family == "sod1d":
        return (1.0,)
    if family == "khi2d":
        return (1.0, 1.0)
    if family == "ot2d":
        return (TWO_PI, TWO_PI)
    if family == "tgv3d":
        return (TWO_PI,) * 3
    return (2.0, 2.0)


def family_shape(family: str, n: int) -> Tuple[int, ...]:
    nd = FAMILIES[family]["ndim"]
    return (n,) * nd


@dataclass
class Request:
    """One solve: family, grid size n (points per axis), end time, arrival
    time (seconds from the start of the stream) and its initial state."""

    rid: int
    family: str
    n: int
    t_end: float
    arrival: float = 0.0
    params: Dict = field(default_factory=dict)
    U0: Optional[np.ndarray] = None
    t0: float = 0.0  # start time (a resumed snapshot starts at its own time)

    @staticmethod
    def resume(rid: int, snap, arrival: float = 0.0) -> "Request":
        """A request that continues a paused solve (phrike_gb300.io.Snapshot)."""
        return Request(rid, snap.family, snap.n, snap.t_end, arrival, dict(snap.params), np.asarray(snap.U), snap.t)

    @property
    def shape(self) -> Tuple[int, ...]:
        return family_shape(self.family, self.n)

    def initial_state(self) -> np.ndarray:
        if self.U0 is not None:
            return self.U0
        f, n, p = self.family, self.n, self.params
        if f == "sod1d":
            U = problems.sod_smoothed(n)
        elif f == "khi2d":
            U = problems.kelvin_helmholtz_2d(n, n, U0=p.get("U0", 1.0), A=p.get("A", 0.01))
        elif f == "ot2d":
            U = problems.orszag_tang_2d(n, n, gamma=FAMILIES[f]["gamma"], B0=p.get("B0", 1.0))
        elif f == "tgv3d":
            U = problems.taylor_green_3d(n, n, n)
        elif f == "lgl2d":
            from .engine import lgl_build
            x = (lgl_build(n, 2.0)[0] - 1.0).cpu().numpy()
            U = problems.acoustic_pulse_lgl_2d(x, x, amp=p.get("amp", 0.01), width2=p.get("width2", 0.01))
        elif f == "lgl1d":
            from .engine import lgl_build
            x = (lgl_build(n, 2.0)[0] - 1.0).cpu().numpy()
            U = problems.acoustic_pulse_lgl_1d(x, amp=p.get("amp", 0.01), width2=p.get("width2", 0.01))
        else:
            raise ValueError(f"unknown family {f!r}")
        self.U0 = U
        return U


def _plan_kw(family: str, device) -> dict:
    o = FAMILIES[family]
    return dict(gamma=o["gamma"], cfl=o["cfl"], filter_params=o["filter"], device=device,
                basis=o.get("basis", "fourier"), gemm_precision=o.get("gemm_precision", "fp32"),
                equations=o.get("equations", "euler"))


def make_plan(family: str, n: int, nsolve: int, device, tile_cols: Optional[int] = None,
              umma_n_tile: Optional[int] = None) -> Plan:
    return Plan(family_shape(family, n), family_lengths(family, n), nsolve=nsolve, tile_cols=tile_cols,
                umma_n_tile=umma_n_tile, **_plan_kw(family, device))


def _prepare_state(req: Request, device, projector: Optional[Plan]) -> torch.Tensor:
    U = torch.as_tensor(req.initial_state(), dtype=torch.float32, device=device).contiguous()
    if req.family == "ot2d" and projector is not None:
        projector.project_state_(U)
    return U


def run_alone(req: Request, device, chunk: int = 20) -> Tuple[torch.Tensor, float]:
    """The plain form: one solve on its own plan, the device CFL loop in
    chunks until t >= t_end (host checks t between chunks).  Returns the final
    state and the wall time of the loop."""
    plan = make_plan(req.family, req.n, 1, device)
    proj = plan if req.family == "ot2d" else None
    U = _prepare_state(req, device, proj)
    t = torch.full((1,), float(req.t0), dtype=torch.float64, device=device)
    te = torch.full((1,), float(req.t_end), dtype=torch.float64, device=device)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    while float(t.item()) < req.t_end - 1e-12:
        plan.run_cfl_(U, chunk, t, te)
    torch.cuda.synchronize(device)
    return U, time.perf_counter() - t0


@dataclass
class _Group:
    family: str
    n: int
    plan: Plan
    U: torch.Tensor
    t: torch.Tensor
    tend: torch.Tensor
    stream: torch.cuda.Stream
    slots: List[Optional[Request]]
    bytes: int
    graph: Optional[torch.cuda.CUDAGraph] = None
    event: Optional[torch.cuda.Event] = None
    in_flight: bool = False
    chunks: int = 0

    @property
    def live(self) -> int:
        return sum(1 for r in self.slots if r is not None)


def _benign_state(family: str, shape, gamma: float) -> np.ndarray:
    """A uniform state at rest for free slots (finite primitives)."""
    nc = 8 if family == "ot2d" else len(shape) + 2
    U = np.zeros((nc,) + tuple(shape))
    U[0] = 1.0
    U[4 if family == "ot2d" else nc - 1] = 1.0 / (gamma - 1.0)
    return U


class Server:
    """Continuous-batching solve server for one GPU.

    ``budget_bytes``: HBM the groups may hold (plan scratch + states); default
    half of the free device memory.  ``slots``: callable (family, n) -> slots
    per group.  ``chunk``: CFL steps per captured chunk.  ``cost``: callable
    (family, n) -> seconds per unit of simulated time of one solve alone;
    groups costing at least ``priority_seconds`` get a high-priority stream.
    """

    def __init__(self, device=None, budget_bytes: Optional[int] = None, chunk: int = 20, slots=None,
                 use_graphs: bool = True, cost=None, priority_seconds: float = 5.0, autotune: bool = False):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget_bytes = free // 2
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.slots_for = slots or self._default_slots
        self.use_graphs = use_graphs
        # cost(family, n) -> seconds of one solve alone per unit of simulated
        # time (e.g. measured by run_alone); groups at or above priority_seconds
        # run on a high-priority stream, so that the long solves that set the
        # stream's makespan are slowed least by the short ones around them
        self.cost = cost
        self.priority_seconds = float(priority_seconds)
        self.autotune = autotune  # measured strided-pass tile width for 2D Fourier groups (autotune.py)
        self.groups: List[_Group] = []
        self.used = 0
        self.projectors: Dict[int, Plan] = {}
        self.results: Dict[int, np.ndarray] = {}
        self.paused: Dict[int, object] = {}
        self.pause_at: Dict[int, float] = {}
        self.completion: Dict[int, float] = {}
        self.admitted_at: Dict[int, float] = {}
        self.max_live = 0
        # initial states are prepared (and MHD ones projected by the shared
        # single-solve projector plans) on one admission stream
        self.admit_stream = torch.cuda.Stream(self.device)

    @staticmethod
    def _default_slots(family: str, n: int) -> int:
        cells = n ** FAMILIES[family]["ndim"]
        if cells <= 128 * 128:
            return 16
        if cells <= 256 * 256:
            return 8
        if cells <= 512 * 512:
            return 4
        return 2

    def _group_bytes(self, family: str, n: int, slots: int) -> int:
        plan_bytes = make_plan_bytes(family, n, slots)
        nc = 8 if family == "ot2d" else FAMILIES[family]["ndim"] + 2
        return plan_bytes + 4 * nc * slots * n ** FAMILIES[family]["ndim"] + 16 * slots

    def _new_group(self, family: str, n: int) -> Optional[_Group]:
        slots = self.slots_for(family, n)
        need = self._group_bytes(family, n, slots)
        if self.used + need > self.budget:
            return None
        shape = family_shape(family, n)
        ben = _benign_state(family, shape, FAMILIES[family]["gamma"])
        U = torch.as_tensor(np.stack([ben] * slots), dtype=torch.float32, device=self.device).contiguous()
        tc = nt = None
        if self.autotune and len(shape) == 2 and FAMILIES[family].get("basis", "fourier") == "fourier":
            from .autotune import tune_tile_cols
            tc, _ = tune_tile_cols(shape, family_lengths(family, n), U, nsolve=slots,
                                   **_plan_kw(family, self.device))
        if self.autotune and len(shape) == 2 and FAMILIES[family].get("gemm_precision") == "bf16x3":
            from .autotune import tune_umma_n_tile
            kw = {k: v for k, v in _plan_kw(family, self.device).items() if k not in ("basis", "gemm_precision")}
            nt, _ = tune_umma_n_tile(shape, family_lengths(family, n), U, nsolve=slots, **kw)
        plan = make_plan(family, n, slots, self.device, tile_cols=tc, umma_n_tile=nt)
        t = torch.zeros(slots, dtype=torch.float64, device=self.device)
        te = torch.zeros(slots, dtype=torch.float64, device=self.device)  # t >= t_end: free
        high = self.cost is not None and float(self.cost(family, n)) >= self.priority_seconds
        stream = torch.cuda.Stream(self.device, priority=-1) if high else torch.cuda.Stream(self.device)
        g = _Group(family, n, plan, U, t, te, stream, [None] * slots, need)
        if self.use_graphs:
            # warm up (kernel attributes, module loading) and capture the chunk
            # while every slot is free, so that a slot's chunk boundaries fall
            # on the same steps as in a run alone (each call re-bases the
            # energy-perturbation reference)
            with torch.cuda.stream(g.stream):
                g.plan.run_cfl_(g.U, 1, g.t, g.tend)
            g.stream.synchronize()
            g.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g.graph, stream=g.stream):
                g.plan.run_cfl_(g.U, self.chunk, g.t, g.tend)
        self.groups.append(g)
        self.used += need
        return g

    def _projector(self, n: int) -> Plan:
        if n not in self.projectors:
            self.projectors[n] = make_plan("ot2d", n, 1, self.device)
        return self.projectors[n]

    def _admit(self, req: Request, now: float) -> bool:
        g = None
        for cand in self.groups:
            if cand.family == req.family and cand.n == req.n and cand.live < len(cand.slots):
                g = cand
                break
        if g is None:
            g = self._new_group(req.family, req.n)
            if g is None:
                return False
        k = g.slots.index(None)
        proj = self._projector(req.n) if req.family == "ot2d" else None
        with torch.cuda.stream(self.admit_stream):
            U0 = _prepare_state(req, self.device, proj)
            ready = torch.cuda.Event()
            ready.record(self.admit_stream)
        # the slot is written on the group stream, between two chunks
        g.stream.wait_event(ready)
        U0.record_stream(g.stream)
        with torch.cuda.stream(g.stream):
            g.U[k].copy_(U0, non_blocking=True)
            g.t[k] = float(req.t0)
            g.tend[k] = float(req.t_end)
        g.slots[k] = req
        self.admitted_at[req.rid] = now
        return True

    def _launch(self, g: _Group) -> None:
        with torch.cuda.stream(g.stream):
            if self.use_graphs:
                g.graph.replay()
            else:
                g.plan.run_cfl_(g.U, self.chunk, g.t, g.tend)
            g.event = torch.cuda.Event()
            g.event.record(g.stream)
        g.in_flight = True
        g.chunks += 1

    def _retire(self, g: _Group, now: float) -> int:
        # read on the group stream: after the chunk and any admission writes
        with torch.cuda.stream(g.stream):
            t = g.t.cpu().numpy()
            te = g.tend.cpu().numpy()
            done = 0
            for k, req in enumerate(g.slots):
                if req is not None and t[k] >= te[k] - 1e-12:
                    self.results[req.rid] = g.U[k].cpu().numpy()
                    self.completion[req.rid] = now
                    g.slots[k] = None
                    done += 1
                elif req is not None and req.rid in self.pause_at and t[k] >= self.pause_at[req.rid]:
                    self.paused[req.rid] = self.preempt(req.rid)  # between two chunks
                    self.completion[req.rid] = now
                    done += 1
        return done

    def _find(self, rid: int):
        for g in self.groups:
            for k, req in enumerate(g.slots):
                if req is not None and req.rid == rid:
                    return g, k
        raise KeyError(f"request {rid} is not resident")

    def snapshot(self, rid: int):
        """Copy a resident solve out between two chunks (a Snapshot with its
        current time); the solve keeps running."""
        from .io import Snapshot
        g, k = self._find(rid)
        with torch.cuda.stream(g.stream):
            U = g.U[k].cpu().numpy()
            t = float(g.t[k].item())
        req = g.slots[k]
        return Snapshot(req.family, req.n, t, float(req.t_end), U, dict(req.params))

    def preempt(self, rid: int):
        """Pause a resident solve: snapshot it and free its slot.  Resume it
        later with serve([Request.resume(rid, snapshot)])."""
        g, k = self._find(rid)
        snap = self.snapshot(rid)
        with torch.cuda.stream(g.stream):
            g.tend[k] = g.t[k]  # a free slot: t >= t_end, the captured chunk skips it
        g.slots[k] = None
        self.admitted_at.pop(rid, None)
        return snap

    def serve(self, requests: List[Request], realtime: bool = True, max_seconds: float = 3600.0,
              pause_at: Optional[Dict[int, float]] = None) -> Dict:
        """Serve a request stream; arrival times are honoured on the host
        clock (``realtime``) or all requests arrive at once.  ``pause_at``
        (request id -> time) pauses a solve at the first chunk boundary at or
        after that time: its Snapshot goes to ``self.paused`` and its slot is
        freed; serve(..) with Request.resume(rid, snapshot) continues it."""
        self.pause_at = dict(pause_at or {})
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending: List[Request] = []
        nxt, finished = 0, 0
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while finished < len(reqs):
            now = time.perf_counter() - t0
            if now > max_seconds:
                raise RuntimeError(f"serving did not finish within {max_seconds} s")
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= now):
                pending.append(reqs[nxt])
                nxt += 1
            progressed = False
            for r in list(pending):  # FIFO per group; other families pass a blocked head
                if self._admit(r, now):
                    pending.remove(r)
                    progressed = True
            live = sum(g.live for g in self.groups)
            self.max_live = max(self.max_live, live)
            for g in self.groups:
                if g.in_flight and g.event.query():
                    g.in_flight = False
                    finished += self._retire(g, time.perf_counter() - t0)
                    progressed = True
                if not g.in_flight and g.live > 0:
                    self._launch(g)
                    progressed = True
            if not progressed:
                time.sleep(0.0002)
        torch.cuda.synchronize(self.device)
        elapsed = time.perf_counter() - t0
        lat = np.array([self.completion[r.rid] - (r.arrival if realtime else 0.0) for r in reqs])
        return {"seconds": elapsed, "requests": len(reqs), "solves_per_s": len(reqs) / elapsed,
                "latency_p50": float(np.percentile(lat, 50)), "latency_p95": float(np.percentile(lat, 95)),
                "latency_p99": float(np.percentile(lat, 99)), "max_live_slots": self.max_live,
                "groups": len(self.groups), "hbm_bytes": self.used, "status": max(
                    [g.plan.status() for g in self.groups] + [0])}


def make_plan_bytes(family: str, n: int, slots: int) -> int:
    """Device bytes a group's plan allocates (ps_batch_scratch_bytes)."""
    import ctypes as C
    from . import _lib
    o = FAMILIES[family]
    lib = _lib.load()
    desc = _lib.PlanDesc()
    nd = o["ndim"]
    _lib.check(lib.ps_plan_desc_init(C.byref(desc), nd))
    for a in range(nd):
        desc.n[a] = n
        desc.length[a] = list(reversed(family_lengths(family, n)))[a]
        if o.get("basis") == "legendre":
            desc.basis[a] = _lib.PS_BASIS_LEGENDRE
    if o.get("equations") == "mhd":
        desc.equations = _lib.PS_EQ_MHD
    if o.get("gemm_precision"):
        desc.gemm_precision = _lib.GEMM_PRECISIONS[o["gemm_precision"]]
    desc.filter_enabled = 1 if (o["filter"] or {}).get("enabled") else 0
    b = C.c_size_t()
    _lib.check(lib.ps_batch_scratch_bytes(C.byref(desc), slots, C.byref(b)))
    return int(b.value)


def request_stream(count: int, rate: float = 200.0, seed: int = 20261203,
                   t_end_range: Tuple[float, float] = (0.1, 1.0), families: Optional[Dict[str, List[int]]] = None
                   ) -> List[Request]:
    """Seeded Poisson stream mixing the six families with uniform size draws
    and t_end ~ U[t_end_range]."""
    fam = families or {"sod1d": [256, 512, 1024, 2048, 4096], "khi2d": [128, 256, 512, 1024], "ot2d": [128, 256, 512],
                       "tgv3d": [32, 64, 128], "lgl2d": [65, 129, 257, 513], "lgl1d": [65, 129, 257, 513]}
    names = sorted(fam)
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        f = names[int(rng.integers(len(names)))]
        n = int(rng.choice(fam[f]))
        params = {}
        if f == "khi2d":
            params = {"U0": float(rng.uniform(0.5, 1.5)), "A": float(rng.uniform(0.005, 0.02))}
        te = float(rng.uniform(*t_end_range))
        out.append(Request(i, f, n, te, t, params))
    return out
