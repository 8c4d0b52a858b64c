"""Solvers with the reference's interface (backend "gb300").

Mirrors SpectralSolver1D/2D/3D of phrike/solver.py (lines 135-422, 527-812,
1237-1513): same constructor arguments, compute_dt / step / run methods, the
same history keys and the same CFL run loop.  A fixed step (scheme "rk4" or
the midpoint "rk2") is one call into the C ABI (ps_step_rk4), which runs the
fused pass kernels including the clamp and the filter cadence; the plan's
step counter plays the role of the reference's _step_counter.  With an
adaptive_config (rk23 / rk45 / rk78) run() drives the device-side embedded
RK loop (ps_run_adaptive).  step() is functional like the reference: it
returns a new tensor and leaves its argument untouched.
"""
from __future__ import annotations

import math
from typing import Any, Callable, Dict, List, Optional

import torch

from .engine import Plan


class _SpectralSolverBase:
    _ndim = 1
    _history_keys: List[str] = []
    _equations = "euler"

    def __init__(self, grid, equations, U0: Optional[Any] = None, scheme: str = "rk4", cfl: float = 0.4,
                 adaptive_config: Optional[Dict] = None, artificial_viscosity_config: Optional[Dict] = None,
                 gravity_config: Optional[Dict] = None):
        # adaptive_config (solver.py:178-204): rk23 / rk45 / rk78 run the
        # device-side embedded-RK loop; another scheme falls back to fixed steps
        adaptive = None
        if adaptive_config and adaptive_config.get("enabled", False):
            method = str(adaptive_config.get("scheme", "rk45")).lower()
            if method in ("rk23", "rk45", "rk78"):
                adaptive = dict(adaptive_config, scheme=method)
                scheme = method
            else:
                scheme = adaptive_config.get("fallback_scheme", "rk4")
        # fixed steps: "rk2" is the midpoint rule and every other name is RK4,
        # as the reference's _fixed_step dispatch (solver.py:259-265, 639-645, 990-996, 1330-1337)
        if adaptive is not None and getattr(grid, "_basis", "fourier") != "fourier":
            raise NotImplementedError("backend 'gb300': adaptive stepping on LGL grids is not implemented")
        av = None
        if artificial_viscosity_config and artificial_viscosity_config.get("enabled", False):
            if self._ndim == 3:
                artificial_viscosity_config = None  # the reference's 3D solver ignores it (solver.py:1266, 1330-1337)
            else:
                av = dict(artificial_viscosity_config)
        gravity = None
        if gravity_config and gravity_config.get("enabled", False):
            # (gx[, gy[, gz]]) along x, y, z (solver.py:82-91, 453-464, 1193-1206)
            gravity = [float(gravity_config.get(k, 0.0)) for k in ("gx", "gy", "gz")[: self._ndim]]
        self.grid = grid
        self.equations = equations
        self.scheme = str(scheme).lower()
        self.cfl = float(cfl)
        self.t = 0.0
        self.U = U0
        self.adaptive_enabled = adaptive is not None
        self.adaptive_config = adaptive
        self.gravity_config = gravity_config
        fp = dict(getattr(grid, "filter_params", None) or {})
        interval = fp.get("interval", None)
        # 1D: cadence 5 by default when artificial viscosity is on (solver.py:220-232)
        default_interval = 5 if (av is not None and self._ndim == 1) else 1
        self.filter_interval = max(1, int(interval)) if interval is not None else default_interval
        self.artificial_viscosity = av
        fp["interval"] = self.filter_interval
        self.plan = Plan(grid._shape, grid._lengths, gamma=float(equations.gamma), dealias=grid.dealias,
                         filter_params=fp, cfl=self.cfl, gravity=gravity, device=grid.device,
                         basis=getattr(grid, "_basis", "fourier"),
                         gemm_precision=getattr(grid, "gemm_precision", "fp32"), equations=self._equations,
                         mhd_config=getattr(grid, "mhd_config", None), av_config=av,
                         scheme="rk2" if self.scheme == "rk2" else "rk4",
                         lgl_bc1d=getattr(grid, "_bc_codes", None))
        self._ark = Plan.adaptive_desc(adaptive) if adaptive is not None else None

    # -- reference interface -----------------------------------------------
    def _spacing(self) -> float:
        raise NotImplementedError

    def compute_dt(self, U: Any) -> float:
        s = float(self.plan.max_wave_speed(self.grid.to_device(U)).item())
        if s <= 0.0:
            return 1e-6
        return self.cfl * self._spacing() / s

    def step(self, U: Any, dt: float) -> torch.Tensor:
        """One step of size dt; with adaptive_config one embedded-RK attempt
        (_adaptive_step: the filtered U_high when accepted, else U).  The
        reference's 2D/3D _adaptive_step passes an extra argument and raises
        (solver.py:662, 1351); here every dimension takes the 1D behaviour."""
        V = self.grid.to_device(U).clone()
        if self.adaptive_enabled:
            f64 = dict(dtype=torch.float64, device=self.plan.device)
            t = torch.zeros((1,), **f64)
            h = torch.full((1,), float(dt), **f64)
            self.plan.run_adaptive_(V, 1, self._ark, t, h.clone(), h)
            return V
        self.plan.step_(V, float(dt))
        return V

    def _record(self, history: Dict[str, List[float]]) -> None:
        cons = self.plan.conserved(self.U).tolist()
        history["time"].append(self.t)
        for key, v in zip(self._history_keys, cons):
            history[key].append(v)

    def run(self, U0: Any, t0: float, t_end: float, output_interval: float = 0.1,
            checkpoint_interval: float = 0.0, outdir: Optional[str] = None,
            on_output: Optional[Callable[[float, Any], None]] = None,
            on_step: Optional[Callable[[int, float, Any], None]] = None, tracers: Optional[Any] = None,
            dt: Optional[float] = None) -> Dict[str, List[float]]:
        """CFL-driven loop of the reference (solver.py:338-422); with ``dt``
        given, fixed steps of that size instead."""
        self.U = self.grid.to_device(U0).clone()
        self._tracers = tracers
        self.t = float(t0)
        next_output = self.t + output_interval
        # snapshots every checkpoint_interval into outdir (solver.py:357-361, 408-417)
        self._outdir = outdir
        self._next_ckpt = (self.t + checkpoint_interval
                           if outdir and checkpoint_interval and checkpoint_interval > 0 else float("inf"))
        self._ckpt_interval = checkpoint_interval
        history: Dict[str, List[float]] = {"time": [], **{k: [] for k in self._history_keys}}
        self._record(history)
        if on_output is not None:
            on_output(self.t, self.U)
        step_dt = float(dt) if dt is not None else self.compute_dt(self.U)
        if self.adaptive_enabled:
            return self._run_adaptive(history, step_dt, t_end, output_interval, next_output, on_output, on_step)
        step_count = 0
        while self.t < t_end - 1e-12:
            h = min(step_dt, t_end - self.t)
            self.plan.step_(self.U, h)
            self.t += h
            if on_step is not None:
                on_step(step_count, h, self.U)
            if tracers is not None:  # after every step with its dt (solver.py:398-399)
                tracers.step(self.grid, self.equations, self.U, h)
            step_count += 1
            if dt is None:
                step_dt = self.compute_dt(self.U)
            if self.t + 1e-12 >= next_output:
                self._record(history)
                if on_output is not None:
                    on_output(self.t, self.U)
                next_output += output_interval
            self._checkpoint()
        self._record(history)
        if on_output is not None:
            on_output(self.t, self.U)
        return history


    def _checkpoint(self) -> None:
        if self._outdir and self.t + 1e-12 >= self._next_ckpt:
            from .io import save_solution_snapshot
            save_solution_snapshot(self._outdir, self.t, self.U, self.grid, self.equations,
                                   tracers=getattr(self, "_tracers", None))
            self._next_ckpt += self._ckpt_interval

    def _run_adaptive(self, history, dt0, t_end, output_interval, next_output, on_output, on_step,
                      chunk: int = 16) -> Dict[str, List[float]]:
        """The adaptive branch of the reference's run loop (solver.py:384-417
        with _adaptive_run_step): attempts run on the device and pause at
        the next output time, so outputs are recorded after the same attempts
        as in the reference.  With on_step every attempt is a separate call
        and on_step sees each accepted attempt (step_count counts attempts,
        rejected ones included).  Tracers, like on_step, take one attempt per
        call and move after every attempt with its attempted dt, rejected
        attempts included, as the reference's loop does (solver.py:384-399)."""
        dev = self.plan.device
        f64 = dict(dtype=torch.float64, device=dev)
        t = torch.full((1,), self.t, **f64)
        te = torch.full((1,), float(t_end), **f64)
        dtv = torch.full((1,), float(dt0), **f64)
        tout = torch.empty((1,), **f64)
        counts = torch.zeros((1, 2), dtype=torch.int32, device=dev)
        step_count = 0
        while self.t < t_end - 1e-12:
            # an output or a checkpoint is still due after this attempt
            behind = self.t + 1e-12 >= min(next_output, self._next_ckpt)
            tracers = getattr(self, "_tracers", None)
            if on_step is not None or tracers is not None or behind:
                dt_used = min(float(dtv.item()), t_end - self.t)
                before = counts[0, 0].item()
                self.plan.run_adaptive_(self.U, 1, self._ark, t, te, dtv, None, counts)
                self.t = float(t.item())
                if counts[0, 0].item() > before and on_step is not None:
                    on_step(step_count, dt_used, self.U)
                if tracers is not None:
                    tracers.step(self.grid, self.equations, self.U, dt_used)
                step_count += 1
            else:
                tout.fill_(min(next_output, self._next_ckpt))
                self.plan.run_adaptive_(self.U, chunk, self._ark, t, te, dtv, tout, counts)
                self.t = float(t.item())
                step_count = int(counts.sum().item())
            if self.t + 1e-12 >= next_output:
                self._record(history)
                if on_output is not None:
                    on_output(self.t, self.U)
                next_output += output_interval
            self._checkpoint()
        self._record(history)
        if on_output is not None:
            on_output(self.t, self.U)
        self.adaptive_counts = counts[0].tolist()
        return history


class SpectralSolver1D(_SpectralSolverBase):
    """phrike/solver.py:135-422; CFL dt = cfl * dx / max(|u| + a)."""

    _ndim = 1
    _history_keys = ["mass", "momentum", "energy"]

    def __init__(self, grid, equations, U0=None, scheme="rk4", cfl=0.4, adaptive_config=None,
                 artificial_viscosity_config=None, gravity_config=None):
        super().__init__(grid, equations, U0, scheme, cfl, adaptive_config, artificial_viscosity_config,
                         gravity_config)

    def _spacing(self) -> float:
        return self.grid.dx


class SpectralSolver2D(_SpectralSolverBase):
    """phrike/solver.py:527-812; CFL dt = cfl * min(dx, dy) / max(|u_x| + a)."""

    _ndim = 2
    _history_keys = ["mass", "momentum_x", "momentum_y", "energy"]

    def __init__(self, grid, equations, U0=None, scheme="rk4", cfl=0.3, adaptive_config=None,
                 artificial_viscosity_config=None, gravity_config=None):
        super().__init__(grid, equations, U0, scheme, cfl, adaptive_config, artificial_viscosity_config,
                         gravity_config)

    def _spacing(self) -> float:
        dx = getattr(self.grid, "dx_min", None) or self.grid.dx
        dy = getattr(self.grid, "dy_min", None) or self.grid.dy
        return min(dx, dy)


class SpectralSolver3D(_SpectralSolverBase):
    """phrike/solver.py:1237-1513; CFL dt = cfl * min(dx, dy, dz) / max(max_i |u_i| + a)."""

    _ndim = 3
    _history_keys = ["mass", "momentum_x", "momentum_y", "momentum_z", "energy"]

    def __init__(self, grid, equations, U0=None, scheme="rk4", cfl=0.25, adaptive_config=None,
                 artificial_viscosity_config=None, gravity_config=None):
        super().__init__(grid, equations, U0, scheme, cfl, adaptive_config, None, gravity_config)

    def _spacing(self) -> float:
        return min(self.grid.dx, self.grid.dy, self.grid.dz)


class SpectralSolverMHD2D(_SpectralSolverBase):
    """2D (2.5D) ideal MHD, RK4 (phrike/solver.py:840-1049, 1169-1170).

    Options come from ``grid.mhd_config`` like the reference (resistivity,
    viscosity, cfl_diff, project_each_substage, divergence_clean, rho_min,
    p_min).  Every RK stage is clamped and projected on the device; after a
    step, at the filter cadence, the spectral filter and the projection.
    Explicit resistivity / viscosity add eta lap(B) / nu lap(rho u) to the
    right-hand side (solver.py:942-954).  run() projects U0 first and records
    magnetic energy, cross helicity and max |div B| as well.
    CFL dt = cfl * min(dx, dy) / max(max(|ux|, |uy|) + sqrt(a^2 + b^2)),
    capped by cfl_diff / (max(eta, nu) k^2_max) with diffusion
    (solver.py:1018-1034).
    """

    _ndim = 2
    _equations = "mhd"
    _history_keys = ["mass", "momentum_x", "momentum_y", "momentum_z", "energy", "magnetic_energy",
                     "cross_helicity"]

    def __init__(self, grid, equations, U0=None, scheme="rk4", cfl=0.3, adaptive_config=None,
                 artificial_viscosity_config=None, gravity_config=None):
        cfg = getattr(grid, "mhd_config", None) or {}
        self.resistivity = float(cfg.get("resistivity", 0.0))
        self.viscosity = float(cfg.get("viscosity", 0.0))
        self.project_each_substage = bool(cfg.get("project_each_substage", True))
        self.divergence_clean = str(cfg.get("divergence_clean", "projection"))
        self.cfl_diff = float(cfg.get("cfl_diff", 1.0))
        if gravity_config and gravity_config.get("enabled", False):
            raise NotImplementedError("backend 'gb300': gravity is not implemented for MHD")
        if adaptive_config and adaptive_config.get("enabled", False) and self._ndim == 1:
            raise NotImplementedError("backend 'gb300': adaptive stepping of 1D MHD is not implemented")
        self.dim = self._ndim
        # the reference's MHD solver takes artificial_viscosity_config for API
        # compatibility and does not use it
        super().__init__(grid, equations, U0, scheme, cfl, adaptive_config, None, None)

    def _spacing(self) -> float:
        return min(self.grid.dx, self.grid.dy)

    def compute_dt(self, U: Any) -> float:
        s = float(self.plan.max_wave_speed(self.grid.to_device(U)).item())
        if s <= 0.0:
            return 1e-6
        dt = self.cfl * self._spacing() / s
        dif = max(self.resistivity, self.viscosity)
        if dif > 0.0:  # parabolic limit, k^2_max = sum over axes of (pi N / L)^2 (solver.py:916-929)
            dt = min(dt, self.cfl_diff / (dif * self._k2_max()))
        return dt

    def _k2_max(self) -> float:
        return (math.pi * self.grid.Nx / self.grid.Lx) ** 2 + (math.pi * self.grid.Ny / self.grid.Ly) ** 2

    def _project_B(self, U: Any) -> torch.Tensor:
        V = self.grid.to_device(U).clone()
        self.plan.project_state_(V)
        return V

    def max_div_b(self, U: Any) -> float:
        t = self.grid.to_device(U)
        return float(torch.max(torch.abs(self.grid.divergence(t[5], t[6]))).item())

    def _record(self, history: Dict[str, List[float]]) -> None:
        super()._record(history)
        history.setdefault("div_b_max", []).append(self.max_div_b(self.U))

    def run(self, U0: Any, t0: float, t_end: float, output_interval: float = 0.1, checkpoint_interval: float = 0.0,
            outdir: Optional[str] = None, on_output: Optional[Callable[[float, Any], None]] = None,
            on_step: Optional[Callable[[int, float, Any], None]] = None, tracers: Optional[Any] = None,
            dt: Optional[float] = None) -> Dict[str, List[float]]:
        """solver.py:1092-1162: the initial state is projected first."""
        return super().run(self._project_B(U0), t0, t_end, output_interval, checkpoint_interval, outdir,
                           on_output, on_step, tracers, dt)


class SpectralSolverMHD3D(SpectralSolverMHD2D):
    """3D ideal/resistive MHD (phrike/solver.py:840-1049, 1173-1174): the
    same stage structure as 2D with the 3D fluxes, the 3D projection after
    every stage and the filter then projection at the cadence; CFL dt =
    cfl * min(dx, dy, dz) / max(max(|ux|, |uy|, |uz|) + sqrt(a^2 + b^2)),
    capped by cfl_diff / (max(eta, nu) k^2_max) with diffusion."""

    _ndim = 3

    def _spacing(self) -> float:
        return min(self.grid.dx, self.grid.dy, self.grid.dz)

    def _k2_max(self) -> float:
        g = self.grid
        return sum((math.pi * n / L) ** 2 for n, L in ((g.Nx, g.Lx), (g.Ny, g.Ly), (g.Nz, g.Lz)))

    def max_div_b(self, U: Any) -> float:
        t = self.grid.to_device(U)
        return float(torch.max(torch.abs(self.grid.divergence(t[5], t[6], t[7]))).item())


class SpectralSolverMHD1D(SpectralSolverMHD2D):
    """1D MHD (phrike/solver.py:840-1049, 1165-1166): the x flux of
    MHDEquations1D, every RK stage clamped and (project_each_substage)
    projected with Bx <- mean(Bx), the filter and the projection at the
    cadence, explicit resistivity / viscosity; whole steps run in one kernel
    per solve.  CFL dt = cfl * dx / max(|u_x| + c_f), c_f the exact fast
    magnetosonic speed along x."""

    _ndim = 1

    def _spacing(self) -> float:
        return self.grid.dx

    def _k2_max(self) -> float:
        return (math.pi * self.grid.N / self.grid.Lx) ** 2

    def max_div_b(self, U: Any) -> float:
        t = self.grid.to_device(U)
        return float(torch.max(torch.abs(self.grid.dx1(t[5]))).item())
