"""Tracer particles on periodic Fourier grids, advanced by leap-frog in the
spectrally interpolated fluid velocity (reference: phrike/tracers.py:35-236).

Positions live on the device as float64 (ndim, P) tensors; ``x``, ``y`` and
``z`` are views of their rows.  One step is one launch of ps_tracers_step:
the velocity u_a = U[1+a]/U[0] of the state is interpolated at every tracer
with the grid's dealias mask and filter (the trigonometric interpolant of
grid.evaluate_fourier_at_points*), and the tracers move by Euler on the
first step and leap-frog afterwards, wrapped into [0, L) per axis.
"""
from __future__ import annotations

from typing import Any, Optional

import numpy as np
import torch


class _FourierTracers:
    _ndim = 1
    _names = ("x",)

    def __init__(self, *coords: Any, mass: float = 1.0) -> None:
        arrs = [np.asarray(c, dtype=np.float64).reshape(-1) for c in coords]
        if any(a.shape != arrs[0].shape for a in arrs):
            raise ValueError(f"{', '.join(n + '0' for n in self._names)} must have the same size")
        self._host0 = np.stack(arrs)
        self._pos: Optional[torch.Tensor] = None
        self._prev: Optional[torch.Tensor] = None
        self.mass = float(mass)
        self._first_step = True

    def _ensure_device(self, device: torch.device) -> None:
        if self._pos is None or self._pos.device != device:
            src = self._host0 if self._pos is None else self._pos.cpu().numpy()
            self._pos = torch.as_tensor(np.ascontiguousarray(src), dtype=torch.float64, device=device)
            self._prev = self._pos.clone()

    def _coord(self, i: int):
        return self._pos[i] if self._pos is not None else self._host0[i]

    @property
    def x(self):
        return self._coord(0)

    def _check_grid(self, grid: Any) -> None:
        if getattr(grid, "_basis", "fourier") != "fourier":
            raise ValueError(f"{type(self).__name__} requires a grid with a Fourier basis")
        if len(grid._shape) != self._ndim:
            raise ValueError(f"{type(self).__name__} needs a {self._ndim}D grid")

    def step(self, grid: Any, equations: Any, U: Any, dt: float, velocity_out: Optional[torch.Tensor] = None
             ) -> None:
        """Advance by dt in the velocity of U (tracers.py step methods)."""
        self._check_grid(grid)
        self._ensure_device(grid.device)
        t = grid.to_device(U)
        grid.plan.tracers_step_(t, self._pos, self._prev, self._first_step, float(dt), velocity_out)
        self._first_step = False


class FourierTracers1D(_FourierTracers):
    """Tracers on a 1D Fourier grid (tracers.py:35-79)."""

    _ndim = 1
    _names = ("x",)

    def __init__(self, x0: Any, mass: float = 1.0) -> None:
        super().__init__(x0, mass=mass)


class FourierTracers2D(_FourierTracers):
    """Tracers on a 2D Fourier grid (tracers.py:82-148)."""

    _ndim = 2
    _names = ("x", "y")

    def __init__(self, x0: Any, y0: Any, mass: float = 1.0) -> None:
        super().__init__(x0, y0, mass=mass)

    @property
    def y(self):
        return self._coord(1)


class FourierTracers3D(_FourierTracers):
    """Tracers on a 3D Fourier grid (tracers.py:151-236)."""

    _ndim = 3
    _names = ("x", "y", "z")

    def __init__(self, x0: Any, y0: Any, z0: Any, mass: float = 1.0) -> None:
        super().__init__(x0, y0, z0, mass=mass)

    @property
    def y(self):
        return self._coord(1)

    @property
    def z(self):
        return self._coord(2)


def tracers_from_config(grid: Any, config: dict) -> Optional[_FourierTracers]:
    """Tracers from a ``tracers`` config block (problems/base.py:961-1021):
    ``enabled``, ``num``, ``layout`` ("random" or "uniform"), ``mass``,
    ``seed``; None when disabled or the grid is not Fourier."""
    tcfg = config or {}
    if not tcfg.get("enabled", False) or getattr(grid, "_basis", "fourier") != "fourier":
        return None
    num = int(tcfg.get("num", 100))
    layout = str(tcfg.get("layout", "random")).lower()
    mass = float(tcfg.get("mass", 1.0))
    rng = np.random.default_rng(tcfg.get("seed", None))
    nd = len(grid._shape)
    lengths = [grid.Lx, getattr(grid, "Ly", None), getattr(grid, "Lz", None)][:nd]
    if layout == "uniform":
        if nd == 1:
            return FourierTracers1D(np.linspace(0.0, lengths[0], num, endpoint=False), mass=mass)
        n = max(1, int(round(num ** (1.0 / nd))))
        axes = [np.linspace(0.0, L, n, endpoint=False) for L in lengths]
        mesh = np.meshgrid(*axes, indexing="ij")
        coords = [m.ravel()[:num] for m in mesh]
    else:
        coords = [rng.uniform(0.0, L, size=num).astype(np.float64) for L in lengths]
    return (FourierTracers1D, FourierTracers2D, FourierTracers3D)[nd - 1](*coords, mass=mass)
