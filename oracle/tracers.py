"""CPU oracle for point evaluation and tracer advection.

TEST INFRASTRUCTURE ONLY: a float64 NumPy restatement of the reference's
spectral point evaluation without finufft (phrike/grid.py:581-618,
1180-1222, 1520-1632) and of the leap-frog tracers (phrike/tracers.py:35-236).
Only the tests, the smoke check and the benchmark's CPU leg may import it.

Parity pin: checked against tests/golden/tracers.npz, produced by running
the reference's own grids and tracer classes (tests/golden/make_golden.py).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .spectral import dealias_mask_1d, exp_filter_1d, physical_wavenumbers


def axis_symbol(n: int, dealias: bool, filter_params: Optional[dict]) -> np.ndarray:
    """mask x sigma along one axis (grid.py:47-63, 87-141 are separable products)."""
    c = dealias_mask_1d(n, dealias)
    if filter_params and filter_params.get("enabled", False):
        c = c * exp_filter_1d(n, int(filter_params.get("p", 8)), float(filter_params.get("alpha", 36.0)))
    return c


def eval_points(f: np.ndarray, points: Sequence[np.ndarray], lengths_xyz: Sequence[float], dealias: bool,
                filter_params: Optional[dict]) -> np.ndarray:
    """Re(sum_k c_k F_k exp(i k.x_p)) / N_total for f of shape (.., Ny, Nx)
    and points given x first (the reference's fallback branch: exponential
    matrices contracted against the masked, filtered spectrum)."""
    nd = f.ndim
    F = np.fft.fftn(f, axes=tuple(range(-nd, 0)))
    shape = f.shape
    for i in range(nd):  # array axis i, spatial axis nd-1-i
        c = axis_symbol(shape[i], dealias, filter_params)
        F = F * c.reshape([-1 if j == i else 1 for j in range(nd)])
    vals = F
    # contract the slowest array axis first: z (3D) or y (2D), then down to x
    for i in range(nd):
        a = nd - 1 - i  # spatial axis of array axis i
        k = physical_wavenumbers(shape[i], lengths_xyz[a])
        E = np.exp(1j * np.asarray(points[a])[:, None] * k[None, :])  # (P, n_i)
        if i == 0:
            vals = np.einsum("pk,k...->p...", E, vals)
        else:
            vals = np.einsum("pk,pk...->p...", E, vals)
    return np.real(vals) / np.prod(shape)


class Tracers:
    """FourierTracers1D/2D/3D in float64: Euler on the first step, then
    leap-frog; positions wrapped with np.mod per axis (tracers.py:50-79)."""

    def __init__(self, *coords: np.ndarray):
        self.pos = [np.asarray(c, dtype=np.float64).copy() for c in coords]
        self.prev = [p.copy() for p in self.pos]
        self.first = True

    def velocity(self, U: np.ndarray, lengths_xyz, dealias, filter_params) -> np.ndarray:
        nd = len(self.pos)
        return np.stack([eval_points(U[1 + a] / U[0], self.pos, lengths_xyz, dealias, filter_params)
                         for a in range(nd)])

    def step(self, U: np.ndarray, dt: float, lengths_xyz, dealias, filter_params) -> None:
        v = self.velocity(U, lengths_xyz, dealias, filter_params)
        for a in range(len(self.pos)):
            if self.first:
                self.prev[a] = self.pos[a].copy()
                new = self.pos[a] + dt * v[a]
            else:
                new = self.prev[a] + 2.0 * dt * v[a]
                self.prev[a] = self.pos[a].copy()
            self.pos[a] = np.mod(new, lengths_xyz[a])
        self.first = False
