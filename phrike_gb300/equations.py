"""Compressible Euler equations with the reference's interface (backend "gb300").

Mirrors EulerEquations1D/2D/3D of phrike/equations.py (lines 217-319,
322-381, 551-637).  These helpers evaluate element-wise formulas on device
tensors for user code (initial conditions, monitoring); the time stepper
itself runs the fused CUDA kernels of phrike_gb300.engine.  The state layout
is [rho, m_1..m_d, E] with momenta ordered x, y, z.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Tuple

import numpy as np
import torch


def _t(x, like=None):
    if isinstance(x, torch.Tensor):
        return x
    dev = like.device if isinstance(like, torch.Tensor) else None
    return torch.as_tensor(np.asarray(x), dtype=torch.float32, device=dev)


@dataclass
class _Euler:
    gamma: float = 1.4
    ndim: int = 1

    def primitive(self, U) -> Tuple:
        U = _t(U)
        rho = U[0]
        vel = [U[1 + i] / rho for i in range(self.ndim)]
        kin = 0.5 * rho * sum(v * v for v in vel)
        p = (self.gamma - 1.0) * (U[self.ndim + 1] - kin)
        return rho, vel, p

    def _conservative(self, rho, vel, p):
        rho = _t(rho)
        vel = [_t(v, rho) for v in vel]
        p = _t(p, rho)
        E = p / (self.gamma - 1.0) + 0.5 * rho * sum(v * v for v in vel)
        return torch.stack([rho] + [rho * v for v in vel] + [E], dim=0)

    def _fluxes(self, U):
        rho, vel, p = self.primitive(U)
        U = _t(U)
        E = U[self.ndim + 1]
        out = []
        for a in range(self.ndim):
            ma = rho * vel[a]
            comps = [ma] + [ma * vel[b] + (p if a == b else 0.0) for b in range(self.ndim)]
            comps.append((E + p) * vel[a])
            out.append(torch.stack(comps, dim=0))
        return out

    def max_wave_speed(self, U) -> float:
        rho, vel, p = self.primitive(U)
        a = torch.sqrt(self.gamma * p / rho)
        if self.ndim == 2:  # |u_x| + a only (equations.py:137-147)
            s = torch.abs(vel[0]) + a
        else:
            s = torch.abs(vel[0])
            for v in vel[1:]:
                s = torch.maximum(s, torch.abs(v))
            s = s + a
        return float(torch.max(s).item())


@dataclass
class EulerEquations1D(_Euler):
    """[rho, m, E] (phrike/equations.py:217-319)."""

    gamma: float = 1.4
    ndim: int = 1

    def primitive(self, U):
        rho, vel, p = super().primitive(U)
        a = torch.sqrt(self.gamma * p / rho)
        return rho, vel[0], p, a

    def conservative(self, rho, u, p):
        return self._conservative(rho, [u], p)

    def flux(self, U):
        return self._fluxes(U)[0]

    def conserved_quantities(self, U) -> Dict[str, float]:
        rho, u, p, _ = self.primitive(U)
        return {"mass": float(rho.double().sum()), "momentum": float((rho * u).double().sum()),
                "energy": float((p / (self.gamma - 1.0) + 0.5 * rho * u * u).double().sum())}


@dataclass
class EulerEquations2D(_Euler):
    """[rho, m_x, m_y, E] (phrike/equations.py:322-381)."""

    gamma: float = 1.4
    ndim: int = 2

    def primitive(self, U):
        rho, vel, p = super().primitive(U)
        return rho, vel[0], vel[1], p

    def conservative(self, rho, ux, uy, p):
        return self._conservative(rho, [ux, uy], p)

    def flux(self, U):
        Fx, Fy = self._fluxes(U)
        return Fx, Fy

    def conserved_quantities(self, U) -> Dict[str, float]:
        """Keeps the reference's unpacking of (rho, ux, uy, p) as (rho, u, p, _)
        (equations.py:372-381): the 'energy' entry uses uy in place of p."""
        rho, u, p, _ = self.primitive(U)
        return {"mass": float(rho.double().sum()), "momentum": float((rho * u).double().sum()),
                "energy": float((p / (self.gamma - 1.0) + 0.5 * rho * u * u).double().sum())}


@dataclass
class EulerEquations3D(_Euler):
    """[rho, m_x, m_y, m_z, E] (phrike/equations.py:551-637)."""

    gamma: float = 1.4
    ndim: int = 3

    def primitive(self, U):
        rho, vel, p = super().primitive(U)
        return rho, vel[0], vel[1], vel[2], p

    def conservative(self, rho, ux, uy, uz, p):
        return self._conservative(rho, [ux, uy, uz], p)

    def flux(self, U):
        Fx, Fy, Fz = self._fluxes(U)
        return Fx, Fy, Fz

    def conserved_quantities(self, U) -> Dict[str, float]:
        rho, ux, uy, uz, p = self.primitive(U)
        kin = 0.5 * rho * (ux * ux + uy * uy + uz * uz)
        return {"mass": float(rho.double().sum()), "momentum_x": float((rho * ux).double().sum()),
                "momentum_y": float((rho * uy).double().sum()), "momentum_z": float((rho * uz).double().sum()),
                "energy": float((p / (self.gamma - 1.0) + kin).double().sum())}
