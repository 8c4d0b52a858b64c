"""Compressible Euler and 2D ideal MHD equations with the reference's
interface (backend "gb300").

Mirrors EulerEquations1D/2D/3D and MHDEquations2D of phrike/equations.py
(lines 217-319, 322-381, 551-637, 770-907).  These helpers evaluate element-wise formulas on device
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


@dataclass
class MHDEquations2D:
    """Ideal compressible MHD in 2D (2.5D: all three vector components, fields
    depending on x and y), conservative state [rho, rho ux, rho uy, rho uz, E,
    Bx, By, Bz] (phrike/equations.py:770-907).  Element-wise helpers on
    device tensors; the stepper runs the CUDA kernels of the engine."""

    gamma: float = 5.0 / 3.0

    def primitive(self, U):
        U = _t(U)
        rho = U[0]
        ux, uy, uz = U[1] / rho, U[2] / rho, U[3] / rho
        Bx, By, Bz = U[5], U[6], U[7]
        kin = 0.5 * rho * (ux * ux + uy * uy + uz * uz)
        mag = 0.5 * (Bx * Bx + By * By + Bz * Bz)
        p = (self.gamma - 1.0) * (U[4] - kin - mag)
        return rho, ux, uy, uz, p, Bx, By, Bz

    def conservative(self, rho, ux, uy, uz, p, Bx, By, Bz):
        rho = _t(rho)
        ux, uy, uz, p, Bx, By, Bz = (_t(v, rho) for v in (ux, uy, uz, p, Bx, By, Bz))
        E = (p / (self.gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz)
             + 0.5 * (Bx * Bx + By * By + Bz * Bz))
        return torch.stack([rho, rho * ux, rho * uy, rho * uz, E, Bx, By, Bz], dim=0)

    def flux(self, U):
        U = _t(U)
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        E = U[4]
        uB = ux * Bx + uy * By + uz * Bz
        ps = p + 0.5 * (Bx * Bx + By * By + Bz * Bz)
        mx, my = rho * ux, rho * uy
        z = torch.zeros_like(rho)
        Fx = torch.stack([mx, mx * ux + ps - Bx * Bx, mx * uy - Bx * By, mx * uz - Bx * Bz,
                          (E + ps) * ux - Bx * uB, z, ux * By - uy * Bx, ux * Bz - uz * Bx], dim=0)
        Fy = torch.stack([my, my * ux - By * Bx, my * uy + ps - By * By, my * uz - By * Bz,
                          (E + ps) * uy - By * uB, uy * Bx - ux * By, z, uy * Bz - uz * By], dim=0)
        return Fx, Fy

    def max_wave_speed(self, U) -> float:
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        a2 = self.gamma * p / rho
        b2 = (Bx * Bx + By * By + Bz * Bz) / rho
        fast = torch.sqrt(torch.clamp(a2 + b2, min=0.0))
        return float(torch.max(torch.maximum(torch.abs(ux), torch.abs(uy)) + fast).item())

    def conserved_quantities(self, U) -> Dict[str, float]:
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        b2 = Bx * Bx + By * By + Bz * Bz
        E = p / (self.gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * b2
        return {"mass": float(rho.double().sum()), "momentum_x": float((rho * ux).double().sum()),
                "momentum_y": float((rho * uy).double().sum()), "momentum_z": float((rho * uz).double().sum()),
                "energy": float(E.double().sum()), "magnetic_energy": float((0.5 * b2).double().sum()),
                "cross_helicity": float((ux * Bx + uy * By + uz * Bz).double().sum())}


@dataclass
class MHDEquations3D(MHDEquations2D):
    """Ideal compressible MHD in 3D, state (8, Nz, Ny, Nx)
    (phrike/equations.py:911-1100): fluxes Fx, Fy, Fz and the isotropic CFL
    bound max(|ux|, |uy|, |uz|) + sqrt(a^2 + b^2)."""

    gamma: float = 5.0 / 3.0

    def flux(self, U):
        U = _t(U)
        Fx, Fy = super().flux(U)
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        ps = p + 0.5 * (Bx * Bx + By * By + Bz * Bz)
        mz = rho * uz
        uB = ux * Bx + uy * By + uz * Bz
        Fz = torch.stack([mz, mz * ux - Bz * Bx, mz * uy - Bz * By, mz * uz + ps - Bz * Bz,
                          (U[4] + ps) * uz - Bz * uB, uz * Bx - ux * Bz, uz * By - uy * Bz,
                          torch.zeros_like(rho)], dim=0)
        return Fx, Fy, Fz

    def max_wave_speed(self, U) -> float:
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        a2 = self.gamma * p / rho
        b2 = (Bx * Bx + By * By + Bz * Bz) / rho
        fast = torch.sqrt(torch.clamp(a2 + b2, min=0.0))
        um = torch.maximum(torch.maximum(torch.abs(ux), torch.abs(uy)), torch.abs(uz))
        return float(torch.max(um + fast).item())


@dataclass
class MHDEquations1D(MHDEquations2D):
    """Ideal compressible MHD varying along x only (phrike/equations.py:659-767):
    the same 8-component state, the x flux alone (its Bx row is zero, so Bx
    stays constant) and |u_x| + c_f (exact fast magnetosonic speed along x)."""

    gamma: float = 5.0 / 3.0

    def flux(self, U):
        return super().flux(U)[0]

    def max_wave_speed(self, U) -> float:
        rho, ux, uy, uz, p, Bx, By, Bz = self.primitive(U)
        a2 = self.gamma * p / rho
        b2 = (Bx * Bx + By * By + Bz * Bz) / rho
        cax2 = Bx * Bx / rho
        disc = torch.clamp((a2 + b2) * (a2 + b2) - 4.0 * a2 * cax2, min=0.0)
        return float(torch.max(torch.abs(ux) + torch.sqrt(0.5 * (a2 + b2 + torch.sqrt(disc)))).item())
