"""CPU oracle for 2D (2.5D) ideal MHD on a periodic Fourier grid.

TEST INFRASTRUCTURE ONLY (see oracle/spectral.py).  Restates, in NumPy
float64, the reference's MHDEquations2D (phrike/equations.py:770-907), the
2D Helmholtz (Leray) projection of Grid2D (grid.py:1297-1327) and the RK4
step of SpectralSolverMHD (solver.py:840-1049) for the ideal case
(resistivity = viscosity = 0).  Pinned against golden vectors produced by
running the reference's NumPy path (tests/golden/make_golden.py).
"""
from __future__ import annotations

from typing import Dict, Optional, Tuple

import numpy as np

from .spectral import FourierBox, fftn, ifftn


def primitive(U: np.ndarray, gamma: float):
    """rho, ux, uy, uz, p, Bx, By, Bz; p = (gamma-1)(E - rho|u|^2/2 - |B|^2/2)
    (equations.py:783-795)."""
    rho = U[0]
    ux, uy, uz = U[1] / rho, U[2] / rho, U[3] / rho
    Bx, By, Bz = U[5], U[6], U[7]
    kin = 0.5 * rho * (ux * ux + uy * uy + uz * uz)
    mag = 0.5 * (Bx * Bx + By * By + Bz * Bz)
    p = (gamma - 1.0) * (U[4] - kin - mag)
    return rho, ux, uy, uz, p, Bx, By, Bz


def conservative(rho, ux, uy, uz, p, Bx, By, Bz, gamma: float) -> np.ndarray:
    """equations.py:797-810"""
    E = p / (gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    return np.array([rho, rho * ux, rho * uy, rho * uz, E, Bx, By, Bz])


def fluxes(U: np.ndarray, gamma: float) -> Tuple[np.ndarray, np.ndarray]:
    """Fx, Fy of equations.py:812-872 (E taken from the state)."""
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    E = U[4]
    uB = ux * Bx + uy * By + uz * Bz
    ps = p + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    mx, my = rho * ux, rho * uy
    z = np.zeros_like(rho)
    Fx = np.array([mx, mx * ux + ps - Bx * Bx, mx * uy - Bx * By, mx * uz - Bx * Bz,
                   (E + ps) * ux - Bx * uB, z, ux * By - uy * Bx, ux * Bz - uz * Bx])
    Fy = np.array([my, my * ux - By * Bx, my * uy + ps - By * By, my * uz - By * Bz,
                   (E + ps) * uy - By * uB, uy * Bx - ux * By, z, uy * Bz - uz * By])
    return Fx, Fy


def max_wave_speed(U: np.ndarray, gamma: float) -> float:
    """max(|ux|, |uy|) + sqrt(a^2 + b^2) (equations.py:874-887)."""
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    a2 = gamma * p / rho
    b2 = (Bx * Bx + By * By + Bz * Bz) / rho
    return float(np.max(np.maximum(np.abs(ux), np.abs(uy)) + np.sqrt(np.maximum(a2 + b2, 0.0))))


def conserved_quantities(U: np.ndarray, gamma: float) -> Dict[str, float]:
    """equations.py:889-907"""
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    b2 = Bx * Bx + By * By + Bz * Bz
    E = p / (gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * b2
    return {"mass": float(rho.sum()), "momentum_x": float((rho * ux).sum()),
            "momentum_y": float((rho * uy).sum()), "momentum_z": float((rho * uz).sum()),
            "energy": float(E.sum()), "magnetic_energy": float((0.5 * b2).sum()),
            "cross_helicity": float((ux * Bx + uy * By + uz * Bz).sum())}


def project_solenoidal(box: FourierBox, Bx: np.ndarray, By: np.ndarray):
    """Grid2D.project_solenoidal (grid.py:1297-1327): Nyquist row/column
    zeroed, then B_hat -= k (k . B_hat) / k^2 (k = 0 kept)."""
    ny, nx = box.shape
    Fx = fftn(Bx, (-2, -1))
    Fy = fftn(By, (-2, -1))
    for F in (Fx, Fy):
        if nx % 2 == 0:
            F[..., :, nx // 2] = 0
        if ny % 2 == 0:
            F[..., ny // 2, :] = 0
    kx = box.k[1][None, :]
    ky = box.k[0][:, None]
    k2 = kx * kx + ky * ky
    k2s = np.where(k2 == 0.0, 1.0, k2)
    coef = (kx * Fx + ky * Fy) / k2s
    return ifftn(Fx - kx * coef, (-2, -1)).real, ifftn(Fy - ky * coef, (-2, -1)).real


class MHDSolver2D:
    """SpectralSolverMHD in 2D, ideal, RK4 (solver.py:942-1049): rhs =
    -(dx1 Fx + dy1 Fy); every stage clamp then project; after the step, at the
    filter cadence, the spectral filter then the projection."""

    def __init__(self, nx: int, ny: int, lx: float = 2 * np.pi, ly: float = 2 * np.pi, gamma: float = 5.0 / 3.0,
                 dealias: bool = True, filter_params: Optional[dict] = None, cfl: float = 0.3,
                 rho_min: float = 1e-10, p_min: float = 1e-12, project_each_substage: bool = True,
                 divergence_clean: str = "projection", scheme: str = "rk4", resistivity: float = 0.0,
                 viscosity: float = 0.0, cfl_diff: float = 1.0):
        fp = filter_params or {}
        self.box = FourierBox((ny, nx), (ly, lx), dealias=dealias, filter_enabled=bool(fp.get("enabled", False)),
                              filter_p=int(fp.get("p", 8)), filter_alpha=float(fp.get("alpha", 36.0)))
        self.gamma = gamma
        self.cfl = cfl
        self.rho_min, self.p_min = rho_min, p_min
        self.project_each_substage = project_each_substage
        self.divergence_clean = divergence_clean
        self.interval = max(1, int(fp.get("interval", 1) or 1))
        self.step_counter = 0
        self.scheme = scheme
        self.resistivity, self.viscosity, self.cfl_diff = resistivity, viscosity, cfl_diff

    def rhs(self, U: np.ndarray) -> np.ndarray:
        """_compute_rhs (solver.py:942-954): flux divergence plus the explicit
        resistivity eta lap(B) and viscosity nu lap(rho u)."""
        Fx, Fy = fluxes(U, self.gamma)
        r = -(self.box.deriv(Fx, 1) + self.box.deriv(Fy, 0))
        if self.resistivity != 0.0:
            for c in (5, 6, 7):
                r[c] = r[c] + self.resistivity * self.box.laplacian(U[c])
        if self.viscosity != 0.0:
            for c in (1, 2, 3):
                r[c] = r[c] + self.viscosity * self.box.laplacian(U[c])
        return r

    def clamp(self, U: np.ndarray) -> np.ndarray:
        """_clamp (solver.py:956-964)"""
        rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, self.gamma)
        return conservative(np.maximum(rho, self.rho_min), ux, uy, uz, np.maximum(p, self.p_min), Bx, By, Bz,
                            self.gamma)

    def project(self, U: np.ndarray) -> np.ndarray:
        """_project_B (solver.py:966-986): project (Bx, By), recompute E with
        the thermal pressure held fixed."""
        if self.divergence_clean == "none":
            return U
        rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, self.gamma)
        Bx, By = project_solenoidal(self.box, U[5], U[6])
        V = U.copy()
        V[5], V[6], V[7] = Bx, By, Bz
        V[4] = p / (self.gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
        return V

    def step(self, U: np.ndarray, dt: float) -> np.ndarray:
        proj = self.project if self.project_each_substage else (lambda x: x)
        k1 = self.rhs(U)
        if self.scheme == "rk2":  # _rk_substages midpoint branch (solver.py:992-996)
            U1 = proj(self.clamp(U + 0.5 * dt * k1))
            Un = proj(self.clamp(U + dt * self.rhs(U1)))
            if self.step_counter % self.interval == 0:
                Un = self.project(self.box.filt(Un))
            self.step_counter += 1
            return Un
        U2 = proj(self.clamp(U + 0.5 * dt * k1))
        k2 = self.rhs(U2)
        U3 = proj(self.clamp(U + 0.5 * dt * k2))
        k3 = self.rhs(U3)
        U4 = proj(self.clamp(U + dt * k3))
        k4 = self.rhs(U4)
        Un = proj(self.clamp(U + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)))
        if self.step_counter % self.interval == 0:
            Un = self.project(self.box.filt(Un))
        self.step_counter += 1
        return Un

    def compute_dt(self, U: np.ndarray) -> float:
        """compute_dt (solver.py:1018-1034), ideal: cfl * min(dx, dy) / max speed."""
        s = max_wave_speed(U, self.gamma)
        if s <= 0.0:
            return 1e-6
        dt = self.cfl * min(self.box.spacing) / s
        dif = max(self.resistivity, self.viscosity)
        if dif > 0.0:  # parabolic limit (solver.py:1028-1033) with k2_max of the grid (916-929)
            k2max = sum(float(np.max(k * k)) for k in self.box.k)
            dt = min(dt, self.cfl_diff / (dif * k2max))
        return dt

    def max_div_b(self, U: np.ndarray) -> float:
        return float(np.max(np.abs(self.box.deriv(U[5], 1) + self.box.deriv(U[6], 0))))


def max_wave_speed_1d(U: np.ndarray, gamma: float) -> float:
    """MHDEquations1D.max_wave_speed (equations.py:735-750): |u_x| + c_f."""
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    a2 = gamma * p / rho
    b2 = (Bx * Bx + By * By + Bz * Bz) / rho
    cax2 = Bx * Bx / rho
    disc = np.maximum((a2 + b2) ** 2 - 4.0 * a2 * cax2, 0.0)
    return float(np.max(np.abs(ux) + np.sqrt(0.5 * (a2 + b2 + np.sqrt(disc)))))


class MHDSolver1D(MHDSolver2D):
    """SpectralSolverMHD with dim 1 (solver.py:840-1049, 1165-1166): the x
    flux of MHDEquations1D (equations.py:698-733, F_Bx = 0), the 1D projection
    Bx <- mean(Bx) with the thermal pressure held fixed (grid.py:554-567,
    solver.py:966-986), clamp, filter cadence and diffusion as in 2D."""

    def __init__(self, n: int, lx: float = 1.0, **kw):
        super().__init__(n, 1, lx, 1.0, **kw)
        fp = kw.get("filter_params") or {}
        self.box = FourierBox((n,), (lx,), dealias=kw.get("dealias", True),
                              filter_enabled=bool(fp.get("enabled", False)), filter_p=int(fp.get("p", 8)),
                              filter_alpha=float(fp.get("alpha", 36.0)))

    def rhs(self, U: np.ndarray) -> np.ndarray:
        Fx, _ = fluxes(U, self.gamma)
        Fx[5] = 0.0
        r = -self.box.deriv(Fx, 0)
        if self.resistivity != 0.0:
            for c in (5, 6, 7):
                r[c] = r[c] + self.resistivity * self.box.laplacian(U[c])
        if self.viscosity != 0.0:
            for c in (1, 2, 3):
                r[c] = r[c] + self.viscosity * self.box.laplacian(U[c])
        return r

    def project(self, U: np.ndarray) -> np.ndarray:
        if self.divergence_clean == "none":
            return U
        rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, self.gamma)
        V = U.copy()
        V[5] = np.full_like(U[5], U[5].mean())
        V[4] = p / (self.gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (V[5] ** 2 + By * By + Bz * Bz)
        return V

    def compute_dt(self, U: np.ndarray) -> float:
        s = max_wave_speed_1d(U, self.gamma)
        if s <= 0.0:
            return 1e-6
        dt = self.cfl * self.box.spacing[0] / s
        dif = max(self.resistivity, self.viscosity)
        if dif > 0.0:
            dt = min(dt, self.cfl_diff / (dif * float(np.max(self.box.k[0] ** 2))))
        return dt

    def max_div_b(self, U: np.ndarray) -> float:
        return float(np.max(np.abs(self.box.deriv(U[5], 0))))


def fluxes_3d(U: np.ndarray, gamma: float):
    """Fx, Fy, Fz of MHDEquations3D.flux (equations.py:946-1038)."""
    Fx, Fy = fluxes(U, gamma)
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    E = U[4]
    uB = ux * Bx + uy * By + uz * Bz
    ps = p + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    mz = rho * uz
    Fz = np.array([mz, mz * ux - Bz * Bx, mz * uy - Bz * By, mz * uz + ps - Bz * Bz,
                   (E + ps) * uz - Bz * uB, uz * Bx - ux * Bz, uz * By - uy * Bz, np.zeros_like(rho)])
    return Fx, Fy, Fz


def max_wave_speed_3d(U: np.ndarray, gamma: float) -> float:
    """max(|ux|, |uy|, |uz|) + sqrt(a^2 + b^2) (equations.py:1040-1061)."""
    rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, gamma)
    a2 = gamma * p / rho
    b2 = (Bx * Bx + By * By + Bz * Bz) / rho
    um = np.maximum(np.maximum(np.abs(ux), np.abs(uy)), np.abs(uz))
    return float(np.max(um + np.sqrt(np.maximum(a2 + b2, 0.0))))


def project_solenoidal_3d(box: FourierBox, Bx: np.ndarray, By: np.ndarray, Bz: np.ndarray):
    """Grid3D.project_solenoidal (grid.py:1649-1684): Nyquist planes zeroed,
    B_hat -= k (k . B_hat) / k^2 (k = 0 kept)."""
    nz, ny, nx = box.shape
    F = [fftn(B, (-3, -2, -1)) for B in (Bx, By, Bz)]
    for G in F:
        if nx % 2 == 0:
            G[..., :, :, nx // 2] = 0
        if ny % 2 == 0:
            G[..., :, ny // 2, :] = 0
        if nz % 2 == 0:
            G[..., nz // 2, :, :] = 0
    kx = box.k[2][None, None, :]
    ky = box.k[1][None, :, None]
    kz = box.k[0][:, None, None]
    k2 = kx * kx + ky * ky + kz * kz
    k2s = np.where(k2 == 0.0, 1.0, k2)
    coef = (kx * F[0] + ky * F[1] + kz * F[2]) / k2s
    return tuple(ifftn(G - k * coef, (-3, -2, -1)).real for G, k in zip(F, (kx, ky, kz)))


class MHDSolver3D(MHDSolver2D):
    """SpectralSolverMHD3D (solver.py:840-1049, 1173-1174): rhs =
    -(dx1 Fx + dy1 Fy + dz1 Fz) + eta lap B + nu lap(rho u); clamp and 3D
    projection after every stage, filter then projection at the cadence;
    CFL dt = cfl min(dx, dy, dz) / max speed, parabolic limit with
    k^2_max = max(kx^2 + ky^2 + kz^2)."""

    def __init__(self, nx: int, ny: int, nz: int, lx: float = 1.0, ly: float = 1.0, lz: float = 1.0, **kw):
        super().__init__(nx, ny, lx, ly, **kw)
        fp = kw.get("filter_params") or {}
        self.box = FourierBox((nz, ny, nx), (lz, ly, lx), dealias=kw.get("dealias", True),
                              filter_enabled=bool(fp.get("enabled", False)), filter_p=int(fp.get("p", 8)),
                              filter_alpha=float(fp.get("alpha", 36.0)))

    def rhs(self, U: np.ndarray) -> np.ndarray:
        Fx, Fy, Fz = fluxes_3d(U, self.gamma)
        r = -(self.box.deriv(Fx, 2) + self.box.deriv(Fy, 1) + self.box.deriv(Fz, 0))
        if self.resistivity != 0.0:
            for c in (5, 6, 7):
                r[c] = r[c] + self.resistivity * self.box.laplacian(U[c])
        if self.viscosity != 0.0:
            for c in (1, 2, 3):
                r[c] = r[c] + self.viscosity * self.box.laplacian(U[c])
        return r

    def project(self, U: np.ndarray) -> np.ndarray:
        if self.divergence_clean == "none":
            return U
        rho, ux, uy, uz, p, Bx, By, Bz = primitive(U, self.gamma)
        Bx, By, Bz = project_solenoidal_3d(self.box, U[5], U[6], U[7])
        V = U.copy()
        V[5], V[6], V[7] = Bx, By, Bz
        V[4] = p / (self.gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
        return V

    def compute_dt(self, U: np.ndarray) -> float:
        s = max_wave_speed_3d(U, self.gamma)
        if s <= 0.0:
            return 1e-6
        dt = self.cfl * min(self.box.spacing) / s
        dif = max(self.resistivity, self.viscosity)
        if dif > 0.0:
            k2max = sum(float(np.max(k * k)) for k in self.box.k)
            dt = min(dt, self.cfl_diff / (dif * k2max))
        return dt

    def max_div_b(self, U: np.ndarray) -> float:
        return float(np.max(np.abs(self.box.deriv(U[5], 2) + self.box.deriv(U[6], 1) + self.box.deriv(U[7], 0))))
