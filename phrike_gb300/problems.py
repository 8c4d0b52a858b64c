"""Initial conditions of the benchmark workloads (host-side NumPy, float64).

The formulas are the analytic set-ups used for the single-solve, batched and
served workloads:

* smoothed Sod-type step, 1D periodic [0, L)            (``sod_smoothed``)
* Taylor-Green vortex, 3D periodic [0, 2 pi)^3           (``taylor_green_3d``)
* Kelvin-Helmholtz shear layer, 2D periodic [0, 1)^2     (``kelvin_helmholtz_2d``)
* Orszag-Tang vortex (ideal MHD), 2D periodic [0, 2 pi)^2 (``orszag_tang_2d``)
* circularly polarized Alfven wave (MHD), 1D periodic (``alfven_cp_1d``)
* Gaussian acoustic pulse on Legendre-Gauss-Lobatto nodes (``acoustic_pulse_lgl_2d``)

All return conservative states with component-first layout and spatial axes
(..., Ny, Nx) / (Nz, Ny, Nx), x last, which is the layout of the reference
(phrike/grid.py:779-780, 1361).
"""
from __future__ import annotations

from typing import Tuple

import numpy as np


def _euler_conservative(rho, vel, p, gamma):
    E = p / (gamma - 1.0) + 0.5 * rho * sum(v * v for v in vel)
    return np.stack([rho] + [rho * v for v in vel] + [E])


def sod_smoothed(N: int, L: float = 1.0, gamma: float = 1.4, width: float = 0.005) -> np.ndarray:
    """rho=1, p=1 on [0.25, 0.75) else rho=0.125, p=0.1, u=0; tanh edges."""
    x = np.linspace(0.0, L, N, endpoint=False)
    s = 0.5 * (np.tanh((x - 0.25 * L) / width) - np.tanh((x - 0.75 * L) / width))
    rho = 0.125 + (1.0 - 0.125) * s
    p = 0.1 + (1.0 - 0.1) * s
    u = np.zeros_like(x)
    return _euler_conservative(rho, [u], p, gamma)


def taylor_green_3d(Nx: int, Ny: int = None, Nz: int = None, gamma: float = 1.4,
                    L: float = 2.0 * np.pi) -> np.ndarray:
    """rho=1, u=sin x cos y cos z, v=-cos x sin y cos z, w=0,
    p = 100/gamma + (cos 2x + cos 2y)(cos 2z + 2)/16 on [0, L)^3."""
    Ny = Nx if Ny is None else Ny
    Nz = Nx if Nz is None else Nz
    x = np.linspace(0.0, L, Nx, endpoint=False)
    y = np.linspace(0.0, L, Ny, endpoint=False)
    z = np.linspace(0.0, L, Nz, endpoint=False)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    rho = np.ones_like(X)
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = 100.0 / gamma + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    return _euler_conservative(rho, [u, v, w], p, gamma)


def kelvin_helmholtz_2d(Nx: int, Ny: int = None, U0: float = 1.0, A: float = 0.01,
                        gamma: float = 1.4) -> np.ndarray:
    """Double shear layer on [0,1)^2: profile s(y) = tanh((y-.25)/.05) - tanh((y-.75)/.05) - 1,
    u = U0 s, rho = 1.5 + 0.5 s, p = 2.5,
    v = A sin(4 pi x)(exp(-(y-.25)^2/.0025) + exp(-(y-.75)^2/.0025))."""
    Ny = Nx if Ny is None else Ny
    x = np.linspace(0.0, 1.0, Nx, endpoint=False)
    y = np.linspace(0.0, 1.0, Ny, endpoint=False)
    X, Y = np.meshgrid(x, y, indexing="xy")
    s = np.tanh((Y - 0.25) / 0.05) - np.tanh((Y - 0.75) / 0.05) - 1.0
    u = U0 * s
    rho = 1.5 + 0.5 * s
    p = 2.5 * np.ones_like(X)
    v = A * np.sin(4.0 * np.pi * X) * (np.exp(-(Y - 0.25) ** 2 / 0.0025)
                                        + np.exp(-(Y - 0.75) ** 2 / 0.0025))
    return _euler_conservative(rho, [u, v], p, gamma)


def orszag_tang_2d(Nx: int, Ny: int = None, gamma: float = 5.0 / 3.0, rho0: float = None, p0: float = None,
                   B0: float = 1.0, L: float = 2.0 * np.pi) -> np.ndarray:
    """Orszag-Tang vortex on [0, L)^2 with the reference's parametrisation
    (problems/problem_list/orszag_tang2d.py:33-66): rho = rho0, p = p0,
    u = -sin(2 pi y/L), v = sin(2 pi x/L), Bx = -B0 sin(2 pi y/L),
    By = B0 sin(4 pi x/L); defaults rho0 = gamma^2, p0 = gamma, B0 = 1,
    L = 2 pi.  8 components in the reference order
    [rho, rho ux, rho uy, rho uz, E, Bx, By, Bz] (equations.py:770-810)."""
    Ny = Nx if Ny is None else Ny
    rho0 = gamma ** 2 if rho0 is None else rho0
    p0 = gamma if p0 is None else p0
    x = np.linspace(0.0, L, Nx, endpoint=False)
    y = np.linspace(0.0, L, Ny, endpoint=False)
    X, Y = np.meshgrid(x, y, indexing="xy")
    k = 2.0 * np.pi / L
    rho = rho0 * np.ones_like(X)
    p = p0 * np.ones_like(X)
    u = -np.sin(k * Y)
    v = np.sin(k * X)
    w = np.zeros_like(X)
    Bx = -B0 * np.sin(k * Y)
    By = B0 * np.sin(2.0 * k * X)
    Bz = np.zeros_like(X)
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    return np.stack([rho, rho * u, rho * v, rho * w, E, Bx, By, Bz])


def alfven_cp_1d(N: int, L: float = 1.0, t: float = 0.0, rho0: float = 1.0, p0: float = 0.1, B0: float = 1.0,
                 b1: float = 0.1, m: int = 1, direction: int = 1, gamma: float = 5.0 / 3.0) -> np.ndarray:
    """Circularly polarized Alfven wave on [0, L) (the reference's alfven1d
    problem, problems/problem_list/alfven1d.py:30-82): rho = rho0, p = p0,
    Bx = B0, (By, Bz) = b1 (cos, sin)(k x - k c_A t), u_perp = -direction
    B_perp / sqrt(rho0), u_x = 0; 8 MHD components."""
    x = np.linspace(0.0, L, N, endpoint=False)
    cA = B0 / np.sqrt(rho0)
    k = 2.0 * np.pi * m / L
    phi = k * x - k * direction * cA * t
    By, Bz = b1 * np.cos(phi), b1 * np.sin(phi)
    rho = np.full_like(x, rho0)
    ux = np.zeros_like(x)
    uy, uz = -direction * By / np.sqrt(rho0), -direction * Bz / np.sqrt(rho0)
    Bx = np.full_like(x, B0)
    E = p0 / (gamma - 1.0) + 0.5 * rho * (uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    return np.stack([rho, rho * ux, rho * uy, rho * uz, E, Bx, By, Bz])


def alfven_cp_3d(Nx: int, Ny: int, Nz: int, Lx: float = 1.0, t: float = 0.0, rho0: float = 1.0, p0: float = 0.1,
                 B0: float = 1.0, b1: float = 0.1, m: int = 1, direction: int = 1,
                 gamma: float = 5.0 / 3.0) -> np.ndarray:
    """The circularly polarized Alfven wave along x in a 3D box (the
    reference's alfven3d problem, problems/problem_list/alfven3d.py:23-50):
    the 1D profile repeated over (z, y); shape (8, Nz, Ny, Nx)."""
    U1 = alfven_cp_1d(Nx, Lx, t, rho0, p0, B0, b1, m, direction, gamma)
    return np.ascontiguousarray(np.broadcast_to(U1[:, None, None, :], (8, Nz, Ny, Nx)))


def acoustic_pulse_lgl_1d(x: np.ndarray, gamma: float = 1.4, amp: float = 0.01, width2: float = 0.01,
                          center: float = 0.0) -> np.ndarray:
    """rho = 1 + amp exp(-(x - center)^2/width2), p = rho^gamma/gamma, u = 0
    on the given node coordinates (domain [-1, 1])."""
    rho = 1.0 + amp * np.exp(-((np.asarray(x) - center) ** 2) / width2)
    p = rho ** gamma / gamma
    return _euler_conservative(rho, [np.zeros_like(rho)], p, gamma)


def acoustic_pulse_lgl_2d(x: np.ndarray, y: np.ndarray, gamma: float = 1.4,
                          amp: float = 0.01, width2: float = 0.01,
                          center: Tuple[float, float] = (0.0, 0.0)) -> np.ndarray:
    """rho = 1 + amp exp(-r^2/width2), p = rho^gamma/gamma, u = v = 0 on
    the given node coordinates (1-D arrays for x and y, domain [-1, 1]^2)."""
    X, Y = np.meshgrid(x, y, indexing="xy")
    r2 = (X - center[0]) ** 2 + (Y - center[1]) ** 2
    rho = 1.0 + amp * np.exp(-r2 / width2)
    p = rho ** gamma / gamma
    z = np.zeros_like(X)
    return _euler_conservative(rho, [z, z], p, gamma)
