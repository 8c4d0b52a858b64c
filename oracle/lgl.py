"""CPU oracle for the 2D Legendre-Gauss-Lobatto (LGL) collocation path.

TEST INFRASTRUCTURE ONLY (see oracle/spectral.py).  Restates, in NumPy
float64, the reference's LGL basis, its wall boundary conditions and the 2D
RK4 step on an LGL x LGL grid.  Pinned against golden vectors produced by
running the reference's torch-CPU float64 backend (tests/golden/make_golden.py).
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import numpy.polynomial.legendre as npleg
from scipy.special import eval_legendre, roots_jacobi

from .spectral import positivity_clamp, primitive


def lgl_nodes_weights(n: int) -> Tuple[np.ndarray, np.ndarray]:
    """Ascending LGL nodes on [-1, 1] and weights 2/(n(n-1) P_{n-1}^2)
    (phrike/basis/legendre.py:523-602, 628-671: interior nodes are the
    Jacobi(1,1) roots in double precision)."""
    if n == 2:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    if n == 3:
        return np.array([-1.0, 0.0, 1.0]), np.array([1 / 3, 4 / 3, 1 / 3])
    xi, _ = roots_jacobi(n - 2, 1.0, 1.0)
    y = np.concatenate([[-1.0], xi, [1.0]])
    P = eval_legendre(n - 1, y)
    w = 2.0 / (n * (n - 1) * P ** 2)
    w[0] = w[-1] = 2.0 / (n * (n - 1))
    return y, w


def legendre_diff_matrix(y: np.ndarray) -> np.ndarray:
    """D_y = dV V^{-1} via a transposed solve (legendre.py:605-624)."""
    n = y.shape[0]
    V = npleg.legvander(y, n - 1)
    dV = np.empty_like(V)
    for k in range(n):
        c = np.zeros(n)
        c[k] = 1.0
        dV[:, k] = npleg.legval(y, npleg.legder(c))
    return np.linalg.solve(V.T, dV.T).T


class LGLAxis:
    """One axis of LGL x LGL: nodes x = (1 - y) L/2 with y descending, so x
    ascends on [0, L]; D_x = -(2/L) D_y (legendre.py:694-729)."""

    def __init__(self, n: int, length: float):
        y, w = lgl_nodes_weights(n)
        order = np.argsort(-y)
        self.y = y[order]
        self.w_ref = w[order]
        self.x = (1.0 - self.y) * (length / 2.0)
        self.D = (-2.0 / length) * legendre_diff_matrix(self.y)
        self.V = npleg.legvander(self.y, n - 1)
        k = np.arange(n, dtype=float)
        self.proj = (2.0 * k + 1.0) / 2.0
        self.n = n

    def nodal_filter(self, p: int, alpha: float) -> np.ndarray:
        """Fn = (V diag(sigma proj) V^T) diag(w_ref), sigma_k = exp(-alpha (k/(N-1))^p)
        (legendre.py:825-841)."""
        k = np.arange(self.n, dtype=float)
        sigma = np.exp(-float(alpha) * (k / max(float(self.n - 1), 1.0)) ** int(p))
        M1 = self.V * (sigma * self.proj)[None, :]
        return (M1 @ self.V.T) * self.w_ref[None, :]


def apply_wall_bc(U: np.ndarray) -> np.ndarray:
    """Solid walls of Grid2D for bc='dirichlet' with no bc_config
    (grid.py:1004-1039, 1072-1154), in place, boundaries in the order
    left, right, top, bottom; per boundary density, momentum_x, momentum_y,
    energy.  Neumann copies the neighbouring interior line; Dirichlet sets the
    normal momentum to 0."""
    # left / right: normal is x
    for side, (dst, src) in (("left", (0, 1)), ("right", (-1, -2))):
        U[0, :, dst] = U[0, :, src]
        U[1, :, dst] = 0.0
        U[2, :, dst] = U[2, :, src]
        U[3, :, dst] = U[3, :, src]
    # top / bottom: normal is y (top = last row)
    for side, (dst, src) in (("top", (-1, -2)), ("bottom", (0, 1))):
        U[0, dst, :] = U[0, src, :]
        U[1, dst, :] = U[1, src, :]
        U[2, dst, :] = 0.0
        U[3, dst, :] = U[3, src, :]
    return U


class LGLSolver2D:
    """RK4 step of SpectralSolver2D on an LGL x LGL grid (solver.py:428-524,
    613-648): BCs in place on the stage input, flux, dx = f Dx^T,
    dy = Dy f, 2D positivity clamp after every stage, filter (if enabled)
    then BCs after the step."""

    def __init__(self, nx: int, ny: int, lx: float = 2.0, ly: float = 2.0, gamma: float = 1.4,
                 filter_params: Optional[dict] = None, cfl: float = 0.3, gravity: Optional[Tuple[float, float]] = None,
                 scheme: str = "rk4"):
        self.ax = LGLAxis(nx, lx)
        self.ay = LGLAxis(ny, ly)
        self.gamma = gamma
        self.cfl = cfl
        fp = filter_params or {}
        self.filter = bool(fp.get("enabled", False))
        self.Fx = self.ax.nodal_filter(int(fp.get("p", 8)), float(fp.get("alpha", 36.0))) if self.filter else None
        self.Fy = self.ay.nodal_filter(int(fp.get("p", 8)), float(fp.get("alpha", 36.0))) if self.filter else None
        self.step_counter = 0
        self.interval = max(1, int(fp.get("interval", 1) or 1))
        self.gravity = gravity
        self.scheme = scheme

    def dx(self, f):
        return f @ self.ax.D.T

    def dy(self, f):
        return np.matmul(self.ay.D, f)  # D_y applied along the second-to-last axis

    def rhs(self, U: np.ndarray) -> np.ndarray:
        """Applies the BCs to U in place first, like _compute_rhs_2d."""
        apply_wall_bc(U)
        rho, vel, p = primitive(U, self.gamma)
        E = U[3]
        mx, my = rho * vel[0], rho * vel[1]
        Fx = np.array([mx, mx * vel[0] + p, mx * vel[1], (E + p) * vel[0]])
        Fy = np.array([my, my * vel[0], my * vel[1] + p, (E + p) * vel[1]])
        r = -(self.dx(Fx) + self.dy(Fy))
        if self.gravity is not None:  # solver.py:453-464
            gx, gy = self.gravity
            r[1] += rho * gx
            r[2] += rho * gy
            r[3] += rho * (gx * vel[0] + gy * vel[1])
        return r

    def clamp(self, U):
        return positivity_clamp(U, self.gamma, 1e-8, 1e-10)

    def step(self, U: np.ndarray, dt: float) -> np.ndarray:
        """The reference mutates U through the BCs of the first stage; the
        caller's array is modified the same way here."""
        k1 = self.rhs(U)
        if self.scheme == "rk2":  # _rk2_step_2d (solver.py:492-500)
            U1 = self.clamp(U + dt * 0.5 * k1)
            Un = self.clamp(U + dt * self.rhs(U1))
        else:
            U2 = self.clamp(U + 0.5 * dt * k1)
            k2 = self.rhs(U2)
            U3 = self.clamp(U + 0.5 * dt * k2)
            k3 = self.rhs(U3)
            U4 = self.clamp(U + dt * k3)
            k4 = self.rhs(U4)
            Un = self.clamp(U + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4))
        if self.step_counter % self.interval == 0:
            if self.filter:
                Un = np.matmul(self.Fy, Un @ self.Fx.T)
            apply_wall_bc(Un)
        self.step_counter += 1
        return Un

    def compute_dt(self, U: np.ndarray) -> float:
        """cfl * min(dx_min, dy_min) / max(|u_x| + a) (solver.py:613-620, Q3)."""
        rho, vel, p = primitive(U, self.gamma)
        s = float(np.max(np.abs(vel[0]) + np.sqrt(self.gamma * p / rho)))
        h = min(float(np.min(np.diff(self.ax.x))), float(np.min(np.diff(self.ay.x))))
        return 1e-6 if s <= 0 else self.cfl * h / s
