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


# wall / neumann boundary codes per (boundary, variable): 0 copy the
# neighbouring interior value, 1 set to zero, 2 leave unchanged
BC_COPY, BC_ZERO, BC_NONE = 0, 1, 2


def bc_codes_1d(bc) -> np.ndarray:
    """Resolve Grid1D's boundary configuration (a string, a per-variable or a
    per-boundary dict; grid.py:184-246) into codes [boundary (left, right)]
    [variable (density, momentum, energy)] following apply_boundary_conditions
    (grid.py:620-735): "wall" (aliases reflective, dirichlet) zeroes the
    momentum and copies the interior value into density and energy;
    "neumann" (alias open) copies for every variable."""
    def norm_bc(v):
        n = str(v).strip().lower()
        return "wall" if n in ("reflective", "dirichlet", "wall") else "neumann" if n in ("neumann", "open") else n

    def norm_var(v):
        n = str(v).strip().lower()
        if n in ("rho", "density"):
            return "density"
        if n in ("p", "pressure"):
            return "pressure"
        if n in ("u", "velocity", "mom", "momentum", "momentum_x"):
            return "momentum"
        return n

    def norm_side(b):
        n = str(b).strip().lower()
        return "left" if n in ("left", "x0", "x_min", "start") else "right" if n in ("right", "x1", "x_max", "end") else n

    g, var_map, side_map = None, None, None
    if isinstance(bc, dict):
        if any(str(k).lower() in ("left", "right", "x0", "x1", "x_min", "x_max", "start", "end") for k in bc):
            side_map = {}
            for bk, vd in bc.items():
                side = norm_side(bk)
                if isinstance(vd, dict):
                    side_map[side] = {norm_var(k): norm_bc(v) for k, v in vd.items()}
                else:
                    side_map[side] = {v: norm_bc(vd) for v in ("density", "momentum", "pressure")}
        else:
            var_map = {norm_var(k): norm_bc(v) for k, v in bc.items()}
    elif isinstance(bc, str) and bc:
        g = norm_bc(bc)

    def get(var, side):
        if side_map is not None and side in side_map:
            return side_map[side].get(var, g or "wall")
        if var_map is not None:
            return var_map.get(var, g or "wall")
        gg = g or "wall"
        if gg == "wall":
            return "wall" if var == "momentum" else "neumann"
        return gg

    codes = np.full((2, 3), BC_NONE, dtype=np.int32)
    for si, side in enumerate(("left", "right")):
        for vi, var in enumerate(("density", "momentum", "pressure")):
            b = get(var, side)
            if var == "momentum":
                codes[si, vi] = BC_ZERO if b in ("wall", "reflective") else BC_COPY if b in ("neumann", "open") else BC_NONE
            else:
                codes[si, vi] = BC_COPY if b in ("neumann", "open", "wall") else BC_NONE
    return codes


def apply_bc_1d(U: np.ndarray, codes: np.ndarray) -> np.ndarray:
    """In place; variables in the order density, momentum, energy and, per
    variable, left then right (grid.py:702-735)."""
    for vi in range(3):
        for si, (dst, src) in enumerate(((0, 1), (-1, -2))):
            c = codes[si, vi]
            if c == BC_COPY:
                U[vi, dst] = U[vi, src]
            elif c == BC_ZERO:
                U[vi, dst] = 0.0
    return U


class LGLSolver1D:
    """SpectralSolver1D on a Legendre grid (solver.py:62-132, 259-269): the
    boundary conditions applied in place to every stage input, flux, rhs =
    -D F (plus constant gravity), 1D clamp after every stage, and after the
    step the nodal filter (if enabled) with the boundary conditions, inside
    the step and again at the filter cadence (_apply_physical_filters)."""

    def __init__(self, n: int, length: float = 1.0, gamma: float = 1.4, filter_params: Optional[dict] = None,
                 cfl: float = 0.4, bc="wall", gravity: Optional[float] = None, scheme: str = "rk4"):
        self.ax = LGLAxis(n, length)
        self.gamma, self.cfl, self.gravity, self.scheme = gamma, cfl, gravity, scheme
        fp = filter_params or {}
        self.filter = bool(fp.get("enabled", False))
        self.F = self.ax.nodal_filter(int(fp.get("p", 8)), float(fp.get("alpha", 36.0))) if self.filter else None
        self.interval = max(1, int(fp.get("interval", 1) or 1))
        self.codes = bc_codes_1d(bc)
        self.step_counter = 0

    def rhs(self, U: np.ndarray) -> np.ndarray:
        apply_bc_1d(U, self.codes)
        rho, vel, p = primitive(U, self.gamma)
        u = vel[0]
        F = np.array([rho * u, rho * u * u + p, (U[2] + p) * u])
        r = -(F @ self.ax.D.T)
        if self.gravity is not None:
            r[1] += rho * self.gravity
            r[2] += rho * self.gravity * u
        return r

    def clamp(self, U):
        return positivity_clamp(U, self.gamma, 1e-10, 1e-12)

    def filt(self, U):
        if self.filter:
            U = U @ self.F.T
        return apply_bc_1d(U, self.codes)

    def step(self, U: np.ndarray, dt: float) -> np.ndarray:
        k1 = self.rhs(U)
        if self.scheme == "rk2":
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
        Un = self.filt(Un)  # inside the step
        if self.step_counter % self.interval == 0:
            Un = self.filt(Un)  # cadence
        self.step_counter += 1
        return Un

    def compute_dt(self, U: np.ndarray) -> float:
        rho, vel, p = primitive(U, self.gamma)
        s = float(np.max(np.abs(vel[0]) + np.sqrt(self.gamma * p / rho)))
        if s <= 0.0:
            return 1e-6
        return self.cfl * float(np.min(np.diff(self.ax.x))) / s
