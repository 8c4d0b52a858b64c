"""CPU oracle for the pseudo-spectral Euler right-hand-side-and-step path.

TEST INFRASTRUCTURE ONLY.  This module restates, in NumPy/SciPy float64, the
algorithm of the reference package (phrike) for the hot path that the CUDA
library replaces.  Only the test-suite, the smoke check and the CPU-baseline
leg of the benchmark may import it; the product never calls it.

Parity pin: the results of this module are checked against golden vectors
produced by running the reference itself (``tests/golden/make_golden.py``).

Every function names the reference lines it follows (paths inside the
reference project).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

try:  # the reference prefers scipy.fft (pocketfft) with a worker count
    from scipy import fft as _fft
except Exception:  # pragma: no cover
    _fft = None


def _workers() -> int:
    w = os.environ.get("PHRIKE_ORACLE_WORKERS")
    if w:
        return max(1, int(w))
    return os.cpu_count() or 1


def fftn(f: np.ndarray, axes) -> np.ndarray:
    if _fft is not None:
        return _fft.fftn(f, axes=axes, workers=_workers())
    return np.fft.fftn(f, axes=axes)


def ifftn(F: np.ndarray, axes) -> np.ndarray:
    if _fft is not None:
        return _fft.ifftn(F, axes=axes, workers=_workers())
    return np.fft.ifftn(F, axes=axes)


# ---------------------------------------------------------------------------
# Spectral tables (grid.py:47-63 for one axis; 87-141 build the separable
# outer products of the same one-axis tables).
# ---------------------------------------------------------------------------

def integer_wavenumbers(n: int) -> np.ndarray:
    """k = fftfreq(n) * n, the signed integer mode index (grid.py:50, 59)."""
    return np.fft.fftfreq(n) * n


def dealias_mask_1d(n: int, dealias: bool) -> np.ndarray:
    """2/3 rule: keep |k| <= n // 3 (grid.py:47-54)."""
    if not dealias:
        return np.ones(n)
    k = integer_wavenumbers(n)
    return (np.abs(k) <= n // 3).astype(float)


def exp_filter_1d(n: int, p: int, alpha: float) -> np.ndarray:
    """sigma = exp(-alpha (|k|/kmax)^p), kmax = max|k| (grid.py:57-63)."""
    k = integer_wavenumbers(n)
    kmax = np.max(np.abs(k)) if n > 0 else 1.0
    eta = np.abs(k) / max(kmax, 1.0)
    return np.exp(-alpha * eta ** p)


def physical_wavenumbers(n: int, length: float) -> np.ndarray:
    """k = 2 pi fftfreq(n, d=L/n) (grid.py:255-257, 1382-1387)."""
    return 2.0 * np.pi * np.fft.fftfreq(n, d=length / n)


@dataclass
class FourierBox:
    """Periodic box of 1-3 dimensions with the reference's spectral operators.

    ``shape`` is the spatial shape in array order (Nz, Ny, Nx) / (Ny, Nx) /
    (N,); ``lengths`` follows the same order.  Fields carry leading component
    axes (..., *shape).
    """

    shape: Tuple[int, ...]
    lengths: Tuple[float, ...]
    dealias: bool = True
    filter_enabled: bool = False
    filter_p: int = 8
    filter_alpha: float = 36.0

    def __post_init__(self) -> None:
        nd = len(self.shape)
        self.ndim = nd
        self.axes = tuple(range(-nd, 0))
        self.k = [physical_wavenumbers(n, L) for n, L in zip(self.shape, self.lengths)]
        # separable mask * sigma (grid.py:87-141; dx1 multiplies both, 512-519)
        mult = np.ones(self.shape)
        for a, n in enumerate(self.shape):
            m1 = dealias_mask_1d(n, self.dealias)
            if self.filter_enabled:
                m1 = m1 * exp_filter_1d(n, self.filter_p, self.filter_alpha)
            view = [1] * nd
            view[a] = n
            mult = mult * m1.reshape(view)
        self.mult = mult
        self.spacing = tuple(L / n for n, L in zip(self.shape, self.lengths))

    def _kview(self, a: int) -> np.ndarray:
        view = [1] * self.ndim
        view[a] = self.shape[a]
        return self.k[a].reshape(view)

    def deriv(self, f: np.ndarray, a: int) -> np.ndarray:
        """Re IFFT(i k_a * mask * sigma * FFT f) over all spatial axes.

        Follows Grid1D.dx1 (grid.py:512-519), Grid2D.dx1/dy1 (1226-1252) and
        Grid3D.dx1/dy1/dz1 (1705-1721): a full N-D complex transform whose
        real part is kept.  ``a`` indexes the spatial shape (0 = slowest).
        """
        F = fftn(f, self.axes)
        F = F * self.mult
        F = F * (1j * self._kview(a))
        return ifftn(F, self.axes).real

    def laplacian(self, f: np.ndarray) -> np.ndarray:
        """Re IFFT(-|k|^2 * mask * sigma * FFT f) (grid.py:569-579, 1329-1338,
        1696-1703)."""
        F = fftn(f, self.axes) * self.mult
        k2 = sum(self._kview(a) ** 2 for a in range(self.ndim))
        return ifftn(-k2 * F, self.axes).real

    def filt(self, f: np.ndarray, real: bool = False) -> np.ndarray:
        """apply_spectral_filter: Re IFFT(mask * sigma * FFT f) (grid.py:524-538,
        1254-1287, 1723-1726).  ``real``: the same operator through real
        half-spectrum transforms (equal up to rounding, since mask * sigma is
        real and even in k)."""
        if real and _fft is not None:
            F = _fft.rfftn(f, axes=self.axes, workers=_workers()) * self.mult[..., : self.shape[-1] // 2 + 1]
            return _fft.irfftn(F, s=self.shape, axes=self.axes, workers=_workers())
        F = fftn(f, self.axes) * self.mult
        return ifftn(F, self.axes).real

    def flux_divergence(self, F: Sequence[np.ndarray]) -> np.ndarray:
        """sum_d dx1_d F_d with F indexed by direction (0 = x), evaluated as
        one spectral sum: IFFT(sum_d i k_d m s FFT F_d).

        The same operator as sum_d deriv(F_d, axis(d)) (grid.py:512-519,
        1226-1252, 1705-1721) by linearity; with the 2/3 mask every Nyquist
        mode is zero, so real half-spectrum transforms give the reference's
        real part exactly up to rounding.  Used for large-grid oracle runs
        (three forward and one inverse real transform per stage instead of
        three full complex round trips); ``tests/test_oracle_golden.py``
        checks it against ``deriv``.
        """
        if not self.dealias or _fft is None:
            return sum(self.deriv(Fd, self.ndim - 1 - d) for d, Fd in enumerate(F))
        nh = self.shape[-1] // 2 + 1
        mult = self.mult[..., :nh]
        acc = None
        for d, Fd in enumerate(F):
            a = self.ndim - 1 - d
            kv = self._kview(a)
            if a == self.ndim - 1:
                kv = kv[..., :nh]
            S = _fft.rfftn(Fd, axes=self.axes, workers=_workers()) * (1j * kv)
            acc = S if acc is None else acc + S
        return _fft.irfftn(acc * mult, s=self.shape, axes=self.axes, workers=_workers())


# ---------------------------------------------------------------------------
# Euler equations (equations.py:36-211 kernels; 217-381, 552-637 classes)
# Conservative state U = [rho, m_1..m_d, E] with m ordered (x, y, z).
# ---------------------------------------------------------------------------

def primitive(U: np.ndarray, gamma: float):
    """rho, velocities (x, y, z order), p (equations.py:36-60, 104-115, 150-164)."""
    d = U.shape[0] - 2
    rho = U[0]
    vel = [U[1 + i] / rho for i in range(d)]
    kin = 0.5 * rho * sum(v * v for v in vel)
    p = (gamma - 1.0) * (U[d + 1] - kin)
    return rho, vel, p


def conservative(rho, vel, p, gamma: float) -> np.ndarray:
    """[rho, rho u_i, p/(gamma-1) + rho |u|^2 / 2] (equations.py:255-278, 321-325, 569-580)."""
    E = p / (gamma - 1.0) + 0.5 * rho * sum(v * v for v in vel)
    return np.array([rho] + [rho * v for v in vel] + [E])


def fluxes(U: np.ndarray, gamma: float):
    """Flux along each axis x, y, z (equations.py:67-86, 118-134, 167-196).

    Returns a list indexed by direction (0 = x): F_a = [m_a, m_a u_b + delta p, (E+p) u_a].
    """
    d = U.shape[0] - 2
    rho, vel, p = primitive(U, gamma)
    E = U[d + 1]
    out = []
    for a in range(d):
        ma = rho * vel[a]
        comps = [ma]
        for b in range(d):
            comps.append(ma * vel[b] + (p if a == b else 0.0))
        comps.append((E + p) * vel[a])
        out.append(np.array(comps))
    return out


def max_wave_speed(U: np.ndarray, gamma: float) -> float:
    """1D: max(|u|+a); 2D: max(|u_x|+a) only; 3D: max(max_i |u_i| + a)
    (equations.py:89-98, 137-147, 199-211)."""
    d = U.shape[0] - 2
    rho, vel, p = primitive(U, gamma)
    a = np.sqrt(gamma * p / rho)
    if d == 2:
        s = np.abs(vel[0]) + a
    else:
        s = np.abs(vel[0])
        for v in vel[1:]:
            s = np.maximum(s, np.abs(v))
        s = s + a
    return float(np.max(s))


def conserved_sums(U: np.ndarray, gamma: float) -> Dict[str, float]:
    """Plain (unweighted) sums recorded by the solvers' record()
    (solver.py:372-377, 741-767, 1439-1468)."""
    d = U.shape[0] - 2
    rho, vel, p = primitive(U, gamma)
    out = {"mass": float(rho.sum())}
    names = ["momentum"] if d == 1 else ["momentum_x", "momentum_y", "momentum_z"][:d]
    for n, v in zip(names, vel):
        out[n] = float((rho * v).sum())
    out["energy"] = float((p / (gamma - 1.0) + 0.5 * rho * sum(v * v for v in vel)).sum())
    return out


def positivity_clamp(U: np.ndarray, gamma: float, rho_min: float, p_min: float) -> np.ndarray:
    """primitive -> max(rho, rho_min), max(p, p_min) -> conservative with the
    unclamped velocity (solver.py:32-59, 467-488)."""
    rho, vel, p = primitive(U, gamma)
    return conservative(np.maximum(rho, rho_min), vel, np.maximum(p, p_min), gamma)


# clamp floors per dimension (solver.py:32 for 1D, 467 for 2D; 3D has none)
CLAMP_FLOORS = {1: (1e-10, 1e-12), 2: (1e-8, 1e-10)}


@dataclass
class EulerSolver:
    """Fixed-dt RK4 stepper of SpectralSolver1D/2D/3D.

    1D: solver.py:62-132 (rhs, rk4 with clamp after every stage, filter inside
    the step) and 259-269 (the cadence filter applied again).
    2D: solver.py:428-524 (clamp each stage, filter by cadence) and 637-648.
    3D: solver.py:1177-1237 (no clamp), 1330-1337 (filter every step).
    Gravity (solver.py:82-91, 453-464, 1193-1206) is supported as constant g;
    artificial viscosity in 1D/2D (solver.py:73-78, 446-451; the 3D solver
    passes none, 1330-1337).
    """

    box: FourierBox
    gamma: float = 1.4
    cfl: float = 0.4
    filter_interval: int = 1
    gravity: Optional[Sequence[float]] = None
    step_counter: int = 0
    av: Optional[Dict] = None  # artificial-viscosity config (1D/2D), see av_terms
    scheme: str = "rk4"        # "rk4" or the midpoint "rk2"
    fused: bool = False        # one spectral sum per stage (FourierBox.flux_divergence)

    @property
    def ndim(self) -> int:
        return self.box.ndim

    def flux_axis_index(self, direction: int) -> int:
        """Direction 0=x,1=y,2=z → spatial axis index in array order."""
        return self.ndim - 1 - direction

    def av_terms(self, U: np.ndarray) -> np.ndarray:
        """SpectralArtificialViscosity.compute_viscosity_terms
        (artificial_viscosity.py:270-403, config 37-105, sensor 124-190,
        coefficient 193-235): sensor s = clip(|grad q| / (|q| + eps) / s_ref,
        0, 1) on q = density, pressure or |u|; nu = nu_max ((s > s_min ? s : 0)
        / s_ref)^p (or a constant); term_i = div(w_i nu grad U_i), with the
        weight looked up by position in the fixed name list."""
        cfg = self.av
        d = self.ndim
        axes = [self.flux_axis_index(a) for a in range(d)]
        mode = str(cfg.get("mode", "sensor")).lower().strip()
        if mode == "constant":
            nu = float(cfg.get("nu_constant", 0.0))
            if nu == 0.0:
                nu = float(cfg.get("nu_max", 1e-3))
            nu = np.full_like(U[0], nu)
        else:
            var = cfg.get("sensor_variable", "density")
            rho, vel, p = primitive(U, self.gamma)
            if var == "density":
                q = U[0]
            elif var == "pressure":
                # the sensor unpacks `_, _, p, _ = primitive(U)` (artificial_viscosity.py:131):
                # in 1D that is p, in 2D (rho, ux, uy, p) it is uy
                q = p if d == 1 else vel[1]
            elif d == 1:
                q = np.abs(vel[0])
            else:
                raise NotImplementedError("the reference's 2D velocity_magnitude sensor broadcasts rows of ux")
            grads = [self.box.deriv(q, ax) for ax in axes]
            gm = np.abs(grads[0]) if d == 1 else np.sqrt(sum(g * g for g in grads))
            sref = float(cfg.get("s_ref", 1.0))
            sen = gm / (np.abs(q) + float(cfg.get("epsilon", 1e-12)))
            if sref > 0:
                sen = np.clip(sen / sref, 0.0, 1.0)
            act = np.where(sen > float(cfg.get("s_min", 0.1)), sen, 0.0)
            if sref > 0:
                act = act / sref
            nu = float(cfg.get("nu_max", 1e-3)) * act ** float(cfg.get("p", 2.0))
        names = ["density", "momentum_x", "momentum_y", "momentum_z", "energy"]
        weights = cfg.get("variable_weights", None) or {}
        out = np.zeros_like(U)
        for i in range(U.shape[0]):
            w = float(weights.get(names[i], 1.0))
            for ax in axes:
                out[i] += self.box.deriv(nu * w * self.box.deriv(U[i], ax), ax)
        return out

    def rhs(self, U: np.ndarray) -> np.ndarray:
        F = fluxes(U, self.gamma)
        if self.fused:
            r = -self.box.flux_divergence(F)
        else:
            r = np.zeros_like(U)
            for a, Fa in enumerate(F):
                r -= self.box.deriv(Fa, self.flux_axis_index(a))
        if self.av is not None and self.ndim < 3:
            r += self.av_terms(U)
        if self.gravity is not None:
            d = self.ndim
            rho, vel, p = primitive(U, self.gamma)
            work = 0.0
            for i in range(d):
                g = float(self.gravity[i])
                r[1 + i] += rho * g
                work = work + g * vel[i]
            r[d + 1] += rho * work
        return r

    def clamp(self, U: np.ndarray) -> np.ndarray:
        if self.ndim == 3:
            return U
        rmin, pmin = CLAMP_FLOORS[self.ndim]
        return positivity_clamp(U, self.gamma, rmin, pmin)

    def rk4(self, U: np.ndarray, dt: float) -> np.ndarray:
        """Classical RK4 with the per-dimension clamp (solver.py:108-120,
        502-513, 1220-1230)."""
        k1 = self.rhs(U)
        U2 = self.clamp(U + 0.5 * dt * k1)
        k2 = self.rhs(U2)
        U3 = self.clamp(U + 0.5 * dt * k2)
        k3 = self.rhs(U3)
        U4 = self.clamp(U + dt * k3)
        k4 = self.rhs(U4)
        Un = U + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)
        Un = self.clamp(Un)
        if self.ndim == 1:
            Un = self.box.filt(Un, self.fused)  # inside _rk4_step (solver.py:119-120)
        return Un

    def rk2(self, U: np.ndarray, dt: float) -> np.ndarray:
        """Midpoint RK2 with the per-dimension clamp (solver.py:96-105,
        492-500, 1211-1216)."""
        k1 = self.rhs(U)
        U1 = self.clamp(U + dt * 0.5 * k1)
        k2 = self.rhs(U1)
        Un = self.clamp(U + dt * k2)
        if self.ndim == 1:
            Un = self.box.filt(Un)  # inside _rk2_step (solver.py:104)
        return Un

    def step(self, U: np.ndarray, dt: float) -> np.ndarray:
        Un = self.rk2(U, dt) if self.scheme == "rk2" else self.rk4(U, dt)
        if self.ndim == 3:
            Un = self.box.filt(Un, self.fused)  # every step (solver.py:1336)
        elif self.step_counter % self.filter_interval == 0:
            Un = self.box.filt(Un, self.fused)  # cadence (solver.py:265-267, 645-646)
        self.step_counter += 1
        return Un

    def compute_dt(self, U: np.ndarray) -> float:
        """cfl * min spacing / max speed (solver.py:235-240, 613-620, 1307-1311)."""
        s = max_wave_speed(U, self.gamma)
        if s <= 0.0:
            return 1e-6
        return self.cfl * min(self.box.spacing) / s

    def run(self, U0: np.ndarray, t0: float, t_end: float, max_steps: Optional[int] = None):
        """CFL-driven loop: dt = min(dt, t_end - t) (solver.py:384-417)."""
        U = U0.copy()
        t = float(t0)
        dt = self.compute_dt(U)
        dts = []
        n = 0
        while t < t_end - 1e-12:
            if max_steps is not None and n >= max_steps:
                break
            dt = min(dt, t_end - t)
            U = self.step(U, dt)
            t += dt
            dts.append(dt)
            dt = self.compute_dt(U)
            n += 1
        return U, t, dts
