"""Initial conditions of the reference's registered problems, built on the host
in NumPy from the reference's own configuration keys and defaults.

Each builder takes the grid's node coordinates (NumPy arrays, as the grid
objects hold them) and the problem's config dict and returns the conservative
state in the reference's component-first layout.  Citations are the
reference's files (phrike/problems/problem_list/*.py).  The builders restate
the published formulas, including the reference's quirks (the
``meshgrid(..., indexing='ij')`` of the 2D Gaussian waves, the float32
velocity of the turbulence generator, the hydrostatic pressure integrations),
so that a config written for the reference produces the same initial state.
"""
from __future__ import annotations

from typing import Any, Dict, Optional, Sequence, Tuple

import numpy as np


def _euler(rho, vel: Sequence[np.ndarray], p, gamma: float) -> np.ndarray:
    """EulerEquations{1,2,3}D.conservative (equations.py:255-278, 321-325, 569-580)."""
    E = p / (gamma - 1.0) + 0.5 * rho * sum(v * v for v in vel)
    return np.array([rho] + [rho * v for v in vel] + [E])


def _mhd(rho, ux, uy, uz, p, Bx, By, Bz, gamma: float) -> np.ndarray:
    """MHDEquations*.conservative (equations.py:690-700, 798-810, 940-950)."""
    E = p / (gamma - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    return np.array([rho, rho * ux, rho * uy, rho * uz, E, Bx, By, Bz])


def _ic(cfg: Dict[str, Any]) -> Dict[str, Any]:
    return cfg.get("initial_conditions", {}) or {}


def ic_smoothing(cfg: Dict[str, Any], rho, u, p, n: int, length: float):
    """BaseProblem.apply_initial_conditions_smoothing for 1D grids
    (problems/base.py:1183-1260, config 156-166): Gaussian smoothing with
    sigma = kernel_size * N / Lx grid points and the configured edge mode."""
    raw = cfg.get("initial_conditions_smoothing", None)
    if not raw or not bool(raw.get("enabled", False)):
        return rho, u, p
    kernel = float(raw.get("kernel_size", 0.0))
    if kernel <= 0:
        return rho, u, p
    from scipy import ndimage
    mode = str(raw.get("mode", "wrap"))
    variables = raw.get("variables", ["density", "velocity", "pressure"])
    sigma = kernel * n / length
    rho_s, u_s, p_s = rho.copy(), u.copy(), p.copy()
    if "density" in variables:
        rho_s = ndimage.gaussian_filter1d(rho, sigma=sigma, mode=mode)
    if "velocity" in variables:
        u_s = ndimage.gaussian_filter1d(u, sigma=sigma, mode=mode)
    if "pressure" in variables:
        p_s = ndimage.gaussian_filter1d(p, sigma=sigma, mode=mode)
    return rho_s, u_s, p_s


# ---------------------------------------------------------------------------
# 1D
# ---------------------------------------------------------------------------

def sod(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """SodProblem (sod.py:18-47, 94-167): left/right states split at
    grid.x0 (default Lx/2); with initial_conditions.smoothing {enabled, sigma}
    a tanh step of width sigma; then the optional Gaussian IC smoothing."""
    g = cfg.get("grid", {}) or {}
    x0 = float(g.get("x0", 0.5 * Lx))
    ic = _ic(cfg)
    left, right = ic["left"], ic["right"]
    sm = ic.get("smoothing", {}) if isinstance(ic, dict) else {}
    sigma = float(sm.get("sigma", 0.0))
    if bool(sm.get("enabled", False)) and sigma > 0.0:
        step = 0.5 * (1.0 + np.tanh((x0 - x) / sigma))
        q = {k: float(right[k]) + (float(left[k]) - float(right[k])) * step for k in ("rho", "u", "p")}
        rho, u, p = q["rho"], q["u"], q["p"]
    else:
        rho = np.where(x < x0, left["rho"], right["rho"]).astype(np.float64)
        u = np.where(x < x0, left["u"], right["u"]).astype(np.float64)
        p = np.where(x < x0, left["p"], right["p"]).astype(np.float64)
    raw = cfg.get("initial_conditions_smoothing", None)
    if raw and bool(raw.get("enabled", False)):
        # primitive round trip of the conservative state (sod.py:143-148)
        U = _euler(rho, [u], p, gamma)
        rho = U[0]
        u = U[1] / rho
        p = (gamma - 1.0) * (U[2] - 0.5 * rho * u * u)
        rho, u, p = ic_smoothing(cfg, rho, u, p, len(x), Lx)
    return _euler(rho, [u], p, gamma)


def acoustic1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """Acoustic1DProblem (acoustic1d.py:27-49, 104-123):
    rho = rho0 (1 + amplitude sin(2 pi k x / Lx)), uniform u0 and p0."""
    ic = _ic(cfg)
    rho0, u0, p0 = float(ic.get("rho0", 1.0)), float(ic.get("u0", 0.0)), float(ic.get("p0", 1.0))
    amp, k = float(ic.get("amplitude", 1e-3)), int(ic.get("k", 1))
    rho = rho0 * (1.0 + amp * np.sin(2.0 * np.pi * k * x / Lx))
    return _euler(rho, [u0 * np.ones_like(x)], p0 * np.ones_like(x), gamma)


def gaussian_wave1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """GaussianWave1DProblem (gaussian_wave1d.py:71-121): a Gaussian
    acoustic packet with the linear relations dp = c^2 drho, du = -c drho/rho0
    on a background u0 ("traveling") or c ("stationary")."""
    ic = _ic(cfg)
    rho0, u0, p0 = float(ic.get("rho0", 1.0)), float(ic.get("u0", 0.0)), float(ic.get("p0", 1.0))
    amp, sigma = float(ic.get("amplitude", 0.1)), float(ic.get("sigma", 0.1))
    x0 = float(ic.get("x0", Lx / 2.0))
    gauss = amp * np.exp(-((x - x0) ** 2) / (2.0 * sigma ** 2))
    cs = np.sqrt(gamma * p0 / rho0)
    ub = cs if ic.get("wave_type", "traveling") == "stationary" else u0
    rho = rho0 + gauss
    u = ub + (-cs * gauss / rho0)
    p = p0 + cs ** 2 * gauss
    return _euler(rho, [u], p, gamma)


def shu_osher1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """ShuOsher1DProblem (shu_osher1d.py:31-59, 113-146): the post-shock state
    (3.857143, 2.629369, 10.33333) for x < 0.5, rho = 1 + 0.2 sin(2 pi x),
    u = 0, p = 1 beyond; then the optional Gaussian IC smoothing."""
    rho = np.where(x < 0.5, 3.857143, 1.0 + 0.2 * np.sin(2.0 * np.pi * x))
    u = np.where(x < 0.5, 2.629369, 0.0)
    p = np.where(x < 0.5, 10.33333, 1.0)
    rho, u, p = ic_smoothing(cfg, rho.astype(np.float64), u.astype(np.float64), p.astype(np.float64), len(x), Lx)
    return _euler(rho, [u], p, gamma)


def hse_1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """HSE1DProblem (hse_1d.py:15-93, 146-179): tanh density step at grid.x0
    of width initial_conditions.smoothing.sigma, u = 0, and the pressure
    integrated from p_left with the trapezoid density and gx (gravity block,
    when enabled)."""
    ic = _ic(cfg)
    rl, rr, pl = float(ic["left"]["rho"]), float(ic["right"]["rho"]), float(ic["left"]["p"])
    grav = cfg.get("gravity", {}) or {}
    gx = float(grav.get("gx", 0.0)) if bool(grav.get("enabled", False)) else 0.0
    x0 = float((cfg.get("grid", {}) or {}).get("x0", 0.5 * Lx))
    sigma = float((ic.get("smoothing", {}) or {}).get("sigma", 0.01))
    step = 0.5 * (1.0 + np.tanh((x0 - x) / sigma))
    rho = rr + (rl - rr) * step
    p = np.zeros_like(x)
    p[0] = pl
    dx = x[1] - x[0]
    for j in range(1, len(x)):
        p[j] = p[j - 1] + 0.5 * (rho[j - 1] + rho[j]) * gx * dx
    return _euler(rho, [np.zeros_like(x)], p, gamma)


def rti_1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """RTI1DProblem (rti_1d.py:25-149 and its create_initial_conditions):
    tanh interface at the middle of the domain (heavy fluid above), velocity
    perturbation A sin(2 pi x / lambda) exp(-(x - xi)^2 / (2 w^2)), pressure
    integrated downward from pressure_top with the trapezoid density and gx."""
    ic = _ic(cfg)
    rh, rl = float(ic.get("rho_heavy", 2.0)), float(ic.get("rho_light", 1.0))
    ptop = float(ic.get("pressure_top", 2.5))
    amp, lam = float(ic.get("perturb_amplitude", 0.01)), float(ic.get("perturb_wavelength", 1.0))
    w = float(ic.get("interface_thickness", 0.05))
    grav = cfg.get("gravity", None)
    g = float(grav.get("gx", 1.0)) if grav and bool(grav.get("enabled", False)) else 0.0
    xi = float(np.min(x)) + 0.5 * (float(np.max(x)) - float(np.min(x)))
    xc = x - xi
    rho = rl + 0.5 * (rh - rl) * (1.0 + np.tanh(xc / w))
    u = amp * np.sin(2.0 * np.pi * x / lam) * np.exp(-0.5 * (xc / w) ** 2)
    p = np.zeros(len(x), dtype=x.dtype)
    p[-1] = ptop
    dxl = np.diff(x)
    for i in range(len(x) - 2, -1, -1):
        p[i] = p[i + 1] - 0.5 * (rho[i] + rho[i + 1]) * g * dxl[i]
    return _euler(rho, [u], p, gamma)


def _alfven_params(cfg: Dict[str, Any]) -> Dict[str, Any]:
    """Alfven1DProblem._ic_params (alfven1d.py:88-97)."""
    ic = _ic(cfg)
    return dict(rho0=float(ic.get("rho0", 1.0)), p0=float(ic.get("p0", 0.1)), B0=float(ic.get("B0", 1.0)),
                b1=float(ic.get("b1", 0.1)), m=int(ic.get("m", 1)), direction=int(ic.get("direction", 1)))


def _alfven(X: np.ndarray, Lx: float, gamma: float, rho0, p0, B0, b1, m, direction) -> np.ndarray:
    """Circularly polarized Alfven wave at t = 0 (alfven1d.py:32-82,
    alfven3d.py:23-47)."""
    k = 2.0 * np.pi * m / Lx
    phi = k * X
    By, Bz = b1 * np.cos(phi), b1 * np.sin(phi)
    inv = 1.0 / np.sqrt(rho0)
    sign = float(direction)
    return _mhd(np.full_like(X, float(rho0)), np.zeros_like(X), -sign * By * inv, -sign * Bz * inv,
                np.full_like(X, float(p0)), np.full_like(X, float(B0)), By, Bz, gamma)


def alfven1d(x: np.ndarray, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """Alfven1DProblem (alfven1d.py:116-119)."""
    return _alfven(x, Lx, gamma, **_alfven_params(cfg))


# ---------------------------------------------------------------------------
# 2D (X, Y: meshes of shape (Ny, Nx), indexing "xy")
# ---------------------------------------------------------------------------

def khi2d(X: np.ndarray, Y: np.ndarray, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """KHI2DProblem (khi2d.py:16-117, 149-177): two tanh shear layers at
    y/Ly = 0.25 and 0.75 of thickness a, outer/inner density and pressure,
    ux = -u0/2 outside and +u0/2 inside, and a vy perturbation
    eps sin(2 pi kx x / Lx) times Gaussians of width sigma at the layers.
    Lx and Ly are the extents of the node coordinates (max - min)."""
    ic = _ic(cfg)
    ro, ri = float(ic.get("rho_outer", 1.0)), float(ic.get("rho_inner", 2.0))
    u0, a = float(ic.get("u0", 1.0)), float(ic.get("shear_thickness", 0.02))
    po, pi_ = float(ic.get("pressure_outer", 1.0)), float(ic.get("pressure_inner", 1.0))
    eps, sig = float(ic.get("perturb_eps", 0.01)), float(ic.get("perturb_sigma", 0.02))
    kx = int(ic.get("perturb_kx", 2))
    Lx, Ly = X.max() - X.min(), Y.max() - Y.min()
    yn = Y / Ly
    prof = np.tanh((yn - 0.25) / a) - np.tanh((yn - 0.75) / a)
    U1, U2 = -0.5 * u0, 0.5 * u0
    ux = U1 + 0.5 * (U2 - U1) * prof
    rho = ro + 0.5 * (ri - ro) * prof
    p = po + 0.5 * (pi_ - po) * prof
    gauss = np.exp(-((yn - 0.25) ** 2) / (2.0 * sig * sig)) + np.exp(-((yn - 0.75) ** 2) / (2.0 * sig * sig))
    uy = eps * np.sin(2.0 * np.pi * kx * X / Lx) * gauss
    return _euler(rho, [ux, uy], p, gamma)


def uniform_2d(X: np.ndarray, Y: np.ndarray, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """Uniform2DProblem (uniform2d.py:14-35, 72-77): rho, p from the config, at rest."""
    ic = _ic(cfg)
    rho = np.full_like(X, float(ic.get("rho", 1.0)))
    p = np.full_like(X, float(ic.get("p", 1.0)))
    return _euler(rho, [np.zeros_like(X), np.zeros_like(X)], p, gamma)


def rti(X: np.ndarray, Y: np.ndarray, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """RTIProblem (rti.py:25-159, 231-266): tanh interface at mid-height
    (heavy above), vy = A sin(2 pi x / lambda) exp(-(y - yi)^2 / (2 w^2)),
    pressure integrated downward from pressure_top with the gravity block's
    gy (when enabled) and the trapezoid density of the first column."""
    ic = _ic(cfg)
    rh, rl = float(ic.get("rho_heavy", 2.0)), float(ic.get("rho_light", 1.0))
    ptop = float(ic.get("pressure_top", 2.5))
    amp, lam = float(ic.get("perturb_amplitude", 0.01)), float(ic.get("perturb_wavelength", 1.0))
    w = float(ic.get("interface_thickness", 0.05))
    grav = cfg.get("gravity", None)
    g = float(grav.get("gy", 1.0)) if grav and bool(grav.get("enabled", False)) else 0.0
    yi = float(np.min(Y)) + 0.5 * (float(np.max(Y)) - float(np.min(Y)))
    yc = Y - yi
    rho = rl + 0.5 * (rh - rl) * (1.0 + np.tanh(yc / w))
    u = np.zeros_like(X)
    v = amp * np.sin(2.0 * np.pi * X / lam) * np.exp(-0.5 * (yc / w) ** 2)
    ny, nx = Y.shape
    yl, rhol = Y[:, 0], rho[:, 0]
    dyl = np.diff(yl)
    pl = np.zeros(ny, dtype=X.dtype)
    pl[-1] = ptop
    for j in range(ny - 2, -1, -1):
        pl[j] = pl[j + 1] - 0.5 * (rhol[j] + rhol[j + 1]) * g * dyl[j]
    p = np.repeat(pl[:, None], nx, axis=1)
    return _euler(rho, [u, v], p, gamma)


def gaussian_wave2d(x: np.ndarray, y: np.ndarray, cfg: Dict[str, Any], gamma: float,
                    legendre: bool) -> np.ndarray:
    """GaussianWave2DProblem (gaussian_wave2d.py:68-135): a Gaussian acoustic
    packet at (x0, y0) with width 1.58 sigma on Legendre grids (at the domain
    centre with width sigma otherwise), travelling along the configured
    angle.  The reference builds its meshes with indexing='ij', so the
    arrays are (Nx, Ny); kept as it is."""
    ic = _ic(cfg)
    rho0, u0, v0, p0 = (float(ic.get(k, d)) for k, d in (("rho0", 1.0), ("u0", 0.0), ("v0", 0.0), ("p0", 1.0)))
    amp, sigma = float(ic.get("amplitude", 0.1)), float(ic.get("sigma", 0.05))
    x0, y0 = float(ic.get("x0", 0.5)), float(ic.get("y0", 0.5))
    angle = float(ic.get("angle", 45.0))
    ar = np.pi * angle / 180.0
    X, Y = np.meshgrid(x, y, indexing="ij")
    if legendre:
        cx, cy, es = x0, y0, sigma * 1.58
    else:
        cx, cy, es = x.max() / 2.0, y.max() / 2.0, sigma
    gauss = amp * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * es ** 2))
    cs = np.sqrt(gamma * p0 / rho0)
    if angle == 0.0 and u0 == 0.0 and v0 == 0.0:
        du, dv = np.zeros_like(gauss), np.zeros_like(gauss)
    else:
        nx, ny = -np.cos(ar), np.sin(ar)
        du, dv = -cs * nx * gauss / rho0, -cs * ny * gauss / rho0
    return _euler(rho0 + gauss, [u0 + du, v0 + dv], p0 + cs ** 2 * gauss, gamma)


def gaussian_wave2d_y(x: np.ndarray, y: np.ndarray, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """GaussianWave2DYProblem (gaussian_wave2d_y.py:46-96): a Gaussian packet
    in y, repeated along x, travelling up or down."""
    ic = _ic(cfg)
    rho0, u0, v0, p0 = (float(ic.get(k, d)) for k, d in (("rho0", 1.0), ("u0", 0.0), ("v0", 0.0), ("p0", 1.0)))
    amp, sigma, y0 = float(ic.get("amplitude", 0.1)), float(ic.get("sigma", 0.05)), float(ic.get("y0", 0.5))
    ny = 1.0 if ic.get("direction", "up") == "up" else -1.0
    gy = amp * np.exp(-((y - y0) ** 2) / (2.0 * sigma ** 2))
    g2 = np.tile(gy, (len(x), 1)).T
    cs = np.sqrt(gamma * p0 / rho0)
    return _euler(rho0 + g2, [u0 + np.zeros_like(g2), v0 - cs * ny * g2 / rho0], p0 + cs ** 2 * g2, gamma)


def orszag_tang2d(X: np.ndarray, Y: np.ndarray, Lx: float, Ly: float, cfg: Dict[str, Any],
                  gamma: float) -> np.ndarray:
    """OrszagTang2DProblem (orszag_tang2d.py:33-66, 91-97): uniform rho0, p0
    (defaults 25/(36 pi), 5/(12 pi)), u = (-sin ky y, sin kx x),
    B = B0 (-sin ky y, sin 2 kx x), B0 default 1/sqrt(4 pi)."""
    ic = _ic(cfg)
    rho0, p0, B0 = ic.get("rho0"), ic.get("p0"), ic.get("B0")
    rho0 = 25.0 / (36.0 * np.pi) if rho0 is None else float(rho0)
    p0 = 5.0 / (12.0 * np.pi) if p0 is None else float(p0)
    B0 = 1.0 / np.sqrt(4.0 * np.pi) if B0 is None else float(B0)
    kx, ky = 2.0 * np.pi / Lx, 2.0 * np.pi / Ly
    z = np.zeros_like(X)
    return _mhd(np.full_like(X, rho0), -np.sin(ky * Y), np.sin(kx * X), z, np.full_like(X, p0),
                -B0 * np.sin(ky * Y), B0 * np.sin(2.0 * kx * X), z, gamma)


# ---------------------------------------------------------------------------
# 3D (X, Y, Z: meshes of shape (Nz, Ny, Nx))
# ---------------------------------------------------------------------------

def tgv3d(X, Y, Z, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """TGV3DProblem (tgv3d.py:18-66, 100-112): u = U0 sin kx cos ky cos kz,
    v = -U0 cos kx sin ky cos kz, w = 0, uniform rho0 and p0 (default 100),
    k from the config (default 2)."""
    ic = _ic(cfg)
    rho0, p0, U0 = float(ic.get("rho0", 1.0)), float(ic.get("p0", 100.0)), float(ic.get("U0", 1.0))
    k = int(ic.get("k", 2))
    u = U0 * np.sin(k * X) * np.cos(k * Y) * np.cos(k * Z)
    v = -U0 * np.cos(k * X) * np.sin(k * Y) * np.cos(k * Z)
    return _euler(rho0 * np.ones_like(X), [u, v, np.zeros_like(X)], p0 * np.ones_like(X), gamma)


def _turbulent_velocity(n1: int, n2: int, n3: int, kmin: float, kmax: float, alpha: float, vrms: float,
                        rng, spectrum: str, slope: float):
    """build_turbulent_velocity of turbulent_velocity_3d (turb3d.py:66-172):
    three standard-normal fields, band-pass envelope (parabolic or power law
    with cosine tapers), mixture alpha of the compressive and solenoidal
    parts, float32 velocities scaled to the target rms."""
    u0 = rng.standard_normal((n1, n2, n3)).astype(np.float64)
    v0 = rng.standard_normal((n1, n2, n3)).astype(np.float64)
    w0 = rng.standard_normal((n1, n2, n3)).astype(np.float64)
    U, V, W = np.fft.fftn(u0), np.fft.fftn(v0), np.fft.fftn(w0)
    kx = np.fft.fftfreq(n1, d=1.0 / n1).reshape(n1, 1, 1)
    ky = np.fft.fftfreq(n2, d=1.0 / n2).reshape(1, n2, 1)
    kz = np.fft.fftfreq(n3, d=1.0 / n3).reshape(1, 1, n3)
    kmag = np.sqrt(kx * kx + ky * ky + kz * kz)
    with np.errstate(invalid="ignore"):
        band = (kmag >= kmin) & (kmag <= kmax)
        if spectrum == "parabolic":
            env = np.clip(np.where(band, (kmag - kmin) * (kmax - kmag), 0.0), 0.0, None)
        elif spectrum == "power_law":
            ks = np.where(kmag == 0.0, 1.0, kmag)
            env = np.where(band, ks ** slope, 0.0)
            dk = kmax - kmin
            k1, k2 = kmin + 0.1 * dk, kmax - 0.1 * dk
            lo = np.where((kmag >= kmin) & (kmag < k1), 0.5 * (1.0 + np.cos(np.pi * (kmag - kmin) / (k1 - kmin))), 1.0)
            hi = np.where((kmag > k2) & (kmag <= kmax), 0.5 * (1.0 + np.cos(np.pi * (kmag - k2) / (kmax - k2))), 1.0)
            env *= lo * hi
        else:
            raise ValueError(f"Unknown spectrum_type: {spectrum}")
        filt = np.sqrt(env, dtype=np.float64)
    ks = np.where(kmag == 0.0, 1.0, kmag)
    dot = kx * U + ky * V + kz * W
    par = [kx * dot / (ks * ks), ky * dot / (ks * ks), kz * dot / (ks * ks)]
    out = []
    for F, Fp in zip((U, V, W), par):
        Mx = (alpha * Fp + (1.0 - alpha) * (F - Fp)) * filt
        Mx[0, 0, 0] = 0.0
        out.append(np.fft.ifftn(Mx).real.astype(np.float32))
    u, v, w = out
    rms = float(np.sqrt(np.mean(u * u + v * v + w * w)))
    if rms > 0:
        s = float(vrms) / rms
        u *= s
        v *= s
        w *= s
    return u, v, w


def _turb_args(ic: Dict[str, Any]):
    return dict(kmin=float(ic.get("kmin", 2.0)), kmax=float(ic.get("kmax", 16.0)),
                alpha=float(ic.get("alpha", 0.3333)), vrms=float(ic.get("vrms", 0.1)),
                spectrum=str(ic.get("spectrum_type", "parabolic")))


def turb3d(X, Y, Z, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """Turb3DProblem (turb3d.py:18-192, 247-276).  The generator works on
    arrays of shape (Nx, Ny, Nz) taken from X.shape = (Nz, Ny, Nx), as the
    reference does (cubic grids line up)."""
    ic = _ic(cfg)
    nz, ny, nx = X.shape
    rng = np.random.default_rng(int(ic.get("seed", 42)))
    u, v, w = _turbulent_velocity(nx, ny, nz, rng=rng, slope=float(ic.get("power_law_slope", -5.0 / 3.0)),
                                  **_turb_args(ic))
    rho0, p0 = float(ic.get("rho0", 1.0)), float(ic.get("p0", 1.0))
    return _euler(rho0 * np.ones_like(X), [u, v, w], p0 * np.ones_like(X), gamma)


def alfven3d(X, Lx: float, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """Alfven3DProblem (alfven3d.py:23-47, 77-81): the wave along x."""
    return _alfven(X, Lx, gamma, **_alfven_params(cfg))


def _banded_random_b(nx: int, ny: int, nz: int, b_rms: float, kmin: float, kmax: float, b0, seed: int):
    """banded_random_b_3d (mhd_turb3d.py:25-66): divergence-free band-limited
    random field of rms b_rms plus the mean field b0, shape (Nz, Ny, Nx)."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, d=1.0 / nx).reshape(1, 1, nx)
    ky = np.fft.fftfreq(ny, d=1.0 / ny).reshape(1, ny, 1)
    kz = np.fft.fftfreq(nz, d=1.0 / nz).reshape(nz, 1, 1)
    kmag = np.sqrt(kx * kx + ky * ky + kz * kz)
    env = np.where((kmag >= kmin) & (kmag <= kmax), 1.0, 0.0)
    k2 = kx * kx + ky * ky + kz * kz
    k2s = np.where(k2 == 0.0, 1.0, k2)

    def field_hat():
        F = np.fft.fftn(rng.standard_normal((nz, ny, nx))) * env
        F[0, 0, 0] = 0.0
        return F

    Fx, Fy, Fz = field_hat(), field_hat(), field_hat()
    coef = (kx * Fx + ky * Fy + kz * Fz) / k2s
    Bx = np.fft.ifftn(Fx - kx * coef).real
    By = np.fft.ifftn(Fy - ky * coef).real
    Bz = np.fft.ifftn(Fz - kz * coef).real
    rms = float(np.sqrt(np.mean(Bx ** 2 + By ** 2 + Bz ** 2)))
    if rms > 0:
        s = float(b_rms) / rms
        Bx *= s
        By *= s
        Bz *= s
    return Bx + float(b0[0]), By + float(b0[1]), Bz + float(b0[2])


def mhd_turb3d(X, Y, Z, cfg: Dict[str, Any], gamma: float) -> np.ndarray:
    """MHDTurb3DProblem (mhd_turb3d.py:88-115): the Turb3D velocity (its
    default power-law slope) and a banded random B with mean field b0."""
    ic = _ic(cfg)
    nz, ny, nx = X.shape
    rng = np.random.default_rng(int(ic.get("seed", 42)))
    u, v, w = _turbulent_velocity(nx, ny, nz, rng=rng, slope=-5.0 / 3.0, **_turb_args(ic))
    rho0, p0 = float(ic.get("rho0", 1.0)), float(ic.get("p0", 1.0))
    Uh = _euler(rho0 * np.ones_like(X), [u, v, w], p0 * np.ones_like(X), gamma)
    rho = Uh[0]
    Bx, By, Bz = _banded_random_b(nx, ny, nz, float(ic.get("b_rms", 0.1)), float(ic.get("b_kmin", 1.0)),
                                  float(ic.get("b_kmax", 5.0)), tuple(ic.get("b0", [0.0, 0.0, 1.0])),
                                  int(ic.get("b_seed", 123)))
    return _mhd(rho, Uh[1] / rho, Uh[2] / rho, Uh[3] / rho, p0 * np.ones_like(rho), Bx, By, Bz, gamma)


# ---------------------------------------------------------------------------
# problem table: name -> (kind, default basis); kind is 1d, 1d_mhd, 2d,
# 2d_mhd, 3d or 3d_mhd (problems/register.py:24-40)
# ---------------------------------------------------------------------------
PROBLEMS: Dict[str, Tuple[str, str]] = {
    "sod": ("1d", "fourier"),
    "acoustic1d": ("1d", "fourier"),
    "gaussian_wave1d": ("1d", "fourier"),
    "shu_osher1d": ("1d", "fourier"),
    "hse_1d": ("1d", "fourier"),
    "rti_1d": ("1d", "legendre"),
    "alfven1d": ("1d_mhd", "fourier"),
    "khi2d": ("2d", "fourier"),
    "uniform_2d": ("2d", "legendre"),
    "rti": ("2d", "legendre"),
    "gaussian_wave2d": ("2d", "legendre"),
    "gaussian_wave2d_y": ("2d", "legendre"),
    "orszag_tang2d": ("2d_mhd", "fourier"),
    "tgv3d": ("3d", "fourier"),
    "turb3d": ("3d", "fourier"),
    "alfven3d": ("3d_mhd", "fourier"),
    "mhd_turb3d": ("3d_mhd", "fourier"),
}


def build(name: str, cfg: Dict[str, Any], gamma: float, x: np.ndarray, y: Optional[np.ndarray] = None,
          z: Optional[np.ndarray] = None, lengths: Sequence[float] = (), legendre: bool = False) -> np.ndarray:
    """Initial state of problem ``name`` on node coordinates x (, y, z) with
    the domain lengths (Lx, Ly, Lz) of the grid.  The coordinates keep their
    dtype: the reference's grids hold float32 nodes at single precision, and
    its hydrostatic integrations accumulate in the nodes' dtype."""
    x = np.asarray(x)
    L = list(lengths)
    one_d = {"sod": sod, "acoustic1d": acoustic1d, "gaussian_wave1d": gaussian_wave1d,
             "shu_osher1d": shu_osher1d, "hse_1d": hse_1d, "rti_1d": rti_1d, "alfven1d": alfven1d}
    if name in one_d:
        return one_d[name](x, L[0], cfg, gamma)
    y = np.asarray(y)
    if name == "gaussian_wave2d":
        return gaussian_wave2d(x, y, cfg, gamma, legendre)
    if name == "gaussian_wave2d_y":
        return gaussian_wave2d_y(x, y, cfg, gamma)
    if z is None:
        X, Y = np.meshgrid(x, y, indexing="xy")
        two_d = {"khi2d": khi2d, "uniform_2d": uniform_2d, "rti": rti}
        if name in two_d:
            return two_d[name](X, Y, cfg, gamma)
        if name == "orszag_tang2d":
            return orszag_tang2d(X, Y, L[0], L[1], cfg, gamma)
        raise ValueError(f"unknown 2D problem {name!r}")
    z = np.asarray(z)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    if name == "tgv3d":
        return tgv3d(X, Y, Z, cfg, gamma)
    if name == "turb3d":
        return turb3d(X, Y, Z, cfg, gamma)
    if name == "alfven3d":
        return alfven3d(X, L[0], cfg, gamma)
    if name == "mhd_turb3d":
        return mhd_turb3d(X, Y, Z, cfg, gamma)
    raise ValueError(f"unknown 3D problem {name!r}")
