"""Grids with the reference's constructor signatures and operators, backed
by the CUDA engine (backend "gb300"): periodic Fourier grids in 1-3D and the
2D LGL x LGL (Legendre-Gauss-Lobatto) grid with solid walls.

Mirrors phrike/grid.py: Grid1D (lines 144-735), Grid2D (775-1354) and
Grid3D (1357-1744).  Arrays are float32 torch tensors on the grid's CUDA
device, component-first with spatial axes (..., [Nz,] [Ny,] Nx).  NumPy
inputs are moved to the device on entry.  Attributes keep the reference's
names and values (x, y, z, dx, dy, dz, k*, dealias_mask, filter_sigma).
"""
from __future__ import annotations

from typing import Any, Dict, Optional, Tuple

import numpy as np
import torch

from .engine import Plan, lgl_build


def _fftfreq_k(n: int, length: float) -> np.ndarray:
    return 2.0 * np.pi * np.fft.fftfreq(n, d=length / n)


def _mask_1d(n: int, dealias: bool) -> np.ndarray:
    if not dealias:
        return np.ones(n)
    k = np.fft.fftfreq(n) * n
    return (np.abs(k) <= n // 3).astype(float)


def _sigma_1d(n: int, fp: Optional[Dict]) -> np.ndarray:
    if not (fp and bool(fp.get("enabled", False))):
        return np.ones(n)
    p = int(fp.get("p", 8))
    alpha = float(fp.get("alpha", 36.0))
    k = np.fft.fftfreq(n) * n
    kmax = np.max(np.abs(k)) if n > 0 else 1.0
    return np.exp(-alpha * (np.abs(k) / max(kmax, 1.0)) ** p)


def _check_backend(backend: str, basis: str = "fourier") -> None:
    if str(backend).lower() != "gb300":
        raise ValueError(f"phrike_gb300 grids implement backend 'gb300' only (got {backend!r})")
    if str(basis).lower() != "fourier":
        raise ValueError(f"Unknown or unsupported basis for the gb300 Fourier grids: {basis!r}")


def _bc_codes_1d(bc: Any) -> list:
    """Boundary codes of a 1D Legendre grid, [side (left, right)] x [variable
    (density, momentum, energy)] flattened: 0 copy the neighbouring interior
    value, 1 zero, 2 leave.  Resolves a string, a per-variable or a
    per-boundary dict like Grid1D (grid.py:184-246, 620-735): "wall" (aliases
    reflective, dirichlet) zeroes the momentum and copies density and energy;
    "neumann" (alias open) copies every variable."""
    def norm_bc(v):
        n = str(v).strip().lower()
        return "wall" if n in ("reflective", "dirichlet", "wall") else "neumann" if n in ("neumann", "open") else n

    def norm_var(v):
        n = str(v).strip().lower()
        return {"rho": "density", "density": "density", "p": "pressure", "pressure": "pressure", "u": "momentum",
                "velocity": "momentum", "mom": "momentum", "momentum": "momentum",
                "momentum_x": "momentum"}.get(n, n)

    def norm_side(b):
        n = str(b).strip().lower()
        return "left" if n in ("left", "x0", "x_min", "start") else "right" if n in ("right", "x1", "x_max", "end") \
            else n

    glob, var_map, side_map = None, None, None
    if isinstance(bc, dict):
        if any(str(k).lower() in ("left", "right", "x0", "x1", "x_min", "x_max", "start", "end") for k in bc):
            side_map = {}
            for bk, vd in bc.items():
                if isinstance(vd, dict):
                    side_map[norm_side(bk)] = {norm_var(k): norm_bc(v) for k, v in vd.items()}
                else:
                    side_map[norm_side(bk)] = {v: norm_bc(vd) for v in ("density", "momentum", "pressure")}
        else:
            var_map = {norm_var(k): norm_bc(v) for k, v in bc.items()}
    elif isinstance(bc, str) and bc:
        glob = norm_bc(bc)

    def get(var, side):
        if side_map is not None and side in side_map:
            return side_map[side].get(var, glob or "wall")
        if var_map is not None:
            return var_map.get(var, glob or "wall")
        g = glob or "wall"
        if g == "wall":
            return "wall" if var == "momentum" else "neumann"
        return g

    codes = []
    for side in ("left", "right"):
        for var in ("density", "momentum", "pressure"):
            b = get(var, side)
            if var == "momentum":
                codes.append(1 if b in ("wall", "reflective") else 0 if b in ("neumann", "open") else 2)
            else:
                codes.append(0 if b in ("neumann", "open", "wall") else 2)
    return codes


def _is_lgl2d(basis_x: str, basis_y: str) -> bool:
    bx, by = str(basis_x).lower(), str(basis_y).lower()
    if bx == "legendre" and by == "legendre":
        return True
    if "legendre" in (bx, by):
        raise ValueError("backend 'gb300' supports Legendre on both axes (LGL x LGL) or Fourier on both, "
                         f"not a hybrid (got basis_x={basis_x!r}, basis_y={basis_y!r})")
    return False


class _FourierGridBase:
    """Shared device plumbing: the plan, tensor conversion, operators."""

    _shape: Tuple[int, ...]
    _lengths: Tuple[float, ...]

    _basis = "fourier"
    gemm_precision = "fp32"

    def _init_plan(self, dealias: bool, filter_params: Optional[Dict], torch_device: Optional[str],
                   precision: str, gamma: float = 1.4) -> None:
        if precision not in ("single", "double"):
            raise ValueError(f"precision must be 'single' or 'double' (got {precision!r})")
        # the engine computes in float32 whatever the requested precision
        self.precision = precision
        dev = torch.device(torch_device if torch_device else "cuda")
        if dev.type != "cuda":
            raise RuntimeError("backend 'gb300' runs on a CUDA device only")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.torch_device = str(dev)
        self.device = dev
        self.filter_params = filter_params
        self.dealias = dealias
        self._gamma = gamma
        self._plans: Dict[float, Plan] = {}
        self.plan = self._plan_for(gamma)

    def _plan_for(self, gamma: float) -> Plan:
        g = float(gamma)
        if g not in self._plans:
            self._plans[g] = Plan(self._shape, self._lengths, gamma=g, dealias=self.dealias,
                                  filter_params=self.filter_params, device=self.device, basis=self._basis,
                                  gemm_precision=self.gemm_precision, lgl_bc1d=getattr(self, "_bc_codes", None))
        return self._plans[g]

    def to_device(self, f: Any) -> torch.Tensor:
        if isinstance(f, torch.Tensor):
            t = f
            if t.device != self.device or t.dtype != torch.float32:
                t = t.to(device=self.device, dtype=torch.float32)
        else:
            t = torch.as_tensor(np.asarray(f), dtype=torch.float32, device=self.device)
        return t.contiguous()

    def _op(self, f: Any, axis: int) -> torch.Tensor:
        t = self.to_device(f)
        shape = t.shape
        return self.plan.derivative(t.reshape((-1,) + self._shape), axis).reshape(shape)

    def laplacian(self, f: Any) -> torch.Tensor:
        """Masked spectral Laplacian Re IFFT(-|k|^2 m s FFT f) (grid.py:569-579,
        1329-1338, 1696-1703)."""
        if self._basis != "fourier":
            raise ValueError("laplacian requires a Fourier basis")
        t = self.to_device(f)
        shape = t.shape
        return self.plan.laplacian(t.reshape((-1,) + self._shape)).reshape(shape)

    def apply_spectral_filter(self, f: Any) -> torch.Tensor:
        t = self.to_device(f)
        shape = t.shape
        return self.plan.filter(t.reshape((-1,) + self._shape)).reshape(shape)

    def _eval_points(self, fields: list, coords: list) -> torch.Tensor:
        """Spectral interpolant (mask x filter) of 1..3 fields at points
        (ps_eval_points); returns (len(fields), P) float32."""
        if self._basis != "fourier":
            raise ValueError("point evaluation requires a Fourier basis")
        f = torch.stack([self.to_device(v).reshape(self._shape) for v in fields]).contiguous()
        pts = torch.stack([torch.as_tensor(c, dtype=torch.float64).reshape(-1).to(self.device) for c in coords])
        return self.plan.eval_points(f, pts.contiguous())

    def apply_boundary_conditions(self, U: Any, equations: Any = None) -> Any:
        """Periodic Fourier grids have no boundary conditions (grid.py:631-632,
        1087-1089); an LGL x LGL grid applies its solid walls in place to a
        float32 device tensor (grid.py:1072-1154) and returns it."""
        if self._basis != "legendre":
            return U
        t = self.to_device(U)
        shape = t.shape
        self.plan.apply_boundary_conditions_(t.reshape((-1,) + self._shape))
        if isinstance(U, torch.Tensor) and t.data_ptr() != U.data_ptr():
            U.copy_(t.reshape(U.shape).to(U.dtype))
            return U
        return t.reshape(shape)


class Grid1D(_FourierGridBase):
    """1D grid: periodic Fourier, or Legendre-Gauss-Lobatto nodes with boundary
    conditions (reference: phrike/grid.py:144-735)."""

    def __init__(self, N: int, Lx: float, basis: str = "fourier", bc: Optional[Any] = None,
                 dealias: bool = True, filter_params: Optional[Dict[str, float]] = None, fft_workers: int = 1,
                 backend: str = "gb300", torch_device: Optional[str] = None, precision: str = "single",
                 debug: bool = False, problem_config: Optional[Dict[str, Any]] = None, gemm_precision: str = "fp32"):
        self.N, self.Lx, self.basis, self.bc = int(N), float(Lx), basis, bc
        self.fft_workers, self.backend, self.debug, self.problem_config = fft_workers, backend, debug, problem_config
        self._shape = (self.N,)
        self._lengths = (self.Lx,)
        self.mhd_config: Optional[Dict[str, Any]] = None  # set by MHD problems (grid.mhd_config)
        if str(basis).lower() == "legendre":
            # LGL nodes on [0, Lx] (grid.py:276-300, basis/legendre.py:681-729); no
            # Fourier masks; bc as in apply_boundary_conditions (grid.py:620-735)
            if str(backend).lower() != "gb300":
                raise ValueError(f"phrike_gb300 grids implement backend 'gb300' only (got {backend!r})")
            self._basis = "legendre"
            self.gemm_precision = str(gemm_precision).lower()
            self._bc_codes = _bc_codes_1d(bc if bc is not None else "dirichlet")
            self._init_plan(dealias, filter_params, torch_device, precision)
            self.x, self.w, self.D = lgl_build(self.N, self.Lx, self.device)
            self.dx = float(torch.min(torch.diff(self.x)).item())
            self.dealias_mask = torch.ones(self.N, dtype=torch.float64, device=self.device)
            self.filter_sigma = torch.ones(self.N, dtype=torch.float64, device=self.device)
            self.k = self.ik = None
            return
        _check_backend(backend, basis)
        self.dx = self.Lx / self.N
        self._init_plan(dealias, filter_params, torch_device, precision)
        self.x = torch.linspace(0.0, self.Lx, self.N + 1, dtype=torch.float64)[:-1].to(self.device)
        self.k = torch.as_tensor(_fftfreq_k(self.N, self.Lx), device=self.device)
        self.ik = 1j * self.k
        self.dealias_mask = torch.as_tensor(_mask_1d(self.N, dealias), device=self.device)
        self.filter_sigma = torch.as_tensor(_sigma_1d(self.N, filter_params), device=self.device)

    def dx1(self, f: Any) -> torch.Tensor:
        return self._op(f, 0)

    def divergence_x(self, Bx: Any) -> torch.Tensor:
        """d(Bx)/dx with the masked derivative (grid.py:550-552)."""
        return self.dx1(Bx)

    def evaluate_fourier_at_points_1d(self, f: Any, xp: Any) -> torch.Tensor:
        """f at arbitrary points through its masked, filtered Fourier series
        (grid.py:581-618)."""
        return self._eval_points([f], [xp])[0]

    def project_solenoidal_x(self, Bx: Any) -> torch.Tensor:
        """The 1D Leray projection keeps only the mean of Bx (grid.py:554-567)."""
        t = self.to_device(Bx)
        return torch.full_like(t, float(t.double().mean().item()))


class Grid2D(_FourierGridBase):
    """2D periodic Fourier grid, spatial axes (Ny, Nx) (reference: phrike/grid.py:775-1354)."""

    def __init__(self, Nx: int, Ny: int, Lx: float, Ly: float, dealias: bool = True,
                 filter_params: Optional[Dict[str, float]] = None, fft_workers: int = 1,
                 backend: str = "gb300", torch_device: Optional[str] = None, precision: str = "single",
                 debug: bool = False, basis_x: str = "fourier", basis_y: str = "fourier",
                 bc: str = "dirichlet", bc_config: Optional[Dict[str, Any]] = None,
                 gemm_precision: str = "fp32"):
        lgl = _is_lgl2d(basis_x, basis_y)
        _check_backend(backend, "fourier")
        self.Nx, self.Ny, self.Lx, self.Ly = int(Nx), int(Ny), float(Lx), float(Ly)
        self.basis_x, self.basis_y, self.bc, self.bc_config = basis_x, basis_y, bc, bc_config
        self.fft_workers, self.backend, self.debug = fft_workers, backend, debug
        self._shape = (self.Ny, self.Nx)
        self._lengths = (self.Ly, self.Lx)
        self.dx, self.dy = self.Lx / self.Nx, self.Ly / self.Ny
        self.dx_min = None
        self.dy_min = None
        self.mhd_config: Optional[Dict[str, Any]] = None  # set by MHD problems (grid.mhd_config)
        self._mhd_plan: Optional[Plan] = None
        if lgl:
            self._init_lgl(dealias, filter_params, torch_device, precision, gemm_precision)
            return
        self._init_plan(dealias, filter_params, torch_device, precision)
        self.x = torch.as_tensor(np.linspace(0.0, self.Lx, self.Nx, endpoint=False), device=self.device)
        self.y = torch.as_tensor(np.linspace(0.0, self.Ly, self.Ny, endpoint=False), device=self.device)
        self.kx = torch.as_tensor(_fftfreq_k(self.Nx, self.Lx), device=self.device)
        self.ky = torch.as_tensor(_fftfreq_k(self.Ny, self.Ly), device=self.device)
        self.ikx = (1j * self.kx)[None, :]
        self.iky = (1j * self.ky)[:, None]
        mx, my = _mask_1d(self.Nx, dealias), _mask_1d(self.Ny, dealias)
        sx, sy = _sigma_1d(self.Nx, filter_params), _sigma_1d(self.Ny, filter_params)
        self.dealias_mask = torch.as_tensor(my[:, None] * mx[None, :], device=self.device)
        self.filter_sigma = torch.as_tensor(sy[:, None] * sx[None, :], device=self.device)

    def _init_lgl(self, dealias: bool, filter_params: Optional[Dict], torch_device: Optional[str],
                  precision: str, gemm_precision: str) -> None:
        """LGL x LGL grid (grid.py:806-840 with LegendreLobattoBasis2D,
        basis/legendre.py:894-934): nodes ascending on [0, L] per axis, solid
        walls for bc "dirichlet" (grid.py:994-1154)."""
        if self.bc_config:
            raise NotImplementedError("backend 'gb300': per-boundary bc_config maps are not implemented "
                                      "(LGL grids use solid walls)")
        if str(self.bc).lower() != "dirichlet":
            raise NotImplementedError(f"backend 'gb300': LGL grids support bc='dirichlet' (walls), got {self.bc!r}")
        self._basis = "legendre"
        self.gemm_precision = str(gemm_precision).lower()
        self._init_plan(dealias, filter_params, torch_device, precision)
        self.x, self.w_x, self.Dx = lgl_build(self.Nx, self.Lx, self.device)
        self.y, self.w_y, self.Dy = lgl_build(self.Ny, self.Ly, self.device)
        self.dx_min = float(torch.min(torch.diff(self.x)).item())
        self.dy_min = float(torch.min(torch.diff(self.y)).item())
        self.kx = self.ky = self.ikx = self.iky = None
        self.dealias_mask = None
        self.filter_sigma = None

    def dx1(self, f: Any) -> torch.Tensor:
        return self._op(f, 0)

    def dy1(self, f: Any) -> torch.Tensor:
        return self._op(f, 1)

    # --- MHD solenoidal helpers (grid.py:1290-1327) ---
    def divergence(self, Bx: Any, By: Any) -> torch.Tensor:
        """dx1(Bx) + dy1(By) with the masked derivative operators."""
        return self.dx1(Bx) + self.dy1(By)

    def project_solenoidal(self, Bx: Any, By: Any) -> Tuple[torch.Tensor, torch.Tensor]:
        """Helmholtz (Leray) projection of (Bx, By); returns new tensors."""
        if self._basis != "fourier":
            raise ValueError("project_solenoidal requires Fourier basis in x and y")
        if self._mhd_plan is None:
            self._mhd_plan = Plan(self._shape, self._lengths, dealias=self.dealias, filter_params=self.filter_params,
                                  device=self.device, equations="mhd")
        bx = self.to_device(Bx).clone()
        by = self.to_device(By).clone()
        self._mhd_plan.project_solenoidal_(bx, by)
        return bx, by

    def evaluate_fourier_at_points(self, f: Any, xp: Any, yp: Any) -> torch.Tensor:
        """f (Ny, Nx) at points (xp, yp) through its masked, filtered Fourier
        series (grid.py:1180-1222)."""
        return self._eval_points([f], [xp, yp])[0]

    def xy_mesh(self) -> Tuple[torch.Tensor, torch.Tensor]:
        Y, X = torch.meshgrid(self.y, self.x, indexing="ij")
        return X, Y


class Grid3D(_FourierGridBase):
    """3D periodic Fourier grid, spatial axes (Nz, Ny, Nx) (reference: phrike/grid.py:1357-1744)."""

    def __init__(self, Nx: int, Ny: int, Nz: int, Lx: float, Ly: float, Lz: float, dealias: bool = True,
                 filter_params: Optional[Dict[str, float]] = None, fft_workers: int = 1,
                 backend: str = "gb300", torch_device: Optional[str] = None, precision: str = "single",
                 debug: bool = False):
        _check_backend(backend)
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.Lx, self.Ly, self.Lz = float(Lx), float(Ly), float(Lz)
        self.fft_workers, self.backend, self.debug = fft_workers, backend, debug
        self._shape = (self.Nz, self.Ny, self.Nx)
        self._lengths = (self.Lz, self.Ly, self.Lx)
        self.dx, self.dy, self.dz = self.Lx / self.Nx, self.Ly / self.Ny, self.Lz / self.Nz
        self.mhd_config: Optional[Dict[str, Any]] = None  # set by MHD problems (grid.mhd_config)
        self._mhd_plan: Optional[Plan] = None
        self._init_plan(dealias, filter_params, torch_device, precision)
        self.x = torch.as_tensor(np.linspace(0.0, self.Lx, self.Nx, endpoint=False), device=self.device)
        self.y = torch.as_tensor(np.linspace(0.0, self.Ly, self.Ny, endpoint=False), device=self.device)
        self.z = torch.as_tensor(np.linspace(0.0, self.Lz, self.Nz, endpoint=False), device=self.device)
        self.kx = torch.as_tensor(_fftfreq_k(self.Nx, self.Lx), device=self.device)
        self.ky = torch.as_tensor(_fftfreq_k(self.Ny, self.Ly), device=self.device)
        self.kz = torch.as_tensor(_fftfreq_k(self.Nz, self.Lz), device=self.device)
        self.ikx = (1j * self.kx)[None, None, :]
        self.iky = (1j * self.ky)[None, :, None]
        self.ikz = (1j * self.kz)[:, None, None]
        m = [_mask_1d(n, dealias) for n in (self.Nz, self.Ny, self.Nx)]
        s = [_sigma_1d(n, filter_params) for n in (self.Nz, self.Ny, self.Nx)]
        self.dealias_mask = torch.as_tensor(m[0][:, None, None] * m[1][None, :, None] * m[2][None, None, :],
                                            device=self.device)
        self.filter_sigma = torch.as_tensor(s[0][:, None, None] * s[1][None, :, None] * s[2][None, None, :],
                                            device=self.device)

    def dx1(self, f: Any) -> torch.Tensor:
        return self._op(f, 0)

    def dy1(self, f: Any) -> torch.Tensor:
        return self._op(f, 1)

    def dz1(self, f: Any) -> torch.Tensor:
        return self._op(f, 2)

    # --- MHD solenoidal helpers (grid.py:1635-1703) ---
    def divergence(self, Vx: Any, Vy: Any, Vz: Any) -> torch.Tensor:
        """dx1(Vx) + dy1(Vy) + dz1(Vz) with the masked derivative operators."""
        return self.dx1(Vx) + self.dy1(Vy) + self.dz1(Vz)

    def project_solenoidal(self, Vx: Any, Vy: Any, Vz: Any) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """Helmholtz (Leray) projection of (Vx, Vy, Vz); returns new tensors
        (ps_project_solenoidal_3d)."""
        if self._mhd_plan is None:
            self._mhd_plan = Plan(self._shape, self._lengths, dealias=self.dealias, filter_params=self.filter_params,
                                  device=self.device, equations="mhd")
        v = [self.to_device(V).clone() for V in (Vx, Vy, Vz)]
        self._mhd_plan.project_solenoidal_3d_(*v)
        return v[0], v[1], v[2]

    def curl(self, Vx: Any, Vy: Any, Vz: Any) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """Curl with the masked derivatives (grid.py:1686-1694)."""
        return (self.dy1(Vz) - self.dz1(Vy), self.dz1(Vx) - self.dx1(Vz), self.dx1(Vy) - self.dy1(Vx))

    def evaluate_fourier_at_points(self, f: Any, xp: Any, yp: Any, zp: Any) -> torch.Tensor:
        """f (Nz, Ny, Nx) at points (xp, yp, zp) (grid.py:1520-1567)."""
        return self._eval_points([f], [xp, yp, zp])[0]

    def evaluate_fourier_at_points_batched_3d(self, fx: Any, fy: Any, fz: Any, xp: Any, yp: Any, zp: Any
                                              ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """Three fields at the same points in one sweep (grid.py:1569-1632)."""
        v = self._eval_points([fx, fy, fz], [xp, yp, zp])
        return v[0], v[1], v[2]

    def xyz_mesh(self) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        Z, Y, X = torch.meshgrid(self.z, self.y, self.x, indexing="ij")
        return X, Y, Z
