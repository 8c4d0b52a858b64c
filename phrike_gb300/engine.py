"""Thin torch-facing wrapper of one C-ABI plan (one solve on one GPU).

Tensors are handed over by device pointer on the caller's current CUDA
stream; the library never sees torch types.  State tensors are float32,
component-first, C-contiguous, shape (ncomp, [Nz,] [Ny,] Nx).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, Optional, Sequence

import torch

from . import _lib


def _stream(device: torch.device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def lgl_build(n: int, length: float, device: Optional[torch.device] = None):
    """LGL nodes (ascending on [0, length]), weights on [-1, 1] and the
    differentiation matrix of one axis, built on the device in float64
    (ps_lgl_build).  Returns three float64 device tensors."""
    lib = _lib.load()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    x = torch.empty(n, dtype=torch.float64, device=dev)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    D = torch.empty((n, n), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.ps_lgl_build(int(n), float(length), _ptr(x), _ptr(w), _ptr(D), _stream(dev)))
    return x, w, D


class Plan:
    """A batch of ``nsolve`` pseudo-spectral Euler solves of one grid
    (1-3 dimensions); ``nsolve=1`` is a single solve.

    ``shape`` is the spatial shape in array order ((N,), (Ny, Nx) or
    (Nz, Ny, Nx)); ``lengths`` follows the same order.  State tensors have
    shape (ncomp, *shape) for one solve and (nsolve, ncomp, *shape) for a batch.
    ``basis="legendre"`` makes a 2D LGL x LGL plan with solid walls;
    ``gemm_precision`` ("fp32", "fp64" or "bf16x3") sets the arithmetic of its
    differentiation-matrix contractions.
    """

    def __init__(self, shape: Sequence[int], lengths: Sequence[float], gamma: float = 1.4,
                 dealias: bool = True, filter_params: Optional[Dict] = None,
                 cfl: Optional[float] = None, gravity: Optional[Sequence[float]] = None,
                 device: Optional[torch.device] = None, nsolve: int = 1, basis: str = "fourier",
                 gemm_precision: str = "fp32", equations: str = "euler", mhd_config: Optional[Dict] = None,
                 av_config: Optional[Dict] = None, scheme: str = "rk4", lgl_bc1d: Optional[Sequence[int]] = None,
                 tile_cols: Optional[int] = None, umma_n_tile: Optional[int] = None):
        lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise RuntimeError("phrike_gb300 plans run on a CUDA device only")
        self.shape = tuple(int(n) for n in shape)
        self.ndim = len(self.shape)
        self.equations = str(equations).lower()
        if self.equations not in ("euler", "mhd"):
            raise ValueError(f"equations must be 'euler' or 'mhd' (got {equations!r})")
        self.ncomp = 8 if self.equations == "mhd" else self.ndim + 2
        desc = _lib.PlanDesc()
        _lib.check(lib.ps_plan_desc_init(C.byref(desc), self.ndim))
        xyz = list(reversed(self.shape))
        lxyz = list(reversed([float(L) for L in lengths]))
        for a in range(self.ndim):
            desc.n[a] = xyz[a]
            desc.length[a] = lxyz[a]
        basis = str(basis).lower()
        if basis not in ("fourier", "legendre"):
            raise ValueError(f"unknown basis {basis!r}")
        self.basis = basis
        for a in range(self.ndim):
            desc.basis[a] = _lib.PS_BASIS_LEGENDRE if basis == "legendre" else _lib.PS_BASIS_FOURIER
        if str(gemm_precision).lower() not in _lib.GEMM_PRECISIONS:
            raise ValueError(f"gemm_precision must be one of {sorted(_lib.GEMM_PRECISIONS)}")
        self.gemm_precision = str(gemm_precision).lower()
        desc.gemm_precision = _lib.GEMM_PRECISIONS[self.gemm_precision]
        if self.equations == "mhd":
            desc.equations = _lib.PS_EQ_MHD
            mc = mhd_config or {}
            desc.mhd_rho_min = float(mc.get("rho_min", 1e-10))
            desc.mhd_p_min = float(mc.get("p_min", 1e-12))
            desc.mhd_project_substages = 1 if bool(mc.get("project_each_substage", True)) else 0
            desc.mhd_divergence_clean = 0 if str(mc.get("divergence_clean", "projection")) == "none" else 1
            desc.mhd_resistivity = float(mc.get("resistivity", 0.0))
            desc.mhd_viscosity = float(mc.get("viscosity", 0.0))
            desc.mhd_cfl_diff = float(mc.get("cfl_diff", 1.0))
        if av_config and av_config.get("enabled", False):
            # ArtificialViscosityConfig fields and defaults (artificial_viscosity.py:37-105)
            mode = str(av_config.get("mode", "sensor")).lower().strip()
            if mode not in ("sensor", "constant"):
                raise ValueError(f"Invalid mode '{mode}'. Must be 'sensor' or 'constant'")
            desc.av_mode = _lib.PS_AV_SENSOR if mode == "sensor" else _lib.PS_AV_CONSTANT
            sensors = {"density": _lib.PS_AV_Q_DENSITY, "pressure": _lib.PS_AV_Q_PRESSURE,
                       "velocity_magnitude": _lib.PS_AV_Q_SPEED}
            var = av_config.get("sensor_variable", "density")
            if var not in sensors:
                raise ValueError(f"Unknown sensor variable: {var}")
            if var == "velocity_magnitude" and mode == "sensor" and self.ndim == 2:
                # the reference's 2D sensor unpacks primitive() as (rho, u, p, _), takes
                # sqrt(u[0]^2 + u[1]^2) of the first two rows of u_x (a 1D array) and
                # its 2D FFT raises (artificial_viscosity.py:133-139, 169-190)
                raise ValueError("velocity_magnitude sensor on a 2D grid: axes exceeds dimensionality of input")
            desc.av_sensor = sensors[var]
            nu_c = float(av_config.get("nu_constant", 0.0))
            if mode == "constant" and nu_c < 0:
                raise ValueError("nu_constant must be non-negative")
            desc.av_nu_max = float(av_config.get("nu_max", 1e-3))
            desc.av_nu_constant = nu_c if nu_c != 0.0 else desc.av_nu_max
            desc.av_s_ref = float(av_config.get("s_ref", 1.0))
            desc.av_s_min = float(av_config.get("s_min", 0.1))
            desc.av_p = float(av_config.get("p", 2.0))
            desc.av_epsilon = float(av_config.get("epsilon", 1e-12))
            # weights by position in the reference's fixed name list
            names = ["density", "momentum_x", "momentum_y", "momentum_z", "energy"]
            wts = av_config.get("variable_weights", None) or {}
            for c in range(5):
                desc.av_weight[c] = float(wts.get(names[c], 1.0))
        if tile_cols is not None:  # 2D strided-pass tile width (ps_plan_desc.tile_cols; autotune.py)
            desc.tile_cols = int(tile_cols)
        if umma_n_tile is not None:  # N tile of the tcgen05 LGL contractions (autotune.py)
            desc.umma_n_tile = int(umma_n_tile)
        if lgl_bc1d is not None:  # 1D Legendre boundary codes (ps_plan_desc.lgl_bc1d)
            for i, c in enumerate(lgl_bc1d):
                desc.lgl_bc1d[i] = int(c)
        scheme = str(scheme).lower()
        if scheme not in ("rk4", "rk2"):
            raise ValueError(f"fixed-step scheme must be 'rk4' or 'rk2' (got {scheme!r})")
        self.scheme = scheme
        desc.scheme = _lib.PS_SCHEME_RK2 if scheme == "rk2" else _lib.PS_SCHEME_RK4
        desc.gamma = float(gamma)
        desc.dealias = 1 if dealias else 0
        fp = filter_params or {}
        desc.filter_enabled = 1 if bool(fp.get("enabled", False)) else 0
        desc.filter_p = int(fp.get("p", 8))
        desc.filter_alpha = float(fp.get("alpha", 36.0))
        desc.filter_interval = max(1, int(fp.get("interval", 1) or 1))
        if cfl is not None:
            desc.cfl = float(cfl)
        if gravity is not None:
            for a, g in enumerate(gravity):
                desc.gravity[a] = float(g)
        self.desc = desc
        self.nsolve = int(nsolve)
        self._handle = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.ps_batch_create(C.byref(desc), self.nsolve, C.byref(self._handle)))
        self._lib = lib

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_handle", None) and self._handle.value:
            with torch.cuda.device(self.device):
                self._lib.ps_plan_destroy(self._handle)
            self._handle = C.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    # -- helpers ----------------------------------------------------------
    def _check_state(self, U: torch.Tensor, nf: Optional[int] = None) -> None:
        nf = self.ncomp if nf is None else nf
        if not isinstance(U, torch.Tensor) or U.device != self.device:
            raise RuntimeError(f"expected a tensor on {self.device}")
        if U.dtype != torch.float32:
            raise RuntimeError(f"expected float32 fields, got {U.dtype}")
        if not U.is_contiguous():
            raise RuntimeError("fields must be C-contiguous")
        if tuple(U.shape[-self.ndim:]) != self.shape or U.numel() != nf * self.cells * self.nsolve:
            raise RuntimeError(f"expected {self.nsolve} solve(s) x {nf} fields of {self.shape}, got {tuple(U.shape)}")

    @property
    def cells(self) -> int:
        c = 1
        for n in self.shape:
            c *= n
        return c

    def scratch_bytes(self) -> int:
        b = C.c_size_t()
        _lib.check(self._lib.ps_batch_scratch_bytes(C.byref(self.desc), self.nsolve, C.byref(b)))
        return int(b.value)

    # -- operations -------------------------------------------------------
    def rhs(self, U: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        self._check_state(U)
        out = torch.empty_like(U) if out is None else out
        _lib.check(self._lib.ps_rhs(self._handle, _ptr(U), _ptr(out), _stream(self.device)))
        return out

    def step_(self, U: torch.Tensor, dt: float = 0.0, dt_dev: Optional[torch.Tensor] = None) -> torch.Tensor:
        """One RK4 step in place (dt from ``dt_dev`` if given: float64 device array, one per solve)."""
        self._check_state(U)
        dptr = _ptr(dt_dev) if dt_dev is not None else None
        _lib.check(self._lib.ps_step_rk4(self._handle, _ptr(U), float(dt), dptr, _stream(self.device)))
        return U

    def step_host_stream(self, inputs: Sequence[torch.Tensor], outputs: Sequence[torch.Tensor], dt: float,
                         nsteps: int = 1) -> None:
        """Advance a stream of independent states held in pinned host memory:
        output i = input i after ``nsteps`` RK4 steps of ``dt``.  The copy of
        state i + 1 to the device and of state i - 1 back to the host overlap
        the steps of state i (three device buffers, one copy stream per
        direction: the copy in of state i + 1 waits only for the copy out of
        state i - 2, so the two directions run at the same time; the steps
        themselves stay on the current stream, in order, since they share the
        plan's scratch).  Returns when every output has landed.  Inputs and
        outputs may repeat the same host tensors."""
        if len(inputs) != len(outputs):
            raise ValueError("inputs and outputs differ in length")
        comp = torch.cuda.current_stream(self.device)
        h2d, d2h = torch.cuda.Stream(self.device), torch.cuda.Stream(self.device)
        nbuf = 3
        bufs, freed = [], [None] * nbuf
        for i, (hi, ho) in enumerate(zip(inputs, outputs)):
            if not (hi.is_pinned() and ho.is_pinned()):
                raise ValueError("host states must be in pinned memory")
            b = i % nbuf
            if len(bufs) <= b:
                bufs.append(torch.empty(hi.shape, dtype=torch.float32, device=self.device))
            with torch.cuda.stream(h2d):
                if freed[b] is not None:
                    h2d.wait_event(freed[b])
                bufs[b].copy_(hi, non_blocking=True)
                loaded = torch.cuda.Event()
                loaded.record(h2d)
            comp.wait_event(loaded)
            self.run_(bufs[b], nsteps, dt) if nsteps > 1 else self.step_(bufs[b], dt)
            stepped = torch.cuda.Event()
            stepped.record(comp)
            with torch.cuda.stream(d2h):
                d2h.wait_event(stepped)
                ho.copy_(bufs[b], non_blocking=True)
                freed[b] = torch.cuda.Event()
                freed[b].record(d2h)
        d2h.synchronize()
        comp.wait_stream(d2h)

    def run_(self, U: torch.Tensor, nsteps: int, dt: float = 0.0,
             dt_dev: Optional[torch.Tensor] = None) -> torch.Tensor:
        self._check_state(U)
        dptr = _ptr(dt_dev) if dt_dev is not None else None
        _lib.check(self._lib.ps_run_steps(self._handle, _ptr(U), int(nsteps), float(dt), dptr,
                                          _stream(self.device)))
        return U

    def run_cfl_(self, U: torch.Tensor, nsteps: int, t: torch.Tensor, t_end: torch.Tensor) -> torch.Tensor:
        """Up to nsteps CFL steps with the time loop on the device; ``t`` and
        ``t_end`` are float64 device tensors of nsolve entries (``t`` advances
        in place, a solve stops at its t_end)."""
        self._check_state(U)
        for x in (t, t_end):
            if x.dtype != torch.float64 or x.device != self.device or x.numel() != self.nsolve:
                raise RuntimeError("t and t_end must be float64 device tensors with one entry per solve")
        _lib.check(self._lib.ps_run_cfl(self._handle, _ptr(U), int(nsteps), _ptr(t), _ptr(t_end),
                                        _stream(self.device)))
        return U

    @staticmethod
    def adaptive_desc(adaptive_config: Optional[dict] = None) -> "_lib.AdaptiveDesc":
        """ps_adaptive_desc from the reference's adaptive_config keys
        (scheme, rtol, atol, safety_factor, min_dt_factor, max_dt_factor,
        max_rejections; solver.py:182-193)."""
        cfg = dict(adaptive_config or {})
        ad = _lib.AdaptiveDesc()
        _lib.load().ps_adaptive_desc_init(C.byref(ad))
        scheme = str(cfg.get("scheme", "rk45")).lower()
        if scheme not in _lib.ARK_METHODS:
            raise ValueError(f"Unknown adaptive method: {scheme}. Supported methods: rk23, rk45, rk78")
        ad.method = _lib.ARK_METHODS[scheme]
        for key in ("rtol", "atol", "safety_factor", "min_dt_factor", "max_dt_factor"):
            if key in cfg:
                setattr(ad, key, float(cfg[key]))
        if "max_rejections" in cfg:
            ad.max_rejections = int(cfg["max_rejections"])
        return ad

    def run_adaptive_(self, U: torch.Tensor, nattempts: int, ad: "_lib.AdaptiveDesc", t: torch.Tensor,
                      t_end: torch.Tensor, dt: torch.Tensor, t_out: Optional[torch.Tensor] = None,
                      counts: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Up to nattempts adaptive embedded-RK attempts per solve, decisions
        on the device (ps_run_adaptive).  ``t``, ``t_end``, ``dt`` (proposed
        step, replaced by dt_next) and ``t_out`` (optional pause time) are
        float64 device tensors of nsolve entries; ``counts`` (optional) is an
        int32 device tensor [nsolve, 2] of accepted and rejected attempts."""
        self._check_state(U)
        for x in [t, t_end, dt] + ([t_out] if t_out is not None else []):
            if x.dtype != torch.float64 or x.device != self.device or x.numel() != self.nsolve:
                raise RuntimeError("t, t_end, dt and t_out must be float64 device tensors with one entry per solve")
        if counts is not None and (counts.dtype != torch.int32 or counts.device != self.device
                                   or counts.numel() != 2 * self.nsolve):
            raise RuntimeError("counts must be an int32 device tensor of nsolve x 2 entries")
        _lib.check(self._lib.ps_run_adaptive(self._handle, _ptr(U), int(nattempts), C.byref(ad), _ptr(t),
                                             _ptr(t_end), _ptr(dt), _ptr(t_out) if t_out is not None else None,
                                             _ptr(counts) if counts is not None else None, _stream(self.device)))
        return U

    def adaptive_reset(self) -> None:
        _lib.check(self._lib.ps_adaptive_reset(self._handle, _stream(self.device)))

    def derivative(self, f: torch.Tensor, axis: int, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """axis 0 = x (last array axis)."""
        nf = f.numel() // (self.cells * self.nsolve)
        self._check_state(f, nf)
        out = torch.empty_like(f) if out is None else out
        _lib.check(self._lib.ps_derivative(self._handle, int(axis), _ptr(f), _ptr(out), nf,
                                           _stream(self.device)))
        return out

    @property
    def tile_cols(self) -> int:
        """Columns per strided-pass tile (2D Fourier plans; 0 otherwise)."""
        return int(self._lib.ps_plan_tile_cols(self._handle))

    def axis_op(self, f: torch.Tensor, axis: int, op: str, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """One-axis operator along ``axis`` (0 = x): op "P" (mask x filter),
        "D" (masked derivative) or "L" (masked second derivative)."""
        ops = {"P": _lib.PS_OP_P, "D": _lib.PS_OP_D, "L": _lib.PS_OP_L}
        nf = f.numel() // (self.cells * self.nsolve)
        self._check_state(f, nf)
        out = torch.empty_like(f) if out is None else out
        _lib.check(self._lib.ps_axis_op(self._handle, int(axis), ops[op], _ptr(f), _ptr(out), nf,
                                        _stream(self.device)))
        return out

    def laplacian(self, f: torch.Tensor) -> torch.Tensor:
        """Sum over axes of L on that axis and P on the others."""
        total = None
        for a in range(self.ndim):
            t = f
            for b in range(self.ndim):
                t = self.axis_op(t, b, "L" if b == a else "P")
            total = t if total is None else total + t
        return total

    def filter(self, f: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        nf = f.numel() // (self.cells * self.nsolve)
        self._check_state(f, nf)
        out = torch.empty_like(f) if out is None else out
        _lib.check(self._lib.ps_filter(self._handle, _ptr(f), _ptr(out), nf, _stream(self.device)))
        return out

    def apply_boundary_conditions_(self, U: torch.Tensor) -> torch.Tensor:
        """Walls of an LGL plan in place (no-op for Fourier plans)."""
        self._check_state(U)
        _lib.check(self._lib.ps_apply_boundary_conditions(self._handle, _ptr(U), _stream(self.device)))
        return U

    def project_state_(self, U: torch.Tensor) -> torch.Tensor:
        """MHD: Helmholtz projection of B and the energy update in place."""
        self._check_state(U)
        _lib.check(self._lib.ps_project_state(self._handle, _ptr(U), _stream(self.device)))
        return U

    def _points(self, pts: torch.Tensor, n: Optional[int] = None) -> int:
        if not (isinstance(pts, torch.Tensor) and pts.device == self.device and pts.dtype == torch.float64
                and pts.is_contiguous() and pts.dim() == 2 and pts.shape[0] == self.ndim):
            raise RuntimeError(f"points must be a contiguous float64 ({self.ndim}, P) tensor on {self.device}")
        if n is not None and pts.shape[1] != n:
            raise RuntimeError("position arrays differ in length")
        return int(pts.shape[1])

    def tracer_method(self, method: str) -> None:
        """Interpolation of eval_points / tracers_step_: "auto" (NUFFT once
        points x cells exceeds 2^24, where the grid allows it), "exact" (the
        trigonometric interpolant, O(points x cells)) or "nufft" (type-2
        NUFFT, within 1e-6 of the exact interpolant)."""
        codes = {"auto": _lib.PS_TRACERS_AUTO, "exact": _lib.PS_TRACERS_EXACT, "nufft": _lib.PS_TRACERS_NUFFT}
        if method not in codes:
            raise ValueError(f"tracer method must be one of {sorted(codes)}, got {method!r}")
        _lib.check(self._lib.ps_tracer_method(self._handle, codes[method]))

    def eval_points(self, f: torch.Tensor, points: torch.Tensor, out: Optional[torch.Tensor] = None
                    ) -> torch.Tensor:
        """Spectral interpolant of the fields f (nf, *shape) (nf <= 3, one
        solve) at points (ndim, P) float64: out (nf, P) float32."""
        if not (f.device == self.device and f.dtype == torch.float32 and f.is_contiguous()):
            raise RuntimeError(f"expected contiguous float32 fields on {self.device}")
        nf = f.numel() // math.prod(self.shape)
        if f.numel() != nf * math.prod(self.shape) or not 1 <= nf <= 3:
            raise RuntimeError(f"expected 1..3 fields of {self.shape}, got {tuple(f.shape)}")
        npts = self._points(points)
        if out is None:
            out = torch.empty((nf, npts), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.ps_eval_points(self._handle, _ptr(f), nf, _ptr(points), npts, _ptr(out),
                                            _stream(self.device)))
        return out

    def tracers_step_(self, U: torch.Tensor, pos: torch.Tensor, prev: torch.Tensor, first: bool, dt: float,
                      velocity_out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """One leap-frog step of tracers in the velocity of U (solve 0):
        pos and prev (ndim, P) float64 updated in place."""
        if not (U.device == self.device and U.dtype == torch.float32 and U.is_contiguous()
                and U.numel() >= self.ncomp * math.prod(self.shape)):
            raise RuntimeError(f"expected a contiguous float32 state of {self.ncomp} x {self.shape}")
        npts = self._points(pos)
        self._points(prev, npts)
        vp = 0
        if velocity_out is not None:
            if not (velocity_out.device == self.device and velocity_out.dtype == torch.float32
                    and velocity_out.is_contiguous() and velocity_out.numel() == self.ndim * npts):
                raise RuntimeError("velocity_out must be a contiguous float32 (ndim, P) tensor")
            vp = _ptr(velocity_out)
        _lib.check(self._lib.ps_tracers_step(self._handle, _ptr(U), _ptr(pos), _ptr(prev), npts, 1 if first else 0,
                                             float(dt), vp, _stream(self.device)))
        return pos

    def project_solenoidal_3d_(self, Bx: torch.Tensor, By: torch.Tensor, Bz: torch.Tensor):
        """3D Helmholtz projection of (Bx, By, Bz) in place (one field per solve each)."""
        for b in (Bx, By, Bz):
            self._check_state(b, 1)
        _lib.check(self._lib.ps_project_solenoidal_3d(self._handle, _ptr(Bx), _ptr(By), _ptr(Bz),
                                                      _stream(self.device)))
        return Bx, By, Bz

    def project_solenoidal_(self, Bx: torch.Tensor, By: torch.Tensor):
        """Helmholtz projection of (Bx, By) in place (one field per solve each)."""
        self._check_state(Bx, 1)
        self._check_state(By, 1)
        _lib.check(self._lib.ps_project_solenoidal(self._handle, _ptr(Bx), _ptr(By), _stream(self.device)))
        return Bx, By

    def max_wave_speed(self, U: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        self._check_state(U)
        out = torch.empty(self.nsolve, dtype=torch.float32, device=self.device) if out is None else out
        _lib.check(self._lib.ps_max_wave_speed(self._handle, _ptr(U), _ptr(out), _stream(self.device)))
        return out

    def conserved(self, U: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        self._check_state(U)
        if out is None:
            nv = 8 if self.equations == "mhd" else self.ncomp
            shape = (nv,) if self.nsolve == 1 else (self.nsolve, nv)
            out = torch.empty(shape, dtype=torch.float64, device=self.device)
        _lib.check(self._lib.ps_conserved(self._handle, _ptr(U), _ptr(out), _stream(self.device)))
        return out

    def steps_done(self):
        """Steps taken per solve by run_cfl_ calls (list of nsolve ints)."""
        arr = (C.c_int * self.nsolve)()
        _lib.check(self._lib.ps_plan_steps_done(self._handle, arr))
        return list(arr)

    def status(self) -> int:
        """Device status word (0 = healthy; 1 = a kernel's bounded TMA wait ran out)."""
        v = C.c_int()
        _lib.check(self._lib.ps_plan_status(self._handle, C.byref(v)))
        return int(v.value)

    # -- launch profiling -------------------------------------------------
    def profile(self, enable: bool = True) -> None:
        """Bracket every pass launch with CUDA events (kind, algorithmic bytes)."""
        _lib.check(self._lib.ps_profile_enable(self._handle, 1 if enable else 0))

    def collect_profile(self) -> Dict[str, Dict[str, float]]:
        """Per-kind {launches, ms, bytes} of the launches since the last collect."""
        n = len(_lib.KIND_NAMES)
        la = (C.c_int * n)()
        ms = (C.c_double * n)()
        by = (C.c_double * n)()
        _lib.check(self._lib.ps_profile_collect(self._handle, n, la, ms, by))
        return {name: {"launches": int(la[i]), "ms": float(ms[i]), "bytes": float(by[i])}
                for i, name in enumerate(_lib.KIND_NAMES) if la[i] > 0}
