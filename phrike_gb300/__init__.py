"""phrike_gb300 — GB300 (sm_103a) engine for the right-hand-side-and-step path
of the pseudo-spectral Euler solver of PHRIKE, under the backend name "gb300".

Public API (mirrors the reference package):
    run_simulation(problem_name, config_path=None, config=None, backend="gb300", ...)
    Grid1D, Grid2D, Grid3D                    (phrike_gb300.grid)
    EulerEquations1D/2D/3D                    (phrike_gb300.equations)
    SpectralSolver1D/2D/3D                    (phrike_gb300.solver)
    engine.Plan                               (direct C-ABI plan handle)
The CUDA library is built in-tree by phrike_gb300._build.build().
"""
from __future__ import annotations

import json
import os
from typing import Any, Dict, Optional, Tuple

__version__ = "0.1.0"

BACKENDS = ("gb300",)


def _load_config(config_path: Optional[str], config: Optional[Dict[str, Any]]) -> Dict[str, Any]:
    """YAML/JSON config loading (phrike/io.py:12-16).  PyYAML is optional."""
    if config is not None:
        return dict(config)
    if config_path is None:
        return {}
    with open(config_path) as f:
        text = f.read()
    if config_path.endswith((".yaml", ".yml")):
        try:
            import yaml  # type: ignore
        except ImportError as e:  # pragma: no cover - depends on the environment
            raise RuntimeError("PyYAML is needed to read YAML configs; pass config=dict(...) instead") from e
        return yaml.safe_load(text) or {}
    return json.loads(text)


def _filter_params(cfg: Dict[str, Any]) -> Optional[Dict[str, Any]]:
    sf = (cfg.get("integration", {}) or {}).get("spectral_filter", None)
    if not sf:
        return None
    return {"enabled": bool(sf.get("enabled", False)), "p": int(sf.get("p", 8)),
            "alpha": float(sf.get("alpha", 36.0)), "interval": sf.get("interval", None)}


def run_simulation(problem_name: str, config_path: Optional[str] = None, config: Optional[Dict[str, Any]] = None,
                   backend: str = "gb300", device: Optional[str] = "cuda", precision: str = "single",
                   generate_video: bool = False, debug: bool = False,
                   outdir: Optional[str] = None) -> Tuple[Any, Dict[str, Any]]:
    """Run one of the built-in problems and return (solver, history), like
    phrike.run_simulation (phrike/__init__.py:14-56).

    Problems: "sod" (1D smoothed Sod step), "tgv3d" (3D Taylor-Green vortex),
    "khi2d" (2D Kelvin-Helmholtz double shear layer), "orszag_tang2d" (2D ideal
    MHD, rho = gamma^2, p = gamma, B0 = 1 on [0, 2 pi)^2 by default).  Config keys follow the
    reference schema: grid.{N|Nx,Ny,Nz, Lx,Ly,Lz, dealias}, physics.gamma,
    integration.{t0, t_end, cfl, scheme, dt, output_interval, spectral_filter},
    initial_conditions.{...}.  integration.dt (fixed step) is an addition.
    """
    if backend not in BACKENDS:
        raise ValueError(f"backend must be one of {BACKENDS} in phrike_gb300 (got {backend!r})")
    if generate_video:
        raise NotImplementedError("video output is outside the step engine")
    from . import equations as E
    from . import grid as G
    from . import problems as P
    from . import solver as S

    cfg = _load_config(config_path, config)
    g = cfg.get("grid", {}) or {}
    phys = cfg.get("physics", cfg.get("equations", {})) or {}
    integ = cfg.get("integration", {}) or {}
    ic = cfg.get("initial_conditions", {}) or {}
    gamma = float(phys.get("gamma", 1.4))
    dealias = bool(g.get("dealias", True))
    fp = _filter_params(cfg)
    kw = dict(dealias=dealias, filter_params=fp, backend=backend, torch_device=device, precision=precision,
              debug=debug)
    name = problem_name.lower()
    # adaptive (integration.adaptive), artificial viscosity and gravity sections,
    # with the reference's defaults (problems/base.py:110-176)
    ad = integ.get("adaptive", None)
    opts: Dict[str, Any] = {}
    if ad:
        opts["adaptive_config"] = dict({"scheme": "rk45", "rtol": 1e-6, "atol": 1e-8, "safety_factor": 0.9,
                                        "min_dt_factor": 0.1, "max_dt_factor": 5.0, "max_rejections": 10,
                                        "fallback_scheme": "rk4"}, **ad, enabled=bool(ad.get("enabled", False)))
    if cfg.get("artificial_viscosity"):
        opts["artificial_viscosity_config"] = dict(cfg["artificial_viscosity"])
    if cfg.get("gravity"):
        opts["gravity_config"] = dict(cfg["gravity"])
    if name == "sod":
        N = int(g.get("N", 1024))
        Lx = float(g.get("Lx", 1.0))
        grid = G.Grid1D(N=N, Lx=Lx, **kw)
        eqs = E.EulerEquations1D(gamma=gamma)
        U0 = P.sod_smoothed(N, Lx, gamma, float(ic.get("width", 0.005)))
        solver = S.SpectralSolver1D(grid, eqs, scheme=integ.get("scheme", "rk4"), cfl=float(integ.get("cfl", 0.4)),
                                    **opts)
    elif name == "tgv3d":
        N = int(g.get("N", 64))
        Nx, Ny, Nz = int(g.get("Nx", N)), int(g.get("Ny", N)), int(g.get("Nz", N))
        L = float(g.get("Lx", 2.0 * 3.141592653589793))
        grid = G.Grid3D(Nx=Nx, Ny=Ny, Nz=Nz, Lx=L, Ly=float(g.get("Ly", L)), Lz=float(g.get("Lz", L)), **kw)
        eqs = E.EulerEquations3D(gamma=gamma)
        U0 = P.taylor_green_3d(Nx, Ny, Nz, gamma, L)
        solver = S.SpectralSolver3D(grid, eqs, scheme=integ.get("scheme", "rk4"), cfl=float(integ.get("cfl", 0.25)),
                                    **opts)
    elif name == "khi2d":
        N = int(g.get("N", 128))
        Nx, Ny = int(g.get("Nx", N)), int(g.get("Ny", N))
        grid = G.Grid2D(Nx=Nx, Ny=Ny, Lx=1.0, Ly=1.0, **kw)
        eqs = E.EulerEquations2D(gamma=gamma)
        U0 = P.kelvin_helmholtz_2d(Nx, Ny, float(ic.get("U0", 1.0)), float(ic.get("A", 0.01)), gamma)
        solver = S.SpectralSolver2D(grid, eqs, scheme=integ.get("scheme", "rk4"), cfl=float(integ.get("cfl", 0.4)),
                                    **opts)
    elif name == "orszag_tang2d":
        N = int(g.get("N", 128))
        Nx, Ny = int(g.get("Nx", N)), int(g.get("Ny", N))
        L = float(g.get("Lx", 2.0 * 3.141592653589793))
        gamma = float(phys.get("gamma", 5.0 / 3.0))
        grid = G.Grid2D(Nx=Nx, Ny=Ny, Lx=L, Ly=float(g.get("Ly", L)), **kw)
        grid.mhd_config = (phys.get("mhd", {}) or {})
        eqs = E.MHDEquations2D(gamma=gamma)
        U0 = P.orszag_tang_2d(Nx, Ny, gamma, ic.get("rho0"), ic.get("p0"), float(ic.get("B0", 1.0)), L)
        solver = S.SpectralSolverMHD2D(grid, eqs, scheme=integ.get("scheme", "rk4"),
                                       cfl=float(integ.get("cfl", 0.3)), **opts)
    elif name == "alfven1d":
        N = int(g.get("N", 128))
        Lx = float(g.get("Lx", 1.0))
        gamma = float(phys.get("gamma", 5.0 / 3.0))
        grid = G.Grid1D(N=N, Lx=Lx, **kw)
        grid.mhd_config = (phys.get("mhd", {}) or {})
        eqs = E.MHDEquations1D(gamma=gamma)
        U0 = P.alfven_cp_1d(N, Lx, 0.0, float(ic.get("rho0", 1.0)), float(ic.get("p0", 0.1)),
                            float(ic.get("B0", 1.0)), float(ic.get("b1", 0.1)), int(ic.get("m", 1)),
                            int(ic.get("direction", 1)), gamma)
        solver = S.SpectralSolverMHD1D(grid, eqs, scheme=integ.get("scheme", "rk4"),
                                       cfl=float(integ.get("cfl", 0.4)), **opts)
    elif name == "alfven3d":
        Nx, Ny, Nz = int(g.get("Nx", 64)), int(g.get("Ny", 8)), int(g.get("Nz", 8))
        Lx = float(g.get("Lx", 1.0))
        gamma = float(phys.get("gamma", 5.0 / 3.0))
        grid = G.Grid3D(Nx=Nx, Ny=Ny, Nz=Nz, Lx=Lx, Ly=float(g.get("Ly", 1.0)), Lz=float(g.get("Lz", 1.0)), **kw)
        grid.mhd_config = (phys.get("mhd", {}) or {})
        eqs = E.MHDEquations3D(gamma=gamma)
        U0 = P.alfven_cp_3d(Nx, Ny, Nz, Lx, 0.0, float(ic.get("rho0", 1.0)), float(ic.get("p0", 0.1)),
                            float(ic.get("B0", 1.0)), float(ic.get("b1", 0.1)), int(ic.get("m", 1)),
                            int(ic.get("direction", 1)), gamma)
        solver = S.SpectralSolverMHD3D(grid, eqs, scheme=integ.get("scheme", "rk4"),
                                       cfl=float(integ.get("cfl", 0.3)), **opts)
    else:
        raise ValueError(f"unknown problem {problem_name!r} "
                         "(available: sod, tgv3d, khi2d, orszag_tang2d, alfven1d, alfven3d)")
    dt = integ.get("dt", None)
    # tracer particles from the ``tracers`` block (problems/base.py:961-1021, 1082-1102)
    from .tracers import tracers_from_config
    tracers = tracers_from_config(grid, cfg.get("tracers", {}) or {})
    history = solver.run(U0, float(integ.get("t0", 0.0)), float(integ.get("t_end", 0.01)),
                         output_interval=float(integ.get("output_interval", 0.1)),
                         checkpoint_interval=float(integ.get("checkpoint_interval", 0.0)), outdir=outdir,
                         tracers=tracers, dt=float(dt) if dt is not None else None)
    solver.tracers = tracers
    return solver, history


def __getattr__(name: str):
    # lazy re-exports so that importing the package does not import torch
    if name in ("Grid1D", "Grid2D", "Grid3D"):
        from . import grid
        return getattr(grid, name)
    if name in ("EulerEquations1D", "EulerEquations2D", "EulerEquations3D", "MHDEquations1D", "MHDEquations2D",
                "MHDEquations3D"):
        from . import equations
        return getattr(equations, name)
    if name in ("SpectralSolver1D", "SpectralSolver2D", "SpectralSolver3D", "SpectralSolverMHD1D",
                "SpectralSolverMHD2D", "SpectralSolverMHD3D"):
        from . import solver
        return getattr(solver, name)
    if name in ("FourierTracers1D", "FourierTracers2D", "FourierTracers3D"):
        from . import tracers
        return getattr(tracers, name)
    raise AttributeError(name)
