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

import os
from typing import Any, Dict, Optional, Tuple

__version__ = "0.1.0"

BACKENDS = ("gb300",)


def _load_config(config_path: Optional[str], config: Optional[Dict[str, Any]]) -> Dict[str, Any]:
    """A config dict, or a YAML/JSON config file (phrike/io.py:12-16); YAML is
    read with PyYAML when installed, else with phrike_gb300.config.load_yaml."""
    if config is not None:
        return dict(config)
    if config_path is None:
        return {}
    from .config import load_config
    return load_config(config_path)


def _filter_params(cfg: Dict[str, Any]) -> Optional[Dict[str, Any]]:
    sf = (cfg.get("integration", {}) or {}).get("spectral_filter", None)
    if not sf:
        return None
    return {"enabled": bool(sf.get("enabled", False)), "p": int(sf.get("p", 8)),
            "alpha": float(sf.get("alpha", 36.0)), "interval": sf.get("interval", None)}


# problem names of the benchmark workloads' initial states (phrike_gb300.problems);
# the reference's own problem names follow the reference's formulas (problem_ics.py)
BASELINE_PROBLEMS = ("baseline_sod1d", "baseline_tgv3d", "baseline_khi2d", "baseline_ot2d")


def _solver_options(cfg: Dict[str, Any]) -> Dict[str, Any]:
    """Adaptive, artificial-viscosity and gravity sections with the reference's
    defaults (problems/base.py:108-176): integration.adaptive, and the
    top-level artificial_viscosity and gravity blocks."""
    integ = cfg.get("integration", {}) or {}
    opts: Dict[str, Any] = {}
    ad = integ.get("adaptive", None)
    if ad:
        opts["adaptive_config"] = {
            "enabled": bool(ad.get("enabled", False)), "scheme": str(ad.get("scheme", "rk45")),
            "rtol": float(ad.get("rtol", 1e-6)), "atol": float(ad.get("atol", 1e-8)),
            "safety_factor": float(ad.get("safety_factor", 0.9)),
            "min_dt_factor": float(ad.get("min_dt_factor", 0.1)),
            "max_dt_factor": float(ad.get("max_dt_factor", 5.0)),
            "max_rejections": int(ad.get("max_rejections", 10)),
            "fallback_scheme": str(ad.get("fallback_scheme", "rk4"))}
    av = cfg.get("artificial_viscosity", None)
    if av:
        opts["artificial_viscosity_config"] = {
            "enabled": bool(av.get("enabled", False)), "mode": str(av.get("mode", "sensor")),
            "nu_constant": float(av.get("nu_constant", 0.0)), "nu_max": float(av.get("nu_max", 1e-3)),
            "s_ref": float(av.get("s_ref", 1.0)), "s_min": float(av.get("s_min", 0.1)),
            "p": float(av.get("p", 2.0)), "epsilon": float(av.get("epsilon", 1e-12)),
            "variable_weights": av.get("variable_weights", {"density": 1.0, "momentum_x": 1.0, "momentum_y": 1.0,
                                                            "momentum_z": 1.0, "energy": 1.0}),
            "sensor_variable": str(av.get("sensor_variable", "density"))}
    gr = cfg.get("gravity", None)
    if gr:
        opts["gravity_config"] = {"enabled": bool(gr.get("enabled", False)), "type": str(gr.get("type", "linear")),
                                  "gx": float(gr.get("gx", 0.0)), "gy": float(gr.get("gy", 0.0)),
                                  "gz": float(gr.get("gz", 0.0))}
    return opts


def _gamma(cfg: Dict[str, Any]) -> float:
    """physics.gamma or equations.gamma, required (problems/base.py:84-92)."""
    for sec in ("equations", "physics"):
        if sec in cfg and "gamma" in (cfg[sec] or {}):
            return float(cfg[sec]["gamma"])
    raise KeyError("Configuration must contain either 'equations.gamma' or 'physics.gamma'")


def _np(t: Any):
    import numpy as np
    return t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)


def _reference_problem(name: str, cfg: Dict[str, Any], kw: Dict[str, Any]):
    """Grid, equations, solver class and initial state of one of the
    reference's registered problems (problems/register.py:24-40), with each
    problem's create_grid rules and create_initial_conditions formulas."""
    from . import equations as E
    from . import grid as G
    from . import problem_ics as IC
    from . import solver as S
    kind, default_basis = IC.PROBLEMS[name]
    g = cfg["grid"]
    gamma = _gamma(cfg)
    mhd = (cfg.get("physics", {}) or {}).get("mhd", {}) or {}
    if kind.startswith("1d"):
        basis = "fourier" if name == "alfven1d" else str(g.get("basis", default_basis)).lower()
        grid = G.Grid1D(N=int(g["N"]), Lx=float(g["Lx"]), basis=basis, bc=g.get("bc", None),
                        dealias=bool(g.get("dealias", True)), problem_config=cfg, **kw)
        xs, L = (_np(grid.x),), (grid.Lx,)
        if kind == "1d_mhd":
            grid.mhd_config = mhd
            eqs, scls = E.MHDEquations1D(gamma=gamma), S.SpectralSolverMHD1D
        else:
            eqs, scls = E.EulerEquations1D(gamma=gamma), S.SpectralSolver1D
    elif kind.startswith("2d"):
        if kind == "2d_mhd":
            bx = by = "fourier"
            Lx, Ly = float(g.get("Lx", 1.0)), float(g.get("Ly", 1.0))
        else:
            bx = str(g.get("basis_x", default_basis)).lower()
            by = str(g.get("basis_y", default_basis)).lower()
            Lx, Ly = float(g["Lx"]), float(g["Ly"])
        dealias = False if name == "uniform_2d" else bool(g.get("dealias", True))
        bc = "dirichlet" if name == "uniform_2d" else g.get("bc", "dirichlet")
        grid = G.Grid2D(Nx=int(g["Nx"]), Ny=int(g["Ny"]), Lx=Lx, Ly=Ly, dealias=dealias, basis_x=bx, basis_y=by,
                        bc=bc, **kw)
        xs, L = (_np(grid.x), _np(grid.y)), (grid.Lx, grid.Ly)
        if kind == "2d_mhd":
            grid.mhd_config = mhd
            eqs, scls = E.MHDEquations2D(gamma=gamma), S.SpectralSolverMHD2D
        else:
            eqs, scls = E.EulerEquations2D(gamma=gamma), S.SpectralSolver2D
    else:
        grid = G.Grid3D(Nx=int(g["Nx"]), Ny=int(g["Ny"]), Nz=int(g["Nz"]), Lx=float(g["Lx"]), Ly=float(g["Ly"]),
                        Lz=float(g["Lz"]), dealias=bool(g.get("dealias", True)), **kw)
        xs, L = (_np(grid.x), _np(grid.y), _np(grid.z)), (grid.Lx, grid.Ly, grid.Lz)
        if kind == "3d_mhd":
            grid.mhd_config = mhd
            eqs, scls = E.MHDEquations3D(gamma=gamma), S.SpectralSolverMHD3D
        else:
            eqs, scls = E.EulerEquations3D(gamma=gamma), S.SpectralSolver3D
    legendre = getattr(grid, "_basis", "fourier") == "legendre"
    if legendre and str(kw.get("precision", "double")).lower() == "single":
        # the reference's LGL grids hold float32 nodes at single precision (its
        # run_simulation writes the precision argument into grid.precision), and
        # the hydrostatic initial states integrate in the nodes' dtype
        xs = tuple(a.astype("float32") for a in xs)
    U0 = IC.build(name, cfg, gamma, *xs, lengths=L, legendre=legendre)
    return grid, eqs, scls, U0


def _baseline_problem(name: str, cfg: Dict[str, Any], kw: Dict[str, Any]):
    """The benchmark workloads' initial states (phrike_gb300.problems) under
    their own names: smoothed Sod, Taylor-Green at p = 100/gamma + ..., the
    tanh double shear layer, Orszag-Tang at rho = gamma^2, p = gamma on
    [0, 2 pi)^2."""
    from . import equations as E
    from . import grid as G
    from . import problems as P
    from . import solver as S
    g = cfg.get("grid", {}) or {}
    phys = cfg.get("physics", cfg.get("equations", {})) or {}
    ic = cfg.get("initial_conditions", {}) or {}
    dealias = bool(g.get("dealias", True))
    if name == "baseline_sod1d":
        gamma = float(phys.get("gamma", 1.4))
        N, Lx = int(g.get("N", 1024)), float(g.get("Lx", 1.0))
        grid = G.Grid1D(N=N, Lx=Lx, dealias=dealias, **kw)
        return grid, E.EulerEquations1D(gamma=gamma), S.SpectralSolver1D, \
            P.sod_smoothed(N, Lx, gamma, float(ic.get("width", 0.005)))
    if name == "baseline_tgv3d":
        gamma = float(phys.get("gamma", 1.4))
        N = int(g.get("N", 64))
        Nx, Ny, Nz = int(g.get("Nx", N)), int(g.get("Ny", N)), int(g.get("Nz", N))
        L = float(g.get("Lx", 2.0 * 3.141592653589793))
        grid = G.Grid3D(Nx=Nx, Ny=Ny, Nz=Nz, Lx=L, Ly=float(g.get("Ly", L)), Lz=float(g.get("Lz", L)),
                        dealias=dealias, **kw)
        return grid, E.EulerEquations3D(gamma=gamma), S.SpectralSolver3D, P.taylor_green_3d(Nx, Ny, Nz, gamma, L)
    if name == "baseline_khi2d":
        gamma = float(phys.get("gamma", 1.4))
        N = int(g.get("N", 128))
        Nx, Ny = int(g.get("Nx", N)), int(g.get("Ny", N))
        grid = G.Grid2D(Nx=Nx, Ny=Ny, Lx=1.0, Ly=1.0, dealias=dealias, **kw)
        return grid, E.EulerEquations2D(gamma=gamma), S.SpectralSolver2D, \
            P.kelvin_helmholtz_2d(Nx, Ny, float(ic.get("U0", 1.0)), float(ic.get("A", 0.01)), gamma)
    gamma = float(phys.get("gamma", 5.0 / 3.0))
    N = int(g.get("N", 128))
    Nx, Ny = int(g.get("Nx", N)), int(g.get("Ny", N))
    L = float(g.get("Lx", 2.0 * 3.141592653589793))
    grid = G.Grid2D(Nx=Nx, Ny=Ny, Lx=L, Ly=float(g.get("Ly", L)), dealias=dealias, **kw)
    grid.mhd_config = (phys.get("mhd", {}) or {})
    return grid, E.MHDEquations2D(gamma=gamma), S.SpectralSolverMHD2D, \
        P.orszag_tang_2d(Nx, Ny, gamma, ic.get("rho0"), ic.get("p0"), float(ic.get("B0", 1.0)), L)


def run_simulation(problem_name: str, config_path: Optional[str] = None, config: Optional[Dict[str, Any]] = None,
                   backend: str = "gb300", device: Optional[str] = "cuda", precision: str = "single",
                   generate_video: bool = False, debug: bool = False,
                   outdir: Optional[str] = None) -> Tuple[Any, Dict[str, Any]]:
    """Run a problem and return (solver, history), like phrike.run_simulation
    (phrike/__init__.py:14-56) with BaseProblem.run (problems/base.py:1024-1181).

    Problem names are the reference's registered problems (sod, acoustic1d,
    gaussian_wave1d, shu_osher1d, hse_1d, rti_1d, alfven1d, khi2d, uniform_2d,
    rti, gaussian_wave2d, gaussian_wave2d_y, orszag_tang2d, tgv3d, turb3d,
    alfven3d, mhd_turb3d), configured by the reference's schema with its
    required keys and defaults, so that a shipped reference config runs the
    same problem: grid (N | Nx, Ny, Nz; Lx, Ly, Lz; dealias; basis | basis_x,
    basis_y; bc), physics.gamma, integration (t0, t_end, cfl, scheme,
    output_interval, checkpoint_interval, spectral_filter, adaptive),
    initial_conditions, initial_conditions_smoothing, artificial_viscosity,
    gravity and tracers.  The benchmark workloads' initial states run as
    baseline_sod1d, baseline_tgv3d, baseline_khi2d and baseline_ot2d.
    integration.dt (a fixed step) is an addition.  Video output is not part
    of the step engine.
    """
    if backend not in BACKENDS:
        raise ValueError(f"backend must be one of {BACKENDS} in phrike_gb300 (got {backend!r})")
    if generate_video:
        raise NotImplementedError("video output is outside the step engine")
    from . import problem_ics as IC

    cfg = _load_config(config_path, config)
    name = problem_name.lower()
    if name not in IC.PROBLEMS and name not in BASELINE_PROBLEMS:
        raise ValueError(f"unknown problem {problem_name!r} (available: "
                         f"{', '.join(list(IC.PROBLEMS) + list(BASELINE_PROBLEMS))})")
    kw = dict(filter_params=_filter_params(cfg), backend=backend, torch_device=device, precision=precision,
              debug=debug)
    if name in IC.PROBLEMS:
        grid, eqs, scls, U0 = _reference_problem(name, cfg, kw)
        integ = cfg["integration"]
        t0, t_end, cfl = float(integ["t0"]), float(integ["t_end"]), float(integ["cfl"])
    else:
        grid, eqs, scls, U0 = _baseline_problem(name, cfg, kw)
        integ = cfg.get("integration", {}) or {}
        cfl_default = {"baseline_sod1d": 0.4, "baseline_tgv3d": 0.25, "baseline_khi2d": 0.4, "baseline_ot2d": 0.3}
        t0, t_end = float(integ.get("t0", 0.0)), float(integ.get("t_end", 0.01))
        cfl = float(integ.get("cfl", cfl_default[name]))
    solver = scls(grid, eqs, scheme=str(integ.get("scheme", "rk4")), cfl=cfl, **_solver_options(cfg))
    if outdir is None and name in IC.PROBLEMS and float(integ.get("checkpoint_interval", 0.0)) > 0:
        io = cfg.get("io", {}) or {}
        outdir = os.path.abspath(io.get("outdir", f"outputs/{cfg.get('problem', name)}"))
    dt = integ.get("dt", None)
    # tracer particles from the ``tracers`` block (problems/base.py:961-1021, 1082-1102)
    from .tracers import tracers_from_config
    tracers = tracers_from_config(grid, cfg.get("tracers", {}) or {})
    history = solver.run(U0, t0, t_end, output_interval=float(integ.get("output_interval", 0.1)),
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
