"""Generate golden vectors by running the reference package (phrike) itself.

Run once where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/phrike-checkout

The reference imports ``yaml`` and ``matplotlib`` only for config loading and
plotting; both are replaced by empty placeholder modules here.  numba is not
installed, so the reference runs its plain-NumPy fallbacks (float64).

Each fixture stores the inputs (or the recipe to rebuild them) and the
reference outputs after a few fixed-dt steps, so the oracle and the CUDA path
can be compared against the reference without the reference present.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def import_reference(path: str):
    for name in ("yaml", "matplotlib", "matplotlib.pyplot", "matplotlib.animation",
                 "matplotlib.colors", "matplotlib.cm"):
        if name not in sys.modules:
            mod = types.ModuleType(name)
            mod.use = lambda *a, **k: None
            sys.modules[name] = mod
    sys.path.insert(0, path)
    import phrike  # noqa: F401
    from phrike import grid, equations, solver
    return grid, equations, solver


def main(ref_path: str, only: str = "") -> None:
    grid, equations, solver = import_reference(ref_path)
    from phrike_gb300 import problems
    if only == "mhd":
        return mhd_fixtures(grid, equations, solver, problems)
    if only == "sources":
        return source_fixtures(grid, equations, solver, problems)
    if only == "adaptive":
        return adaptive_fixtures(grid, equations, solver, problems)
    if only == "rk2":
        return rk2_fixtures(grid, equations, solver, problems)
    if only == "mhd_diffusion":
        return mhd_diffusion_fixtures(grid, equations, solver, problems)
    if only == "mhd1d":
        return mhd1d_fixtures(grid, equations, solver, problems)
    if only == "mhd3d":
        return mhd3d_fixtures(grid, equations, solver, problems)
    if only == "tracers":
        return tracer_fixtures(grid, equations, solver, problems)
    if only == "problems":
        return problem_ic_fixtures(ref_path)
    if only == "lgl1d":
        return lgl1d_fixtures(grid, equations, solver, problems)

    out = {}

    # --- operator fixtures: random fields through dx1/dy1/dz1/filter -------
    rng = np.random.default_rng(20261203)
    filt = {"enabled": True, "p": 8, "alpha": 36.0}
    ops = {}
    for dealias in (True, False):
        for fon in (False, True):
            tag = f"d{int(dealias)}f{int(fon)}"
            fp = filt if fon else None
            g1 = grid.Grid1D(N=64, Lx=1.0, dealias=dealias, filter_params=fp)
            f1 = rng.standard_normal((3, 64))
            ops[f"g1_{tag}_in"] = f1
            ops[f"g1_{tag}_dx"] = g1.dx1(f1.copy())
            ops[f"g1_{tag}_filt"] = g1.apply_spectral_filter(f1.copy())
            g2 = grid.Grid2D(Nx=32, Ny=16, Lx=1.0, Ly=0.5, dealias=dealias, filter_params=fp)
            f2 = rng.standard_normal((2, 16, 32))
            ops[f"g2_{tag}_in"] = f2
            ops[f"g2_{tag}_dx"] = g2.dx1(f2.copy())
            ops[f"g2_{tag}_dy"] = g2.dy1(f2.copy())
            ops[f"g2_{tag}_filt"] = g2.apply_spectral_filter(f2.copy())
            g3 = grid.Grid3D(Nx=16, Ny=8, Nz=16, Lx=2 * np.pi, Ly=np.pi, Lz=4 * np.pi,
                             dealias=dealias, filter_params=fp)
            f3 = rng.standard_normal((1, 16, 8, 16))
            ops[f"g3_{tag}_in"] = f3
            ops[f"g3_{tag}_dx"] = g3.dx1(f3.copy())
            ops[f"g3_{tag}_dy"] = g3.dy1(f3.copy())
            ops[f"g3_{tag}_dz"] = g3.dz1(f3.copy())
            ops[f"g3_{tag}_filt"] = g3.apply_spectral_filter(f3.copy())
    np.savez_compressed(os.path.join(HERE, "fourier_ops.npz"), **ops)

    # --- 1D Sod, filter p=8 alpha=36, dealias, dt=2e-5 ------------------
    for N, nsteps in ((128, 5), (1024, 3)):
        g = grid.Grid1D(N=N, Lx=1.0, dealias=True, filter_params=dict(filt))
        eq = equations.EulerEquations1D(gamma=1.4)
        s = solver.SpectralSolver1D(g, eq, scheme="rk4", cfl=0.4)
        U0 = problems.sod_smoothed(N)
        rhs0 = solver._compute_rhs(g, eq, U0.copy())
        U = U0.copy()
        for _ in range(nsteps):
            U = s.step(U, 2e-5)
        np.savez_compressed(os.path.join(HERE, f"sod1d_n{N}.npz"), U0=U0, rhs0=rhs0, U=U,
                            dt=2e-5, nsteps=nsteps, dt_cfl0=s.compute_dt(U0),
                            cons=np.array([eq.conserved_quantities(U)[k]
                                           for k in ("mass", "momentum", "energy")]))

    # --- 3D TGV, dealias, filter off, dt=1e-3 --------------------------
    for (Nx, Ny, Nz), nsteps in (((16, 16, 16), 3), ((16, 8, 32), 2)):
        g = grid.Grid3D(Nx=Nx, Ny=Ny, Nz=Nz, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, dealias=True)
        eq = equations.EulerEquations3D(gamma=1.4)
        s = solver.SpectralSolver3D(g, eq, scheme="rk4", cfl=0.25)
        U0 = problems.taylor_green_3d(Nx, Ny, Nz)
        rhs0 = solver._compute_rhs_3d(g, eq, U0.copy())
        U = U0.copy()
        for _ in range(nsteps):
            U = s.step(U, 1e-3)
        np.savez_compressed(os.path.join(HERE, f"tgv3d_{Nx}x{Ny}x{Nz}.npz"), U0=U0, rhs0=rhs0,
                            U=U, dt=1e-3, nsteps=nsteps, dt_cfl0=s.compute_dt(U0),
                            speed0=eq.max_wave_speed(U0))

    # --- 2D KHI, CFL 0.4 run loop --------------------------------------
    for (Nx, Ny), nsteps in (((32, 32), 4), ((64, 16), 3)):
        g = grid.Grid2D(Nx=Nx, Ny=Ny, Lx=1.0, Ly=1.0, dealias=True)
        eq = equations.EulerEquations2D(gamma=1.4)
        s = solver.SpectralSolver2D(g, eq, scheme="rk4", cfl=0.4)
        U0 = problems.kelvin_helmholtz_2d(Nx, Ny, U0=1.2, A=0.015)
        rhs0 = solver._compute_rhs_2d(g, eq, U0.copy())
        U = U0.copy()
        t = 0.0
        dts = []
        dt = s.compute_dt(U)
        for _ in range(nsteps):
            U = s.step(U, dt)
            t += dt
            dts.append(dt)
            dt = s.compute_dt(U)
        np.savez_compressed(os.path.join(HERE, f"khi2d_{Nx}x{Ny}.npz"), U0=U0, rhs0=rhs0, U=U,
                            dts=np.array(dts), t=t, U0_param=1.2, A=0.015)

    # --- 2D LGL x LGL acoustic pulse, walls, torch-CPU float64 backend -----
    # (the NumPy fallback of LegendreLobattoBasis2D.dy returns transposed
    # axes when numba is absent, so the torch path is the correct reference)
    import torch
    for (nx, ny), nsteps, dt in (((17, 17), 3, 1e-4), ((33, 17), 2, 1e-4)):
        g = grid.Grid2D(Nx=nx, Ny=ny, Lx=2.0, Ly=2.0, basis_x="legendre", basis_y="legendre",
                        bc="dirichlet", backend="torch", torch_device="cpu", precision="double")
        eq = equations.EulerEquations2D(gamma=1.4)
        s = solver.SpectralSolver2D(g, eq, scheme="rk4", cfl=0.3)
        x = np.asarray(g.x.cpu().numpy() if hasattr(g.x, "cpu") else g.x)
        y = np.asarray(g.y.cpu().numpy() if hasattr(g.y, "cpu") else g.y)
        U0 = problems.acoustic_pulse_lgl_2d(x - 1.0, y - 1.0, gamma=1.4, amp=0.2, width2=0.05)
        Ut = torch.from_numpy(U0.copy())
        rhs0 = solver._compute_rhs_2d(g, eq, Ut.clone()).numpy()
        U = Ut.clone()
        for _ in range(nsteps):
            U = s.step(U, dt)
        Dx = g._legendre_basis._Dx
        Dy = g._legendre_basis._Dy
        np.savez_compressed(os.path.join(HERE, f"lgl2d_{nx}x{ny}.npz"), U0=U0, rhs0=rhs0, U=U.numpy(), dt=dt,
                            nsteps=nsteps, x=x, y=y, Dx=Dx, Dy=Dy, dt_cfl0=s.compute_dt(torch.from_numpy(U0)),
                            amp=0.2, width2=0.05)

    mhd_fixtures(grid, equations, solver, problems)
    source_fixtures(grid, equations, solver, problems)
    print("golden fixtures written to", HERE)


def source_fixtures(grid, equations, solver, problems) -> None:
    """Gravity (2D KHI, 3D TGV) and artificial viscosity (1D Sod, 2D KHI,
    sensor and constant modes) through the reference's NumPy path."""
    grav2 = {"enabled": True, "gx": 0.3, "gy": -1.0}
    grav3 = {"enabled": True, "gx": 0.2, "gy": -0.5, "gz": 1.0}
    out = {}
    g2 = grid.Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True)
    s2 = solver.SpectralSolver2D(g2, equations.EulerEquations2D(gamma=1.4), cfl=0.4, gravity_config=grav2)
    U0 = problems.kelvin_helmholtz_2d(32, 32, U0=1.2, A=0.015)
    U = U0.copy()
    for _ in range(3):
        U = s2.step(U, 2e-3)
    out["grav2d_U0"], out["grav2d_U"] = U0, U
    out["grav2d_rhs0"] = solver._compute_rhs_2d(g2, s2.equations, U0.copy(), None, grav2)
    g3 = grid.Grid3D(Nx=16, Ny=16, Nz=16, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, dealias=True)
    s3 = solver.SpectralSolver3D(g3, equations.EulerEquations3D(gamma=1.4), cfl=0.25, gravity_config=grav3)
    T0 = problems.taylor_green_3d(16, 16, 16)
    T = T0.copy()
    for _ in range(2):
        T = s3.step(T, 1e-3)
    out["grav3d_U0"], out["grav3d_U"] = T0, T
    out["grav3d_rhs0"] = solver._compute_rhs_3d(g3, s3.equations, T0.copy(), None, grav3)
    # artificial viscosity, 1D (sensor mode, default cadence 5) and 2D (sensor / constant)
    av_sensor = {"enabled": True, "mode": "sensor", "nu_max": 2e-3, "s_ref": 1.0, "s_min": 0.1, "p": 2.0,
                 "epsilon": 1e-12, "sensor_variable": "density"}
    g1 = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params={"enabled": True, "p": 8, "alpha": 36.0})
    s1 = solver.SpectralSolver1D(g1, equations.EulerEquations1D(gamma=1.4), cfl=0.4,
                                 artificial_viscosity_config=av_sensor)
    S0 = problems.sod_smoothed(128)
    S = S0.copy()
    for _ in range(7):
        S = s1.step(S, 2e-5)
    out["av1d_U0"], out["av1d_U"], out["av1d_interval"] = S0, S, s1.filter_interval
    out["av1d_rhs0"] = solver._compute_rhs(g1, s1.equations, S0.copy(), s1.artificial_viscosity, None)
    for mode, cfg in (("sensor", dict(av_sensor, sensor_variable="pressure")),
                      ("constant", {"enabled": True, "mode": "constant", "nu_constant": 1e-3})):
        g2b = grid.Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True)
        s2b = solver.SpectralSolver2D(g2b, equations.EulerEquations2D(gamma=1.4), cfl=0.4,
                                      artificial_viscosity_config=cfg)
        V = U0.copy()
        for _ in range(3):
            V = s2b.step(V, 2e-3)
        out[f"av2d_{mode}_U"] = V
        out[f"av2d_{mode}_rhs0"] = solver._compute_rhs_2d(g2b, s2b.equations, U0.copy(), s2b.artificial_viscosity,
                                                           None)
    np.savez_compressed(os.path.join(HERE, "sources.npz"), **out)

def mhd3d_fixtures(grid, equations, solver, problems) -> None:
    """3D MHD (SpectralSolverMHD3D) on the cases of tests/mhd3d_cases.py:
    rhs, the projected state, fixed-dt steps, the CFL dt, div B and the
    conserved sums; plus a short CFL run of the Alfven case."""
    sys.path.insert(0, os.path.dirname(HERE))
    import mhd3d_cases as MC
    out = {}
    for name, (nx, ny, nz, lx, ly, lz, filt, cfg, scheme, dt, nsteps) in MC.CASES.items():
        g = grid.Grid3D(Nx=nx, Ny=ny, Nz=nz, Lx=lx, Ly=ly, Lz=lz, dealias=True,
                        filter_params=dict(filt) if filt else None)
        g.mhd_config = dict(cfg)
        eq = equations.MHDEquations3D(gamma=MC.GAMMA)
        s = solver.SpectralSolverMHD3D(g, eq, scheme=scheme, cfl=0.3)
        U0 = MC.initial_state(name)
        out[f"{name}_U0"] = U0
        out[f"{name}_rhs0"] = s._compute_rhs(U0.copy())
        out[f"{name}_P0"] = s._project_B(U0.copy())
        U = U0.copy()
        for _ in range(nsteps):
            U = s.step(U, dt)
        out[f"{name}_U"] = U
        out[f"{name}_dt0"] = s.compute_dt(U0)
        out[f"{name}_divb_U"] = s.max_div_b(U)
        c = eq.conserved_quantities(U)
        out[f"{name}_cons"] = np.array([c[k] for k in ("mass", "momentum_x", "momentum_y", "momentum_z", "energy",
                                                        "magnetic_energy", "cross_helicity")])
    nx, ny, nz, lx, ly, lz, filt = MC.CASES["alfven"][:7]
    g = grid.Grid3D(Nx=nx, Ny=ny, Nz=nz, Lx=lx, Ly=ly, Lz=lz, dealias=True, filter_params=dict(filt))
    g.mhd_config = {}
    s = solver.SpectralSolverMHD3D(g, equations.MHDEquations3D(gamma=MC.GAMMA), cfl=0.3)
    seen = []
    s.run(MC.initial_state("alfven"), 0.0, 0.05, output_interval=0.05, on_step=lambda n, dt, U: seen.append(dt))
    out["cfl_U"], out["cfl_t"], out["cfl_dts"] = np.asarray(s.U), s.t, np.asarray(seen)
    np.savez_compressed(os.path.join(HERE, "mhd3d.npz"), **out)


def tracer_fixtures(grid, equations, solver, problems) -> None:
    """Tracers (tracers.py) and point evaluation (grid.py evaluate_fourier_at_*)
    on the cases of tests/tracer_cases.py: a random field and the velocity
    at the initial tracer positions, the tracer positions after STEPS
    leap-frog steps in the fixed state, and a KHI 32^2 run (CFL 0.4,
    t_end 0.02) with 30 tracers through SpectralSolver2D.run."""
    sys.path.insert(0, os.path.dirname(HERE))
    import tracer_cases as TC
    from phrike import tracers as T
    out = {}
    for name, (shape, lengths, dealias, filt, _) in TC.CASES.items():
        nd = len(shape)
        fp = dict(filt) if filt else None
        if nd == 1:
            g = grid.Grid1D(N=shape[0], Lx=lengths[0], dealias=dealias, filter_params=fp)
            eq = equations.EulerEquations1D(gamma=TC.GAMMA)
        elif nd == 2:
            g = grid.Grid2D(Nx=shape[1], Ny=shape[0], Lx=lengths[1], Ly=lengths[0], dealias=dealias,
                            filter_params=fp)
            eq = equations.EulerEquations2D(gamma=TC.GAMMA)
        else:
            g = grid.Grid3D(Nx=shape[2], Ny=shape[1], Nz=shape[0], Lx=lengths[2], Ly=lengths[1], Lz=lengths[0],
                            dealias=dealias, filter_params=fp)
            eq = equations.EulerEquations3D(gamma=TC.GAMMA)
        U = TC.state(name)
        f = TC.field(name)
        pos = TC.tracer_positions(name)
        prim = eq.primitive(U)
        vel = [prim[1 + a] for a in range(nd)]
        if nd == 1:
            fv = g.evaluate_fourier_at_points_1d(f, pos[0])
            vv = [g.evaluate_fourier_at_points_1d(vel[0], pos[0])]
            tr = T.FourierTracers1D(pos[0])
        elif nd == 2:
            fv = g.evaluate_fourier_at_points(f, pos[0], pos[1])
            vv = [g.evaluate_fourier_at_points(v, pos[0], pos[1]) for v in vel]
            tr = T.FourierTracers2D(pos[0], pos[1])
        else:
            fv = g.evaluate_fourier_at_points(f, pos[0], pos[1], pos[2])
            vv = list(g.evaluate_fourier_at_points_batched_3d(vel[0], vel[1], vel[2], pos[0], pos[1], pos[2]))
            tr = T.FourierTracers3D(pos[0], pos[1], pos[2])
        for _ in range(TC.STEPS):
            tr.step(g, eq, U.copy(), TC.DT)
        out[f"{name}_f"] = np.asarray(fv)
        out[f"{name}_vel"] = np.stack(vv)
        out[f"{name}_pos"] = np.stack([tr.x] + ([tr.y] if nd > 1 else []) + ([tr.z] if nd > 2 else []))
    # a solver run with tracers (problems/base.py:1082-1102 -> solver.run(..., tracers=))
    g = grid.Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True)
    eq = equations.EulerEquations2D(gamma=1.4)
    s = solver.SpectralSolver2D(g, eq, scheme="rk4", cfl=0.4)
    U0 = problems.kelvin_helmholtz_2d(32, 32, U0=1.0, A=0.01)
    rng = np.random.default_rng(99)
    x0, y0 = rng.uniform(0, 1, 30), rng.uniform(0, 1, 30)
    tr = T.FourierTracers2D(x0, y0)
    s.run(U0.copy(), 0.0, 0.02, output_interval=1.0, tracers=tr)
    out["khi_x0"], out["khi_y0"] = x0, y0
    out["khi_pos"] = np.stack([tr.x, tr.y])
    out["khi_U"] = s.U
    np.savez_compressed(os.path.join(HERE, "tracers.npz"), **out)


def lgl1d_fixtures(grid, equations, solver, problems) -> None:
    """1D Legendre (LGL) grid with SpectralSolver1D: nodes, D, a Gaussian
    density/pressure pulse with a velocity bump between walls; rhs, RK4 steps
    with the nodal filter (cadence 2), a per-boundary/per-variable bc map
    with RK2, gravity, and the CFL dt."""
    out = {}
    for tag, n, fp, bc, scheme, grav in (
            ("wall", 33, {"enabled": True, "p": 8, "alpha": 36.0, "interval": 2}, None, "rk4", None),
            ("mixed", 41, None, {"left": {"density": "neumann", "momentum": "wall", "pressure": "open"},
                                 "right": "neumann"}, "rk2", -1.5)):
        g = grid.Grid1D(N=n, Lx=2.0, basis="legendre", bc=bc, filter_params=fp)
        x = np.asarray(g.x)
        rho = 1.0 + 0.2 * np.exp(-((x - 0.8) ** 2) / 0.02)
        p = rho ** 1.4 / 1.4
        u = 0.1 * np.sin(np.pi * x / 2.0) ** 2
        U0 = np.stack([rho, rho * u, p / 0.4 + 0.5 * rho * u * u])
        gc = {"enabled": True, "gx": grav} if grav is not None else None
        s = solver.SpectralSolver1D(g, equations.EulerEquations1D(gamma=1.4), scheme=scheme, cfl=0.4,
                                    gravity_config=gc)
        out[f"{tag}_x"] = x
        out[f"{tag}_U0"] = U0
        out[f"{tag}_rhs0"] = solver._compute_rhs(g, s.equations, U0.copy(), None, gc)
        out[f"{tag}_dt0"] = s.compute_dt(U0)
        U = U0.copy()
        for _ in range(5):
            U = s.step(U, 2e-4)
        out[f"{tag}_U"] = U
    np.savez_compressed(os.path.join(HERE, "lgl1d.npz"), **out)


def mhd1d_fixtures(grid, equations, solver, problems) -> None:
    """1D MHD (SpectralSolverMHD1D): the circularly polarized Alfven wave with
    a compressive perturbation and a non-uniform Bx (so the projection acts),
    filter on; ideal RK4 and resistive/viscous RK2 runs, plus a CFL run."""
    out = {}
    x = np.linspace(0.0, 1.0, 128, endpoint=False)
    U0 = problems.alfven_cp_1d(128)
    U0[0] *= 1.0 + 0.05 * np.sin(2 * np.pi * x)
    U0[1] = 0.02 * np.cos(4 * np.pi * x)
    U0[5] += 0.01 * np.sin(6 * np.pi * x)
    out["U0"] = U0
    for tag, cfg, scheme in (("ideal", {}, "rk4"), ("diff", {"resistivity": 0.01, "viscosity": 0.005}, "rk2")):
        g = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params={"enabled": True, "p": 8, "alpha": 36.0})
        g.mhd_config = dict(cfg)
        s = solver.SpectralSolverMHD1D(g, equations.MHDEquations1D(gamma=5.0 / 3.0), scheme=scheme, cfl=0.4)
        out[f"{tag}_rhs0"] = s._compute_rhs(U0.copy())
        out[f"{tag}_P0"] = s._project_B(U0.copy())
        U = U0.copy()
        for _ in range(4):
            U = s.step(U, 1e-3)
        out[f"{tag}_U"] = U
        out[f"{tag}_dt0"] = s.compute_dt(U0)
    g = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params={"enabled": True, "p": 8, "alpha": 36.0})
    g.mhd_config = {}
    s = solver.SpectralSolverMHD1D(g, equations.MHDEquations1D(gamma=5.0 / 3.0), cfl=0.4)
    seen = []
    s.run(U0.copy(), 0.0, 0.05, output_interval=0.05, on_step=lambda n, dt, U: seen.append(dt))
    out["cfl_U"], out["cfl_t"], out["cfl_dts"] = np.asarray(s.U), s.t, np.asarray(seen)
    np.savez_compressed(os.path.join(HERE, "mhd1d.npz"), **out)


def mhd_diffusion_fixtures(grid, equations, solver, problems) -> None:
    """2D MHD with explicit resistivity and viscosity: rhs, CFL dt (with the
    parabolic limit) and RK4 steps, filter on (32x32) and off with dealias
    off (32x16, so the Nyquist modes take part)."""
    out = {}
    for tag, (nx, ny), fp, dealias, eta, nu in (("a", (32, 32), {"enabled": True, "p": 8, "alpha": 36.0}, True,
                                                  0.02, 0.01),
                                                 ("b", (32, 16), None, False, 0.2, 0.0)):
        L = 2.0 * np.pi
        g = grid.Grid2D(Nx=nx, Ny=ny, Lx=L, Ly=L, dealias=dealias, filter_params=fp)
        g.mhd_config = {"resistivity": eta, "viscosity": nu, "project_each_substage": True,
                        "divergence_clean": "projection", "cfl_diff": 0.8}
        s = solver.SpectralSolverMHD2D(g, equations.MHDEquations2D(gamma=5.0 / 3.0), cfl=0.3)
        U0 = problems.orszag_tang_2d(nx, ny, gamma=5.0 / 3.0)
        X, Y = np.meshgrid(np.asarray(g.x), np.asarray(g.y), indexing="xy")
        U0[1] += 0.1 * np.sin(3 * X) * np.cos(2 * Y)
        U0[7] = 0.1 * np.cos(X + Y)
        U0 = s._project_B(U0)
        U = U0.copy()
        for _ in range(3):
            U = s.step(U, 1e-3)
        out[f"{tag}_U0"], out[f"{tag}_U"] = U0, U
        out[f"{tag}_rhs0"] = s._compute_rhs(U0.copy())
        out[f"{tag}_dt"] = s.compute_dt(U0)
    np.savez_compressed(os.path.join(HERE, "mhd_diffusion.npz"), **out)


def rk2_fixtures(grid, equations, solver, problems) -> None:
    """scheme="rk2" (midpoint) fixed steps of every solver: 1D Sod (filter on,
    cadence 2), 2D KHI, 3D TGV and 2D MHD Orszag-Tang."""
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    out = {}
    g1 = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params=dict(fp, interval=2))
    s1 = solver.SpectralSolver1D(g1, equations.EulerEquations1D(gamma=1.4), scheme="rk2", cfl=0.4)
    U = problems.sod_smoothed(128)
    out["sod_U0"] = U
    for _ in range(5):
        U = s1.step(U, 2e-4)
    out["sod_U"] = U
    g2 = grid.Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True, filter_params=fp)
    s2 = solver.SpectralSolver2D(g2, equations.EulerEquations2D(gamma=1.4), scheme="rk2", cfl=0.4)
    V = problems.kelvin_helmholtz_2d(32, 32, U0=1.2, A=0.015)
    out["khi_U0"] = V
    for _ in range(4):
        V = s2.step(V, 1e-3)
    out["khi_U"] = V
    g3 = grid.Grid3D(Nx=16, Ny=16, Nz=16, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, dealias=True)
    s3 = solver.SpectralSolver3D(g3, equations.EulerEquations3D(gamma=1.4), scheme="rk2", cfl=0.25)
    T = problems.taylor_green_3d(16)
    out["tgv_U0"] = T
    for _ in range(3):
        T = s3.step(T, 1e-3)
    out["tgv_U"] = T
    L = 2.0 * np.pi
    gm = grid.Grid2D(Nx=32, Ny=32, Lx=L, Ly=L, dealias=True, filter_params=fp)
    gm.mhd_config = {"resistivity": 0.0, "viscosity": 0.0, "project_each_substage": True,
                     "divergence_clean": "projection"}
    sm = solver.SpectralSolverMHD2D(gm, equations.MHDEquations2D(gamma=5.0 / 3.0), scheme="rk2", cfl=0.3)
    M = problems.orszag_tang_2d(32, 32, gamma=5.0 / 3.0)
    M = sm._project_B(M)
    out["ot_U0"] = M
    for _ in range(3):
        M = sm.step(M, 2e-3)
    out["ot_U"] = M
    np.savez_compressed(os.path.join(HERE, "rk2.npz"), **out)


def adaptive_fixtures(grid, equations, solver, problems) -> None:
    """Adaptive embedded RK through the reference's own run loops: every
    accepted attempt's (step_count, dt) from on_step, the final state and
    time.  step_count counts attempts, so its gaps are the rejections."""
    out = {}
    fp = {"enabled": True, "p": 8, "alpha": 36.0}

    def run(tag, s, U0, t_end):
        seen = []
        hist = s.run(U0.copy(), 0.0, t_end, output_interval=t_end / 2,
                     on_step=lambda n, dt, U: seen.append((n, dt)))
        out[f"{tag}_U0"] = U0
        out[f"{tag}_U"] = np.asarray(s.U)
        out[f"{tag}_t"] = s.t
        out[f"{tag}_steps"] = np.array(seen, dtype=np.float64).reshape(-1, 2)
        out[f"{tag}_hist_t"] = np.asarray(hist["time"])

    cases = [
        # tag, dim, scheme, controller overrides, t_end
        ("sod_rk45", 1, "rk45", {}, 0.01),
        ("sod_rk23_tight", 1, "rk23", {"rtol": 1e-9, "atol": 1e-11, "max_rejections": 2}, 0.003),
    ]
    for tag, _, scheme, extra, t_end in cases:
        g = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params=fp)
        cfg = dict({"enabled": True, "scheme": scheme}, **extra)
        s = solver.SpectralSolver1D(g, equations.EulerEquations1D(gamma=1.4), cfl=0.4, adaptive_config=cfg)
        run(tag, s, problems.sod_smoothed(128), t_end)
    # 1D with artificial viscosity and gravity in the stage right-hand sides
    av = {"enabled": True, "mode": "sensor", "nu_max": 2e-3, "s_ref": 1.0, "s_min": 0.1, "p": 2.0,
          "epsilon": 1e-12, "sensor_variable": "density"}
    g = grid.Grid1D(N=128, Lx=1.0, dealias=True, filter_params=fp)
    s = solver.SpectralSolver1D(g, equations.EulerEquations1D(gamma=1.4), cfl=0.4,
                                adaptive_config={"enabled": True, "scheme": "rk45"},
                                artificial_viscosity_config=av, gravity_config={"enabled": True, "gx": -2.0})
    run("sod_av_grav_rk45", s, problems.sod_smoothed(128), 0.005)
    # 2D KHI with gravity (its adaptive right-hand side has no viscosity)
    g2 = grid.Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True, filter_params=fp)
    s2 = solver.SpectralSolver2D(g2, equations.EulerEquations2D(gamma=1.4), cfl=0.4,
                                 adaptive_config={"enabled": True, "scheme": "rk23", "rtol": 1e-7},
                                 gravity_config={"enabled": True, "gx": 0.3, "gy": -1.0})
    run("khi_rk23", s2, problems.kelvin_helmholtz_2d(32, 32, U0=1.2, A=0.015), 0.02)
    # 3D TGV with the reference's 8-stage "rk78"
    g3 = grid.Grid3D(Nx=16, Ny=16, Nz=16, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, dealias=True)
    s3 = solver.SpectralSolver3D(g3, equations.EulerEquations3D(gamma=1.4), cfl=0.25,
                                 adaptive_config={"enabled": True, "scheme": "rk78", "rtol": 1e-7})
    run("tgv_rk78", s3, problems.taylor_green_3d(16), 0.05)
    # 2D MHD Orszag-Tang with a divergent B perturbation (run projects U0 first)
    L = 2.0 * np.pi
    gm = grid.Grid2D(Nx=32, Ny=32, Lx=L, Ly=L, dealias=True, filter_params=fp)
    gm.mhd_config = {"resistivity": 0.0, "viscosity": 0.0, "project_each_substage": True,
                     "divergence_clean": "projection"}
    sm = solver.SpectralSolverMHD2D(gm, equations.MHDEquations2D(gamma=5.0 / 3.0), cfl=0.3,
                                    adaptive_config={"enabled": True, "scheme": "rk45"})
    M0 = problems.orszag_tang_2d(32, 32, gamma=5.0 / 3.0)
    X, Y = np.meshgrid(np.asarray(gm.x), np.asarray(gm.y), indexing="xy")
    M0[5] += 0.05 * np.cos(X) * np.cos(2.0 * Y)
    run("ot_rk45", sm, M0, 0.15)
    np.savez_compressed(os.path.join(HERE, "adaptive.npz"), **out)


def mhd_fixtures(grid, equations, solver, problems) -> None:
    """2D ideal MHD: Orszag-Tang (rho = gamma^2, p = gamma, B0 = 1 on
    [0, 2 pi)^2) plus a divergent perturbation of B that the projection
    removes and an out-of-plane field; NumPy backend."""
    for (nx, ny), fon, nsteps, dt in (((32, 32), True, 3, 2e-3), ((32, 16), False, 2, 2e-3)):
        fp = {"enabled": True, "p": 8, "alpha": 36.0} if fon else None
        L = 2.0 * np.pi
        g = grid.Grid2D(Nx=nx, Ny=ny, Lx=L, Ly=L, dealias=True, filter_params=fp)
        g.mhd_config = {"resistivity": 0.0, "viscosity": 0.0, "project_each_substage": True,
                        "divergence_clean": "projection"}
        eq = equations.MHDEquations2D(gamma=5.0 / 3.0)
        s = solver.SpectralSolverMHD2D(g, eq, scheme="rk4", cfl=0.3)
        U0 = problems.orszag_tang_2d(nx, ny, gamma=5.0 / 3.0)
        X, Y = np.meshgrid(np.asarray(g.x), np.asarray(g.y), indexing="xy")
        U0[5] += 0.05 * np.cos(X) * np.cos(2.0 * Y)   # div B != 0
        U0[6] += 0.03 * np.sin(3.0 * X) * np.sin(Y)
        U0[7] = 0.1 * np.cos(X + Y)                     # out-of-plane field
        rhs0 = s._compute_rhs(U0.copy())
        P0 = s._project_B(U0.copy())
        U = U0.copy()
        for _ in range(nsteps):
            U = s.step(U, dt)
        cons0 = eq.conserved_quantities(U0)
        np.savez_compressed(os.path.join(HERE, f"mhd2d_{nx}x{ny}.npz"), U0=U0, rhs0=rhs0, P0=P0, U=U, dt=dt,
                            nsteps=nsteps, filter=int(fon), dt_cfl0=s.compute_dt(U0),
                            cons0=np.array([cons0[k] for k in ("mass", "momentum_x", "momentum_y", "momentum_z",
                                                               "energy", "magnetic_energy", "cross_helicity")]),
                            divb_P0=s.max_div_b(P0), divb_U0=s.max_div_b(U0))


# (problem name, shipped config file, grid overrides) for the initial-condition
# fixtures: each shipped config of a registered problem, at a small grid
PROBLEM_CASES = [
    ("sod", "sod.yaml", {"N": 64}),
    ("sod", "legendre_sod.yaml", {"N": 33}),
    ("acoustic1d", "acoustic1d.yaml", {"N": 64}),
    ("gaussian_wave1d", "gaussian_wave_traveling.yaml", {"N": 64}),
    ("gaussian_wave1d", "acoustic_legendre_dirichlet.yaml", {"N": 33}),
    ("shu_osher1d", "shu_osher1d.yaml", {"N": 64}),
    ("hse_1d", "hse_1d_test.yaml", {"N": 33}),
    ("rti_1d", "rti_1d_athena.yaml", {"N": 33}),
    ("alfven1d", "alfven1d.yaml", {"N": 64}),
    ("khi2d", "khi2d.yaml", {"Nx": 32, "Ny": 16}),
    ("khi2d", "khi2d_4k.yaml", {"Nx": 48, "Ny": 27}),
    ("uniform_2d", "uniform_2d_small.yaml", {"Nx": 9, "Ny": 9}),
    ("rti", "rti.yaml", {"Nx": 17, "Ny": 33}),
    ("gaussian_wave2d", "gaussian_wave2d.yaml", {"Nx": 17, "Ny": 17}),
    ("gaussian_wave2d_y", "gaussian_wave2d_y.yaml", {"Nx": 17, "Ny": 17}),
    ("orszag_tang2d", "orszag_tang2d.yaml", {"Nx": 32, "Ny": 16}),
    ("tgv3d", "tgv3d.yaml", {"Nx": 16, "Ny": 16, "Nz": 8}),
    ("turb3d", "turb3d.yaml", {"Nx": 16, "Ny": 16, "Nz": 16}),
    ("alfven3d", "alfven3d.yaml", {"Nx": 16, "Ny": 8, "Nz": 8}),
    ("mhd_turb3d", "mhd_turb3d.yaml", {"Nx": 16, "Ny": 16, "Nz": 16}),
]


def problem_ic_fixtures(ref_path: str) -> None:
    """Initial states of the reference's registered problems from its shipped
    configs (grids shrunk): the config (read with phrike_gb300.config.load_yaml,
    PyYAML being absent), the reference grid's node coordinates in their own
    dtype, and the problem's create_initial_conditions(grid).  Written to
    problem_ics.npz."""
    import json
    import tempfile
    from phrike.problems import ProblemRegistry
    from phrike.problems import register  # noqa: F401
    from phrike_gb300.config import load_yaml
    out = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)  # the problems create their output directories
        try:
            for i, (name, fname, over) in enumerate(PROBLEM_CASES):
                with open(os.path.join(ref_path, "configs", fname)) as f:
                    cfg = load_yaml(f.read())
                cfg["grid"].update(over)
                cfg.setdefault("io", {})["outdir"] = os.path.join(tmp, f"case{i}")
                prob = ProblemRegistry.create_problem(name, config=json.loads(json.dumps(cfg)))
                grid = prob.create_grid("numpy", None, False)
                U0 = np.asarray(prob.create_initial_conditions(grid), dtype=np.float64)
                out[f"c{i}_name"] = name
                out[f"c{i}_file"] = fname
                out[f"c{i}_config"] = json.dumps(cfg)
                out[f"c{i}_gamma"] = prob.gamma
                for ax in ("x", "y", "z"):
                    if getattr(grid, ax, None) is not None:
                        out[f"c{i}_{ax}"] = np.asarray(getattr(grid, ax))  # native dtype (float32 for single)
                out[f"c{i}_L"] = np.array([float(getattr(grid, a)) for a in ("Lx", "Ly", "Lz") if hasattr(grid, a)])
                out[f"c{i}_legendre"] = int(getattr(grid, "_legendre_basis", None) is not None
                                            or str(getattr(grid, "basis", "fourier")).lower() == "legendre"
                                            or str(getattr(grid, "basis_x", "fourier")).lower() == "legendre")
                out[f"c{i}_U0"] = U0
                print(name, fname, U0.shape)
        finally:
            os.chdir(cwd)
    out["ncases"] = len(PROBLEM_CASES)
    np.savez_compressed(os.path.join(HERE, "problem_ics.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", sys.argv[2] if len(sys.argv) > 2 else "")
