"""3D ideal and resistive MHD on the GPU against the reference's vectors and
the float64 oracle: right-hand side (flux divergence, eta lap B, nu lap(rho u)),
the 3D Helmholtz projection (div B), RK4/RK2 steps with per-stage clamp and
projection and the filter cadence, the CFL loop, batches and the solver API.

Tolerances: float32 state and float32 FFTs; errors are per group (density,
momentum, energy, B), relative to the group's norm with a floor of 1e-2 of
the state's norm (the Alfven wave's density right-hand side is exactly zero).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _errs(G, R):
    G = np.asarray(G, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    floor = 1e-2 * np.linalg.norm(R)
    return [float(np.linalg.norm(G[sl] - R[sl]) / max(np.linalg.norm(R[sl]), floor))
            for sl in (slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8))]


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


def _plan(name, nsolve=1, cfl=0.3):
    import mhd3d_cases as MC
    from phrike_gb300.engine import Plan
    nx, ny, nz, lx, ly, lz, filt, cfg, scheme = MC.CASES[name][:9]
    return Plan((nz, ny, nx), (lz, ly, lx), gamma=MC.GAMMA, filter_params=filt, cfl=cfl, nsolve=nsolve,
                equations="mhd", mhd_config=dict(cfg), scheme=scheme)


@pytest.mark.parametrize("name", ["alfven", "turb"])
def test_mhd3d_matches_reference(cuda_device, name):
    import mhd3d_cases as MC
    from oracle import mhd as M
    z = golden("mhd3d.npz")
    nx, ny, nz, lx, ly, lz, filt, cfg, scheme, dt, nsteps = MC.CASES[name]
    p = _plan(name)
    rhs = p.rhs(_dev(z[f"{name}_U0"])).cpu().numpy()
    assert max(_errs(rhs, z[f"{name}_rhs0"])) < 2e-5, _errs(rhs, z[f"{name}_rhs0"])
    P = _dev(z[f"{name}_U0"])
    p.project_state_(P)
    P = P.cpu().numpy()
    assert max(_errs(P, z[f"{name}_P0"])) < 1e-6, _errs(P, z[f"{name}_P0"])
    s = M.MHDSolver3D(nx, ny, nz, lx, ly, lz, gamma=MC.GAMMA, filter_params=filt)
    assert s.max_div_b(P.astype(np.float64)) < 2e-5
    U = _dev(z[f"{name}_U0"])
    p.run_(U, nsteps, dt)
    G = U.cpu().numpy()
    assert max(_errs(G, z[f"{name}_U"])) < 2e-6, _errs(G, z[f"{name}_U"])
    cons = p.conserved(U).cpu().numpy()
    np.testing.assert_allclose(cons[:7], z[f"{name}_cons"], rtol=2e-6, atol=2e-3)
    sp = float(p.max_wave_speed(_dev(z[f"{name}_U0"])).item())
    dt0 = 0.3 * min(lx / nx, ly / ny, lz / nz) / sp
    if cfg:  # the parabolic cap of explicit diffusion
        k2 = sum((np.pi * n / L) ** 2 for n, L in ((nx, lx), (ny, ly), (nz, lz)))
        dt0 = min(dt0, 1.0 / (max(cfg.values()) * k2))
    assert abs(dt0 - float(z[f"{name}_dt0"])) < 1e-6 * float(z[f"{name}_dt0"])
    assert p.status() == 0


def test_mhd3d_cfl_run_matches_reference(cuda_device):
    """The device CFL loop to t = 0.05 (Alfven wave, filter on) takes the
    reference's step sequence."""
    import torch
    import mhd3d_cases as MC
    z = golden("mhd3d.npz")
    p = _plan("alfven")
    U = _dev(MC.initial_state("alfven"))
    p.project_state_(U)  # run() projects U0 first (solver.py:1117-1118)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    te = torch.full((1,), 0.05, dtype=torch.float64, device="cuda")
    p.run_cfl_(U, 50, t, te)
    assert abs(float(t.item()) - 0.05) < 1e-12
    assert p.steps_done() == [len(z["cfl_dts"])]
    assert max(_errs(U.cpu().numpy(), z["cfl_U"])) < 2e-6


def test_mhd3d_batch_matches_alone(cuda_device):
    import torch
    import mhd3d_cases as MC
    U0 = MC.initial_state("turb")
    states = [U0, U0 * np.array([1, 1.1, 0.9, 1, 1, 1, 1, 1])[:, None, None, None]]
    pb = _plan("turb", nsolve=2)
    Ub = _dev(np.stack(states))
    pb.run_(Ub, 3, 1e-3)
    for i, st in enumerate(states):
        p1 = _plan("turb")
        U1 = _dev(st)
        p1.run_(U1, 3, 1e-3)
        assert torch.equal(U1, Ub[i]), i


@pytest.mark.parametrize("n", [32, 64])
def test_mhd3d_projection_properties(cuda_device, n):
    """A random B on n^3 (and an anisotropic box): after the projection div B
    is at float32 rounding, a second projection changes nothing beyond
    rounding, and the projection matches the oracle."""
    from oracle import mhd as M
    from oracle.spectral import FourierBox
    from phrike_gb300.grid import Grid3D
    rng = np.random.default_rng(n)
    L = (2.0, 1.0, 3.0)
    g = Grid3D(Nx=n, Ny=n // 2, Nz=n, Lx=L[0], Ly=L[1], Lz=L[2])
    B = [rng.standard_normal((n, n // 2, n)).astype(np.float32) for _ in range(3)]
    bx, by, bz = g.project_solenoidal(*B)
    box = FourierBox((n, n // 2, n), (L[2], L[1], L[0]), dealias=True)
    want = M.project_solenoidal_3d(box, *[b.astype(np.float64) for b in B])
    for got, w in zip((bx, by, bz), want):
        assert np.linalg.norm(got.cpu().numpy() - w) < 5e-6 * np.linalg.norm(w)
    div = g.divergence(bx, by, bz).abs().max().item()
    scale = max(b.abs().max().item() for b in (bx, by, bz)) * np.pi * n / min(L)
    assert div < 1e-5 * scale
    cx, cy, cz = g.project_solenoidal(bx, by, bz)
    for a, b in ((bx, cx), (by, cy), (bz, cz)):
        assert (a - b).abs().max().item() < 1e-5 * a.abs().max().item()


def test_mhd3d_solver_api(cuda_device):
    """SpectralSolverMHD3D.run with the reference-shaped history (including
    magnetic energy, cross helicity and div B) on the Alfven wave."""
    import mhd3d_cases as MC
    from phrike_gb300.equations import MHDEquations3D
    from phrike_gb300.grid import Grid3D
    from phrike_gb300.solver import SpectralSolverMHD3D
    z = golden("mhd3d.npz")
    g = Grid3D(Nx=32, Ny=8, Nz=8, Lx=1.0, Ly=1.0, Lz=1.0, filter_params=dict(MC.FILTER))
    g.mhd_config = {}
    s = SpectralSolverMHD3D(g, MHDEquations3D(gamma=MC.GAMMA), cfl=0.3)
    seen = []
    h = s.run(MC.initial_state("alfven"), 0.0, 0.05, output_interval=0.05, on_step=lambda n, dt, U: seen.append(dt))
    np.testing.assert_allclose(seen, z["cfl_dts"], rtol=1e-5)
    assert max(_errs(s.U.cpu().numpy(), z["cfl_U"])) < 2e-6
    assert h["div_b_max"][-1] < 1e-4 and len(h["magnetic_energy"]) == len(h["time"])
