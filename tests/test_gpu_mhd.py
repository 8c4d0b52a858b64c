"""2D ideal MHD on the GPU against the oracle and the reference's golden
vectors: right-hand side, the Helmholtz projection (div B), RK4 steps with
per-stage clamp and projection, the filter cadence, CFL runs, batches and the
reference-shaped solver API.

Tolerances: float32 state and float32 FFTs.  The Orszag-Tang state is O(1),
so right-hand sides and short runs agree with the float64 reference to a few
1e-7 relative per field; div B after a projection is at the float32
rounding level of B times the largest wavenumber.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import mhd as M
from phrike_gb300 import problems

pytestmark = pytest.mark.gpu

G53 = 5.0 / 3.0
TWO_PI = 2.0 * np.pi


def _plan(nx, ny, nsolve=1, filt=None, cfl=0.3, **mc):
    from phrike_gb300.engine import Plan
    return Plan((ny, nx), (TWO_PI, TWO_PI), gamma=G53, filter_params=filt, cfl=cfl, nsolve=nsolve,
                equations="mhd", mhd_config=mc or None)


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


def _errs(G, R):
    """L2 errors of density, momentum (vector), energy and B (vector), each
    relative to its group's norm with a floor of 1e-2 of the whole state's
    norm: the Orszag-Tang flow is divergence-free, so the density right-hand
    side is nearly zero and judged against the others' scale."""
    G = np.asarray(G, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    floor = 1e-2 * np.linalg.norm(R)
    out = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8)):
        out.append(float(np.linalg.norm(G[sl] - R[sl]) / max(np.linalg.norm(R[sl]), floor)))
    return out


@pytest.mark.parametrize("nx,ny", [(32, 32), (32, 16)])
def test_mhd_matches_reference(cuda_device, nx, ny):
    z = golden(f"mhd2d_{nx}x{ny}.npz")
    fp = {"enabled": True, "p": 8, "alpha": 36.0} if int(z["filter"]) else None
    p = _plan(nx, ny, filt=fp)
    U0 = _dev(z["U0"])
    rhs = p.rhs(U0).cpu().numpy()
    assert max(_errs(rhs, z["rhs0"])) < 2e-5, _errs(rhs, z["rhs0"])
    P = _dev(z["U0"])
    p.project_state_(P)
    P = P.cpu().numpy()
    assert max(_errs(P, z["P0"])) < 1e-6, _errs(P, z["P0"])
    s = M.MHDSolver2D(nx, ny, filter_params=fp)
    assert s.max_div_b(P.astype(np.float64)) < 1e-5
    U = _dev(z["U0"])
    p.run_(U, int(z["nsteps"]), float(z["dt"]))
    G = U.cpu().numpy()
    assert max(_errs(G, z["U"])) < 2e-6, _errs(G, z["U"])
    cons = p.conserved(_dev(z["U0"])).cpu().numpy()
    np.testing.assert_allclose(cons[:7], z["cons0"], rtol=1e-6, atol=1e-4)
    sp = float(p.max_wave_speed(_dev(z["U0"])).item())
    dt = 0.3 * TWO_PI / nx / sp
    assert abs(dt - float(z["dt_cfl0"])) < 1e-6 * float(z["dt_cfl0"])
    assert p.status() == 0


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_mhd_orszag_tang_vs_oracle(cuda_device, n):
    """Orszag-Tang (rho = gamma^2, p = gamma, B0 = 1), filter on, 10 steps of
    dt = 1e-3 against the float64 oracle; every pencil length of the serving
    range including the grouped 512-point pencils."""
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = problems.orszag_tang_2d(n, n, gamma=G53)
    s = M.MHDSolver2D(n, n, filter_params=fp)
    R = s.project(U0)
    for _ in range(10):
        R = s.step(R, 1e-3)
    p = _plan(n, n, filt=fp)
    U = _dev(U0)
    p.project_state_(U)
    p.run_(U, 10, 1e-3)
    G = U.cpu().numpy()
    errs = _errs(G, R)
    assert max(errs) < 5e-6, errs
    assert s.max_div_b(G.astype(np.float64)) < 2e-4
    assert p.status() == 0


def test_mhd_batch_matches_alone(cuda_device):
    import torch
    n = 64
    states = [problems.orszag_tang_2d(n, n, gamma=G53, B0=b) for b in (1.0, 0.5, 0.8)]
    pb = _plan(n, n, nsolve=3)
    Ub = _dev(np.stack(states))
    pb.run_(Ub, 5, 2e-3)
    for i, st in enumerate(states):
        p1 = _plan(n, n)
        U1 = _dev(st)
        p1.run_(U1, 5, 2e-3)
        assert torch.equal(U1, Ub[i]), i


def test_mhd_batch_of_sixteen_256_matches_alone(cuda_device):
    """On 256^2 grids the last pass is split into the right-hand side and an
    elementwise update; a batch of sixteen runs the passes in other shapes
    than a solve alone: the MHD x pass with its 8 transform jobs in one CTA
    instead of one job per CTA, the projection's x passes 8 pencils per CTA
    instead of 2 and its y pass 4 columns instead of 2, the right-hand side
    8 columns with all component pairs in one CTA instead of 4 columns with
    one pair per CTA.  Each pencil's arithmetic is the same in every shape:
    the states are bit-identical."""
    import torch
    n = 256
    states = [problems.orszag_tang_2d(n, n, gamma=G53, B0=0.5 + 0.05 * b) for b in range(16)]
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    pb = _plan(n, n, nsolve=16, filt=fp)
    Ub = _dev(np.stack(states))
    pb.run_(Ub, 3, 1e-3)
    for i in (0, 9, 15):
        p1 = _plan(n, n, filt=fp)
        U1 = _dev(states[i])
        p1.run_(U1, 3, 1e-3)
        assert torch.equal(U1, Ub[i]), i
    assert pb.status() == 0


def test_mhd_cfl_run_vs_oracle(cuda_device):
    import torch
    n, t_end = 64, 0.05
    U0 = problems.orszag_tang_2d(n, n, gamma=G53)
    s = M.MHDSolver2D(n, n, cfl=0.3)
    R, t, steps = U0.copy(), 0.0, 0
    while t < t_end - 1e-12:
        dt = min(s.compute_dt(R), t_end - t)
        R = s.step(R, dt)
        t += dt
        steps += 1
    p = _plan(n, n, cfl=0.3)
    U = _dev(U0)
    tt = torch.zeros(1, dtype=torch.float64, device="cuda")
    te = torch.full((1,), t_end, dtype=torch.float64, device="cuda")
    p.run_cfl_(U, steps + 2, tt, te)
    assert abs(float(tt.item()) - t_end) < 1e-12
    assert p.steps_done() == [steps]
    assert max(_errs(U.cpu().numpy(), R)) < 5e-6


def test_mhd_solver_api_and_projection_helpers(cuda_device):
    """SpectralSolverMHD2D.run (projects U0 first, CFL loop, history keys)
    and Grid2D.project_solenoidal / divergence against the oracle."""
    from phrike_gb300.equations import MHDEquations2D
    from phrike_gb300.grid import Grid2D
    from phrike_gb300.solver import SpectralSolverMHD2D
    n = 32
    z = golden("mhd2d_32x32.npz")
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    grid = Grid2D(Nx=n, Ny=n, Lx=TWO_PI, Ly=TWO_PI, filter_params=fp, backend="gb300")
    grid.mhd_config = {"resistivity": 0.0, "viscosity": 0.0}
    bx, by = grid.project_solenoidal(z["U0"][5], z["U0"][6])
    assert rel_l2(bx.cpu().numpy(), z["P0"][5]) < 1e-6 and rel_l2(by.cpu().numpy(), z["P0"][6]) < 1e-6
    assert float(grid.divergence(bx, by).abs().max()) < 1e-5
    solver = SpectralSolverMHD2D(grid, MHDEquations2D(gamma=G53), cfl=0.3)
    hist = solver.run(z["U0"], 0.0, 0.02, output_interval=0.01)
    s = M.MHDSolver2D(n, n, filter_params=fp, cfl=0.3)
    R, t = s.project(z["U0"]), 0.0
    while t < 0.02 - 1e-12:
        dt = min(s.compute_dt(R), 0.02 - t)
        R = s.step(R, dt)
        t += dt
    assert max(_errs(solver.U.cpu().numpy(), R)) < 5e-6
    for key in ("mass", "energy", "magnetic_energy", "cross_helicity", "div_b_max"):
        assert key in hist and len(hist[key]) == len(hist["time"])
    assert max(hist["div_b_max"]) < 1e-4
    assert abs(hist["mass"][-1] - hist["mass"][0]) < 1e-6 * abs(hist["mass"][0])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_mhd_resistivity_viscosity_match_reference(tag, cuda_device):
    """Explicit resistivity eta lap(B) and viscosity nu lap(rho u) (the
    spectral Laplacian with mask and filter; case b without dealiasing, so the
    Nyquist modes take part) against the reference: right-hand side, the CFL
    dt with the parabolic limit, and three RK4 steps."""
    import torch
    from phrike_gb300.engine import Plan
    from phrike_gb300.grid import Grid2D
    from phrike_gb300.equations import MHDEquations2D
    from phrike_gb300.solver import SpectralSolverMHD2D
    z = golden("mhd_diffusion.npz")
    (nx, ny), fp, dealias, eta, nu = {"a": ((32, 32), {"enabled": True, "p": 8, "alpha": 36.0}, True, 0.02, 0.01),
                                      "b": ((32, 16), None, False, 0.2, 0.0)}[tag]
    mc = {"resistivity": eta, "viscosity": nu, "cfl_diff": 0.8}
    plan = Plan((ny, nx), (2 * np.pi, 2 * np.pi), gamma=5.0 / 3.0, dealias=dealias, filter_params=fp,
                equations="mhd", mhd_config=mc)
    U0 = torch.as_tensor(z[f"{tag}_U0"], dtype=torch.float32, device=cuda_device).contiguous()
    rhs = plan.rhs(U0).double().cpu().numpy()
    assert max(_errs(rhs, z[f"{tag}_rhs0"])) < 2e-5, _errs(rhs, z[f"{tag}_rhs0"])
    U = U0.clone()
    plan.run_(U, 3, 1e-3)
    assert max(_errs(U.double().cpu().numpy(), z[f"{tag}_U"])) < 2e-5
    g = Grid2D(Nx=nx, Ny=ny, Lx=2 * np.pi, Ly=2 * np.pi, dealias=dealias, filter_params=fp, backend="gb300")
    g.mhd_config = mc
    s = SpectralSolverMHD2D(g, MHDEquations2D(gamma=5.0 / 3.0), cfl=0.3)
    dt = s.compute_dt(U0)
    assert abs(dt - float(z[f"{tag}_dt"])) < 1e-5 * float(z[f"{tag}_dt"])
    # the device CFL loop applies the same cap: one step from t = 0 takes that dt
    t = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    te = torch.ones(1, dtype=torch.float64, device=cuda_device)
    plan.run_cfl_(U0.clone(), 1, t, te)
    assert abs(t.item() - dt) < 1e-5 * dt
