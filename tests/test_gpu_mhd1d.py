"""1D MHD (SpectralSolverMHD1D) on the GPU against the reference's own runs
(tests/golden/mhd1d.npz): right-hand side, the 1D projection, ideal RK4 and
resistive/viscous RK2 steps, the CFL run through the solver API, and the
circularly polarized Alfven wave after one period against its exact
solution."""
import numpy as np
import pytest

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu

FP = {"enabled": True, "p": 8, "alpha": 36.0}


def _errs(G, R):
    G = np.asarray(G, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    floor = 1e-2 * np.linalg.norm(R)
    return [float(np.linalg.norm(G[g] - R[g]) / max(np.linalg.norm(R[g]), floor))
            for g in (slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8))]


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda").contiguous()


@pytest.mark.parametrize("tag", ["ideal", "diff"])
def test_mhd1d_matches_reference(tag, cuda_device):
    from phrike_gb300.engine import Plan
    z = golden("mhd1d.npz")
    mc = {"resistivity": 0.01, "viscosity": 0.005} if tag == "diff" else {}
    plan = Plan((128,), (1.0,), gamma=5.0 / 3.0, filter_params=FP, equations="mhd", mhd_config=mc, cfl=0.4,
                scheme="rk2" if tag == "diff" else "rk4")
    U0 = _dev(z["U0"])
    assert max(_errs(plan.rhs(U0).cpu().numpy(), z[f"{tag}_rhs0"])) < 2e-5
    P = U0.clone()
    plan.project_state_(P)
    assert rel_l2(P.cpu().numpy(), z[f"{tag}_P0"]) < 1e-6
    U = U0.clone()
    plan.run_(U, 4, 1e-3)
    assert max(_errs(U.cpu().numpy(), z[f"{tag}_U"])) < 2e-5


def test_mhd1d_cfl_run_matches_reference(cuda_device):
    from phrike_gb300.equations import MHDEquations1D
    from phrike_gb300.grid import Grid1D
    from phrike_gb300.solver import SpectralSolverMHD1D
    z = golden("mhd1d.npz")
    g = Grid1D(N=128, Lx=1.0, dealias=True, filter_params=FP, backend="gb300")
    g.mhd_config = {}
    s = SpectralSolverMHD1D(g, MHDEquations1D(gamma=5.0 / 3.0), cfl=0.4)
    dts = []
    hist = s.run(z["U0"], 0.0, 0.05, output_interval=0.05, on_step=lambda n, dt, U: dts.append(dt))
    np.testing.assert_allclose(dts, z["cfl_dts"], rtol=2e-5)
    assert abs(s.t - float(z["cfl_t"])) < 1e-9
    assert max(_errs(s.U.cpu().numpy(), z["cfl_U"])) < 2e-5
    assert max(hist["div_b_max"]) < 1e-4
    # the device CFL loop takes the same steps
    import torch
    from phrike_gb300.engine import Plan
    plan = Plan((128,), (1.0,), gamma=5.0 / 3.0, filter_params=FP, equations="mhd", cfl=0.4)
    U = _dev(z["U0"])
    plan.project_state_(U)
    t = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    te = torch.full((1,), 0.05, dtype=torch.float64, device=cuda_device)
    plan.run_cfl_(U, 1000, t, te)
    assert plan.steps_done()[0] == len(dts)
    assert max(_errs(U.cpu().numpy(), z["cfl_U"])) < 2e-5


def test_alfven_wave_one_period(cuda_device):
    """The circularly polarized Alfven wave is an exact nonlinear solution:
    after one period (t = L / c_A) the state returns to the initial one up to
    the time-stepping error (float32, N = 64)."""
    import torch
    from phrike_gb300 import problems
    from phrike_gb300.engine import Plan
    N, T = 64, 1.0
    plan = Plan((N,), (1.0,), gamma=5.0 / 3.0, filter_params=FP, equations="mhd", cfl=0.4)
    U0 = problems.alfven_cp_1d(N)
    U = _dev(U0)
    t = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    te = torch.full((1,), T, dtype=torch.float64, device=cuda_device)
    plan.run_cfl_(U, 100000, t, te)
    G = U.cpu().numpy()
    err = float(np.sqrt(np.mean((G[6] - U0[6]) ** 2 + (G[7] - U0[7]) ** 2)))
    assert err < 1e-4 * 0.1, err
    assert np.allclose(G[5], 1.0, atol=1e-6)
