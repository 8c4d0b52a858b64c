"""Batched solves (one plan, many independent solves of one grid) and the
device-side CFL time loop.  Each solve of a batch must give the same result
as the same solve run alone (same kernels and arithmetic per solve:
tolerance 1e-6 relative L2), and CFL runs must follow the oracle's run loop
(dt sequence and end state, 1e-5)."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import spectral as O
from phrike_gb300 import problems
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu


def dev(x, device):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device=device)


def test_batch_3d_matches_solves_alone(cuda_device):
    N = 16
    rng = np.random.default_rng(11)
    U0 = np.stack([problems.taylor_green_3d(N) * (1.0 + 0.1 * rng.random()) for _ in range(3)])
    U0[:, 4] = problems.taylor_green_3d(N)[4]  # keep the energy positive and O(1e2)
    batch = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device, nsolve=3)
    Ub = dev(U0, cuda_device)
    batch.run_(Ub, 3, 1e-3)
    out = Ub.double().cpu().numpy()
    for s in range(3):
        one = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device)
        U1 = dev(U0[s], cuda_device)
        one.run_(U1, 3, 1e-3)
        assert rel_l2(out[s], U1.double().cpu().numpy()) < 1e-6
    assert batch.status() == 0
    cons = batch.conserved(Ub).cpu().numpy()
    assert cons.shape == (3, 5)


def test_batch_2d_cfl_run_matches_oracle(cuda_device):
    N = 64
    params = [(1.0, 0.01), (0.7, 0.02), (1.3, 0.005), (1.1, 0.015)]
    U0 = np.stack([problems.kelvin_helmholtz_2d(N, N, U0=u, A=a) for u, a in params])
    tend = np.array([0.01, 0.02, 0.005, 0.015])
    plan = Plan((N, N), (1.0, 1.0), cfl=0.4, device=cuda_device, nsolve=4)
    U = dev(U0, cuda_device)
    t = torch.zeros(4, dtype=torch.float64, device=cuda_device)
    te = torch.as_tensor(tend, device=cuda_device)
    plan.run_cfl_(U, 400, t, te)
    torch.cuda.synchronize()
    np.testing.assert_allclose(t.cpu().numpy(), tend, rtol=0, atol=1e-12)
    out = U.double().cpu().numpy()
    for s in range(4):
        o = O.EulerSolver(O.FourierBox((N, N), (1.0, 1.0), dealias=True), cfl=0.4)
        ref, tt, dts = o.run(U0[s].astype(np.float32).astype(np.float64), 0.0, float(tend[s]))
        for c in (0, 1, 3):
            assert rel_l2(out[s][c], ref[c]) < 1e-5, (s, c, rel_l2(out[s][c], ref[c]))
    assert plan.status() == 0


def test_batch_1d_cfl_run_matches_oracle(cuda_device):
    N = 256
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = np.stack([problems.sod_smoothed(N), problems.sod_smoothed(N, width=0.01)])
    tend = np.array([0.002, 0.003])
    plan = Plan((N,), (1.0,), filter_params=fp, cfl=0.4, device=cuda_device, nsolve=2)
    U = dev(U0, cuda_device)
    t = torch.zeros(2, dtype=torch.float64, device=cuda_device)
    plan.run_cfl_(U, 10000, t, torch.as_tensor(tend, device=cuda_device))
    torch.cuda.synchronize()
    np.testing.assert_allclose(t.cpu().numpy(), tend, rtol=0, atol=1e-12)
    out = U.double().cpu().numpy()
    for s in range(2):
        o = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True), cfl=0.4)
        ref, tt, dts = o.run(U0[s].astype(np.float32).astype(np.float64), 0.0, float(tend[s]))
        for c in (0, 2):
            assert rel_l2(out[s][c], ref[c]) < 1e-5, (s, c, rel_l2(out[s][c], ref[c]))


def test_solve_alone_vs_in_the_mix_2d(cuda_device):
    """The same solve in a batch of 8 (others with different data and end
    times) and alone: identical within 1e-6."""
    N = 32
    rng = np.random.default_rng(7)
    U0 = np.stack([problems.kelvin_helmholtz_2d(N, N, U0=0.5 + rng.random(), A=0.005 + 0.015 * rng.random())
                   for _ in range(8)])
    tend = 0.005 + 0.01 * rng.random(8)
    plan = Plan((N, N), (1.0, 1.0), cfl=0.4, device=cuda_device, nsolve=8)
    U = dev(U0, cuda_device)
    t = torch.zeros(8, dtype=torch.float64, device=cuda_device)
    plan.run_cfl_(U, 500, t, torch.as_tensor(tend, device=cuda_device))
    mix = U.double().cpu().numpy()
    for s in (0, 5):
        one = Plan((N, N), (1.0, 1.0), cfl=0.4, device=cuda_device, nsolve=1)
        U1 = dev(U0[s], cuda_device)
        t1 = torch.zeros(1, dtype=torch.float64, device=cuda_device)
        one.run_cfl_(U1, 500, t1, torch.as_tensor(tend[s:s + 1], device=cuda_device))
        assert rel_l2(mix[s], U1.double().cpu().numpy()) < 1e-6


def test_ensemble_uneven_sizes_graphs(cuda_device):
    """Ensemble of KHI solves on two grids advanced with captured CUDA graphs:
    every solve reaches its own end time and equals the solve run alone."""
    from phrike_gb300.ensemble import Ensemble, SolveSpec
    rng = np.random.default_rng(3)
    specs = []
    for n in (32, 64, 32, 64, 32):
        specs.append(SolveSpec((n, n), (1.0, 1.0),
                               problems.kelvin_helmholtz_2d(n, n, U0=0.5 + rng.random(), A=0.01),
                               t_end=0.004 + 0.006 * rng.random()))
    ens = Ensemble(specs, cfl=0.4, device=cuda_device)
    stats = ens.run(chunk=7, use_graphs=True)
    assert stats["status"] == 0
    for i, sp in enumerate(specs):
        assert abs(ens.time(i) - sp.t_end) < 1e-12
        alone = Plan(sp.shape, sp.lengths, cfl=0.4, device=cuda_device)
        U1 = dev(sp.U0, cuda_device)
        t1 = torch.zeros(1, dtype=torch.float64, device=cuda_device)
        alone.run_cfl_(U1, 200, t1, torch.tensor([sp.t_end], dtype=torch.float64, device=cuda_device))
        assert rel_l2(ens.state(i).double().cpu().numpy(), U1.double().cpu().numpy()) < 1e-6


def test_autotuned_tile_widths_change_speed_only(cuda_device):
    """Every allowed strided-pass tile width gives the same state bit for bit
    (the pencil arithmetic does not depend on it); the autotuner returns one
    of them with its timing table."""
    from phrike_gb300.autotune import tune_tile_cols
    N, ns = 128, 4
    U0 = np.stack([problems.kelvin_helmholtz_2d(N, N, U0=1.0 + 0.1 * i, A=0.01) for i in range(ns)])
    U = dev(U0, cuda_device)
    best, times = tune_tile_cols((N, N), (1.0, 1.0), U, nsolve=ns, cfl=0.4, device=cuda_device)
    assert best in times and set(times) <= {4, 8, 16} and len(times) >= 2
    outs = []
    for T in sorted(times):
        plan = Plan((N, N), (1.0, 1.0), cfl=0.4, device=cuda_device, nsolve=ns, tile_cols=T)
        assert plan.tile_cols == T
        V = U.clone()
        plan.run_(V, 5, 1e-4)
        outs.append(V)
    for V in outs[1:]:
        assert torch.equal(outs[0], V)
    with pytest.raises(RuntimeError):
        Plan((N, N), (1.0, 1.0), device=cuda_device, tile_cols=32)
