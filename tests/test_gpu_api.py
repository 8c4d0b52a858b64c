"""The reference-shaped Python API (Grid*, EulerEquations*, SpectralSolver*,
run_simulation with backend "gb300") on the GPU, against the oracle."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import spectral as O
from phrike_gb300 import problems, run_simulation
from phrike_gb300.equations import EulerEquations2D, EulerEquations3D
from phrike_gb300.grid import Grid1D, Grid2D, Grid3D
from phrike_gb300.solver import SpectralSolver2D, SpectralSolver3D

pytestmark = pytest.mark.gpu


def test_grid_operators_match_oracle(cuda_device):
    rng = np.random.default_rng(3)
    g = Grid3D(Nx=32, Ny=16, Nz=8, Lx=1.0, Ly=2.0, Lz=3.0, backend="gb300")
    box = O.FourierBox((8, 16, 32), (3.0, 2.0, 1.0), dealias=True)
    f = rng.standard_normal((2, 8, 16, 32))
    for axis, op in enumerate((g.dx1, g.dy1, g.dz1)):
        out = op(f).double().cpu().numpy()
        assert rel_l2(out, box.deriv(f, 2 - axis)) < 2e-6
    g1 = Grid1D(N=64, Lx=1.0, filter_params={"enabled": True, "p": 8, "alpha": 36.0}, backend="gb300")
    b1 = O.FourierBox((64,), (1.0,), dealias=True, filter_enabled=True)
    x = rng.standard_normal((3, 64))
    assert rel_l2(g1.dx1(x).double().cpu().numpy(), b1.deriv(x, 0)) < 2e-6
    assert rel_l2(g1.apply_spectral_filter(x).double().cpu().numpy(), b1.filt(x)) < 2e-6
    assert tuple(g.dealias_mask.shape) == (8, 16, 32)


def test_solver3d_step_is_functional_and_matches_oracle(cuda_device):
    N = 32
    g = Grid3D(Nx=N, Ny=N, Nz=N, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, backend="gb300")
    eqs = EulerEquations3D(gamma=1.4)
    solver = SpectralSolver3D(g, eqs)
    U0 = problems.taylor_green_3d(N)
    Ud = g.to_device(U0)
    U1 = solver.step(Ud, 1e-3)
    assert not torch.equal(U1, Ud)  # argument untouched, new state returned
    s = O.EulerSolver(O.FourierBox((N, N, N), (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    ref = s.step(U0.astype(np.float32).astype(np.float64), 1e-3)
    assert rel_l2(U1.double().cpu().numpy()[4], ref[4]) < 1e-6
    dt = solver.compute_dt(Ud)
    assert abs(dt - s.compute_dt(U0)) / dt < 1e-6


def test_solver2d_cfl_run_matches_oracle(cuda_device):
    N = 64
    g = Grid2D(Nx=N, Ny=N, Lx=1.0, Ly=1.0, backend="gb300")
    solver = SpectralSolver2D(g, EulerEquations2D(gamma=1.4), cfl=0.4)
    U0 = problems.kelvin_helmholtz_2d(N, N, U0=1.0, A=0.01)
    hist = solver.run(U0, 0.0, 0.01, output_interval=0.005)
    s = O.EulerSolver(O.FourierBox((N, N), (1.0, 1.0), dealias=True), cfl=0.4)
    ref, t, _ = s.run(U0.astype(np.float32).astype(np.float64), 0.0, 0.01)
    assert abs(solver.t - t) < 1e-12
    out = solver.U.double().cpu().numpy()
    for c in (0, 1, 3):
        assert rel_l2(out[c], ref[c]) < 1e-5
    assert set(hist) == {"time", "mass", "momentum_x", "momentum_y", "energy"}
    assert abs(hist["mass"][-1] - hist["mass"][0]) / hist["mass"][0] < 1e-6


def test_run_simulation_sod_fixed_dt(cuda_device):
    cfg = {"grid": {"N": 256, "Lx": 1.0, "dealias": True},
           "physics": {"gamma": 1.4},
           "integration": {"t0": 0.0, "t_end": 2e-3, "dt": 2e-5, "output_interval": 1e-3,
                           "spectral_filter": {"enabled": True, "p": 8, "alpha": 36.0}}}
    solver, hist = run_simulation("baseline_sod1d", config=cfg, backend="gb300")
    s = O.EulerSolver(O.FourierBox((256,), (1.0,), dealias=True, filter_enabled=True))
    ref = problems.sod_smoothed(256).astype(np.float32).astype(np.float64)
    for _ in range(100):
        ref = s.step(ref, 2e-5)
    out = solver.U.double().cpu().numpy()
    assert rel_l2(out[0], ref[0]) < 1e-5 and rel_l2(out[2], ref[2]) < 1e-5
    assert len(hist["time"]) >= 3


def test_run_writes_reference_snapshots(cuda_device, tmp_path):
    """run(..., checkpoint_interval, outdir) writes snapshot_t*.npz files in
    the reference's layout, readable by load_checkpoint, at the same
    times as the reference's loop (after the step that reaches each
    checkpoint time)."""
    import numpy as np
    from phrike_gb300 import EulerEquations2D, Grid2D, problems
    from phrike_gb300.io import load_checkpoint
    from phrike_gb300.solver import SpectralSolver2D
    g = Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, backend="gb300")
    s = SpectralSolver2D(g, EulerEquations2D(gamma=1.4), cfl=0.4)
    U0 = problems.kelvin_helmholtz_2d(32, 32)
    times = []
    s.run(U0, 0.0, 0.02, output_interval=0.01, checkpoint_interval=0.005, outdir=str(tmp_path),
          on_step=lambda n, dt, U: times.append(s.t))
    files = sorted(p.name for p in tmp_path.glob("snapshot_t*.npz"))
    assert len(files) >= 3
    d = load_checkpoint(str(tmp_path / files[-1]))
    assert d["U"].shape == (4, 32, 32) and set(d["primitive_vars"]) == {"rho", "ux", "uy", "p"}
    assert d["meta"]["Nx"] == 32 and abs(d["meta"]["gamma"] - 1.4) < 1e-12
    assert np.isfinite(d["U"]).all() and d["t"] in times


def test_2d_velocity_magnitude_sensor_raises_like_the_reference(cuda_device):
    """The reference's 2D velocity-magnitude AV sensor raises ValueError
    (its q is a 1D array); plans asking for it raise the same error, while
    the 1D form is accepted."""
    from phrike_gb300.engine import Plan
    av = {"enabled": True, "sensor_variable": "velocity_magnitude"}
    with pytest.raises(ValueError):
        Plan((16, 16), (1.0, 1.0), av_config=av)
    Plan((64,), (1.0,), av_config=av)


def test_step_host_stream_matches_steps(cuda_device):
    """Pinned host states through step_host_stream equal each state stepped
    on the device by step_ (same kernels, copies overlapped)."""
    from phrike_gb300.engine import Plan
    N = 32
    plan = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device)
    rng = np.random.default_rng(4)
    states = [problems.taylor_green_3d(N) * (1.0 + 0.05 * rng.random()) for _ in range(5)]
    hin = [torch.as_tensor(s, dtype=torch.float32).pin_memory() for s in states]
    hout = [torch.empty_like(h).pin_memory() for h in hin]
    plan.step_host_stream(hin, hout, 1e-3, nsteps=2)
    for h, o in zip(hin, hout):
        U = h.to(cuda_device)
        plan.run_(U, 2, 1e-3)
        assert torch.equal(U.cpu(), o)


@pytest.mark.parametrize("shape", [(64,), (32, 64), (16, 8, 32)])
@pytest.mark.parametrize("filt", [False, True])
def test_laplacian_and_curl_match_oracle(cuda_device, shape, filt):
    """Grid*.laplacian (masked, Nyquist kept) and Grid3D.curl against the
    float64 oracle on random fields."""
    fp = {"enabled": True, "p": 8, "alpha": 36.0} if filt else None
    lengths = tuple(1.0 + 0.5 * i for i in range(len(shape)))
    xyz = list(reversed(shape))
    lxyz = list(reversed(lengths))
    if len(shape) == 1:
        g = Grid1D(N=shape[0], Lx=lengths[0], filter_params=fp)
    elif len(shape) == 2:
        g = Grid2D(Nx=xyz[0], Ny=xyz[1], Lx=lxyz[0], Ly=lxyz[1], filter_params=fp)
    else:
        g = Grid3D(Nx=xyz[0], Ny=xyz[1], Nz=xyz[2], Lx=lxyz[0], Ly=lxyz[1], Lz=lxyz[2], filter_params=fp)
    box = O.FourierBox(shape, lengths, dealias=True, filter_enabled=filt)
    rng = np.random.default_rng(len(shape))
    f = rng.standard_normal(shape)
    lap = g.laplacian(f.astype(np.float32)).double().cpu().numpy()
    assert rel_l2(lap, box.laplacian(f)) < 2e-6
    if len(shape) == 3:
        V = [rng.standard_normal(shape) for _ in range(3)]
        C = g.curl(*[v.astype(np.float32) for v in V])
        want = (box.deriv(V[2], 1) - box.deriv(V[1], 0), box.deriv(V[0], 0) - box.deriv(V[2], 2),
                box.deriv(V[1], 2) - box.deriv(V[0], 1))
        for got, w in zip(C, want):
            assert rel_l2(got.double().cpu().numpy(), w) < 2e-6
