"""Point evaluation and tracer advection on the GPU (ps_eval_points,
ps_tracers_step) against the reference's vectors and the float64 oracle.

Tolerances.  The fields are float32 on the device; the kernel sums
sum_j f_j K_x K_y K_z with float32 weights and float64 accumulation across
units, so values agree with the float64 interpolant of the same float32
field to a few 1e-7 of the field's largest value (bounds below 2e-6), and
with the reference's float64 field to its float32 rounding on top.
Positions move by dt * v per step, so they agree to far below 1e-6."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

NAMES = ["d1", "d1_nyq", "d2", "d2_nyq", "d3", "d3_nyq"]


def _grid(name):
    import tracer_cases as TC
    from phrike_gb300.grid import Grid1D, Grid2D, Grid3D
    shape, lengths, dealias, filt, _ = TC.CASES[name]
    fp = dict(filt) if filt else None
    if len(shape) == 1:
        return Grid1D(N=shape[0], Lx=lengths[0], dealias=dealias, filter_params=fp)
    if len(shape) == 2:
        return Grid2D(Nx=shape[1], Ny=shape[0], Lx=lengths[1], Ly=lengths[0], dealias=dealias, filter_params=fp)
    return Grid3D(Nx=shape[2], Ny=shape[1], Nz=shape[0], Lx=lengths[2], Ly=lengths[1], Lz=lengths[0],
                  dealias=dealias, filter_params=fp)


def _tracers(pos):
    from phrike_gb300 import tracers as T
    return (T.FourierTracers1D, T.FourierTracers2D, T.FourierTracers3D)[len(pos) - 1](*pos)


@pytest.mark.parametrize("name", NAMES)
def test_point_evaluation_matches_reference(cuda_device, name):
    import tracer_cases as TC
    from oracle import tracers as OT
    z = golden("tracers.npz")
    shape, lengths, dealias, filt, _ = TC.CASES[name]
    g = _grid(name)
    pos = TC.tracer_positions(name)
    f32 = TC.field(name).astype(np.float32)
    if len(shape) == 1:
        got = g.evaluate_fourier_at_points_1d(f32, pos[0])
    else:
        got = g.evaluate_fourier_at_points(f32, *pos)
    got = got.cpu().numpy().astype(np.float64)
    want = OT.eval_points(f32.astype(np.float64), pos, list(reversed(lengths)), dealias, filt)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() < 2e-6 * scale, np.abs(got - want).max() / scale
    assert np.abs(got - z[f"{name}_f"]).max() < 5e-6 * scale


@pytest.mark.parametrize("name", NAMES)
def test_tracers_match_reference(cuda_device, name):
    import torch
    import tracer_cases as TC
    z = golden("tracers.npz")
    shape, lengths, dealias, filt, num = TC.CASES[name]
    g = _grid(name)
    U = torch.as_tensor(TC.state(name), dtype=torch.float32, device="cuda")
    tr = _tracers(TC.tracer_positions(name))
    vel = torch.empty((len(shape), num), dtype=torch.float32, device="cuda")
    tr.step(g, None, U, TC.DT, velocity_out=vel)
    v = vel.cpu().numpy()
    assert np.abs(v - z[f"{name}_vel"]).max() < 5e-6 * np.abs(z[f"{name}_vel"]).max()
    for _ in range(TC.STEPS - 1):
        tr.step(g, None, U, TC.DT)
    pos = np.stack([tr.x.cpu().numpy()] + ([tr.y.cpu().numpy()] if len(shape) > 1 else [])
                   + ([tr.z.cpu().numpy()] if len(shape) > 2 else []))
    assert np.abs(pos - z[f"{name}_pos"]).max() < 1e-7
    for a, L in enumerate(reversed(lengths)):
        assert (pos[a] >= 0).all() and (pos[a] < L).all()


def test_batched_3d_matches_single(cuda_device):
    import tracer_cases as TC
    g = _grid("d3")
    pos = TC.tracer_positions("d3")
    rng = np.random.default_rng(3)
    fs = [rng.standard_normal(TC.CASES["d3"][0]).astype(np.float32) for _ in range(3)]
    vb = g.evaluate_fourier_at_points_batched_3d(*fs, *pos)
    for f, v in zip(fs, vb):
        s = g.evaluate_fourier_at_points(f, *pos)
        np.testing.assert_allclose(v.cpu().numpy(), s.cpu().numpy(), rtol=0, atol=1e-6 * float(np.abs(f).max()))


@pytest.mark.parametrize("shape,lengths,dealias,num", [((64, 64, 64), (1.0, 2.0, 3.0), True, 200),
                                                       ((4096,), (1.0,), False, 16),
                                                       ((256, 512), (1.0, 1.0), True, 64)])
def test_point_evaluation_larger_grids(cuda_device, shape, lengths, dealias, num):
    """Config-size grids (several tracers per CTA, and the one-tracer path
    whose tables need more shared memory at 4096 points) against the oracle."""
    from oracle import tracers as OT
    from phrike_gb300.grid import Grid1D, Grid2D, Grid3D
    rng = np.random.default_rng(5)
    f = rng.standard_normal(shape).astype(np.float32)
    pos = [rng.uniform(0, L, num) for L in reversed(lengths)]
    if len(shape) == 1:
        g = Grid1D(N=shape[0], Lx=lengths[0], dealias=dealias)
        got = g.evaluate_fourier_at_points_1d(f, pos[0])
    elif len(shape) == 2:
        g = Grid2D(Nx=shape[1], Ny=shape[0], Lx=lengths[1], Ly=lengths[0], dealias=dealias)
        got = g.evaluate_fourier_at_points(f, *pos)
    else:
        g = Grid3D(Nx=shape[2], Ny=shape[1], Nz=shape[0], Lx=lengths[2], Ly=lengths[1], Lz=lengths[0],
                   dealias=dealias)
        got = g.evaluate_fourier_at_points(f, *pos)
    want = OT.eval_points(f.astype(np.float64), pos, list(reversed(lengths)), dealias, None)
    scale = np.abs(want).max()
    assert np.abs(got.cpu().numpy() - want).max() < 3e-6 * scale, np.abs(got.cpu().numpy() - want).max() / scale


def test_solver_run_with_tracers_matches_reference(cuda_device, tmp_path):
    """KHI 32^2, CFL 0.4 to t = 0.02 with 30 tracers through
    SpectralSolver2D.run(..., tracers=): tracers move after every step with
    its dt (solver.py:398-399); a checkpoint carries their positions."""
    from phrike_gb300 import problems
    from phrike_gb300.equations import EulerEquations2D
    from phrike_gb300.grid import Grid2D
    from phrike_gb300.io import load_checkpoint
    from phrike_gb300.solver import SpectralSolver2D
    z = golden("tracers.npz")
    g = Grid2D(Nx=32, Ny=32, Lx=1.0, Ly=1.0, dealias=True)
    s = SpectralSolver2D(g, EulerEquations2D(gamma=1.4), scheme="rk4", cfl=0.4)
    tr = _tracers([z["khi_x0"], z["khi_y0"]])
    s.run(problems.kelvin_helmholtz_2d(32, 32, U0=1.0, A=0.01), 0.0, 0.02, output_interval=1.0,
          checkpoint_interval=0.01, outdir=str(tmp_path), tracers=tr)
    pos = np.stack([tr.x.cpu().numpy(), tr.y.cpu().numpy()])
    assert np.abs(pos - z["khi_pos"]).max() < 1e-6
    snaps = sorted(tmp_path.glob("snapshot_*.npz"))
    assert snaps
    ck = load_checkpoint(str(snaps[-1]))
    assert ck["tracer_x"].shape == (30,) and ck["tracer_mass"] == 1.0


def test_tracers_reject_legendre_grids(cuda_device):
    from phrike_gb300.grid import Grid1D
    from phrike_gb300.tracers import FourierTracers1D
    g = Grid1D(N=17, Lx=2.0, basis="legendre")
    with pytest.raises(ValueError):
        FourierTracers1D(np.array([0.5])).step(g, None, np.ones((3, 17), np.float32), 1e-3)
