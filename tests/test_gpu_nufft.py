"""NUFFT point evaluation (ps_tracer_method PS_TRACERS_NUFFT) against the
exact trigonometric interpolant: the float64 oracle (oracle/tracers.py, the
reference's no-finufft branch) and the GPU's exact path.  The reference's
finufft branch asks for eps = 1e-6 (grid.py:611, 1214, 1555); the bound here
is a relative L2 error over the points of 1e-6 (kernel error about 3e-8 per
axis at 8 points of support, float32 fields and sums on top)."""
import numpy as np
import pytest
import torch

from oracle import tracers as OT
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu

FILTER = {"enabled": True, "p": 8, "alpha": 36.0}
CASES = [  # shape (array order), lengths (array order), dealias, filter
    ((64,), (1.0,), True, True),
    ((48,), (2.0,), False, False),
    ((32, 48), (1.0, 1.5), True, False),
    ((40, 30), (2.0, 1.0), False, True),
    ((16, 24, 32), (1.0, 2.0, 3.0), True, True),
    ((16, 16, 16), (2 * np.pi,) * 3, False, False),
]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _points(rng, lengths_xyz, n):
    pts = [rng.uniform(0.0, L, n) for L in lengths_xyz]
    for a, L in enumerate(lengths_xyz):  # grid-aligned and edge positions
        pts[a][:4] = [0.0, L * (1 - 1e-12), L / 3.0, 0.5 * L]
    return pts


@pytest.mark.parametrize("shape,lengths,dealias,filt", CASES)
def test_nufft_points_match_exact_interpolant(cuda_device, shape, lengths, dealias, filt):
    rng = np.random.default_rng(11 + sum(shape))
    nd = len(shape)
    nf = min(3, nd + 1)
    f = rng.standard_normal((nf,) + tuple(shape))
    lengths_xyz = tuple(reversed(lengths))
    pts = _points(rng, lengths_xyz, 3000)
    ref = np.stack([OT.eval_points(f[c].astype(np.float32).astype(np.float64), pts, lengths_xyz, dealias,
                                   FILTER if filt else None) for c in range(nf)])
    plan = Plan(shape, lengths, dealias=dealias, filter_params=FILTER if filt else None, device=cuda_device)
    fd = torch.as_tensor(f, dtype=torch.float32, device=cuda_device).contiguous()
    pd = torch.as_tensor(np.stack(pts), dtype=torch.float64, device=cuda_device).contiguous()
    plan.tracer_method("nufft")
    nu = plan.eval_points(fd, pd).double().cpu().numpy()
    plan.tracer_method("exact")
    ex = plan.eval_points(fd, pd).double().cpu().numpy()
    e_nu, e_ex, e_pair = _rel(nu, ref), _rel(ex, ref), _rel(nu, ex)
    print(f"\n{shape} dealias={dealias} filter={filt}: nufft {e_nu:.2e}, exact {e_ex:.2e}, nufft-exact {e_pair:.2e}")
    assert e_nu < 1e-6, e_nu
    assert e_pair < 1e-6, e_pair
    plan.close()


def test_nufft_tracers_follow_exact_tracers(cuda_device):
    """Leap-frog tracers in the velocity of a Taylor-Green state: NUFFT and
    exact interpolation give the same positions to 1e-7 after five steps of
    dt = 1e-2 (velocities differ by a few 1e-7 of their size)."""
    from phrike_gb300 import problems
    n, L = 32, 2 * np.pi
    U = torch.as_tensor(problems.taylor_green_3d(n), dtype=torch.float32, device=cuda_device).contiguous()
    rng = np.random.default_rng(5)
    pos0 = torch.as_tensor(rng.uniform(0, L, (3, 4096)), dtype=torch.float64, device=cuda_device).contiguous()
    out = {}
    for method in ("nufft", "exact"):
        plan = Plan((n, n, n), (L, L, L), device=cuda_device)
        plan.tracer_method(method)
        pos, prev = pos0.clone(), pos0.clone()
        vel = torch.empty((3, 4096), dtype=torch.float32, device=cuda_device)
        for i in range(5):
            plan.tracers_step_(U, pos, prev, i == 0, 1e-2, vel)
        out[method] = (pos.cpu().numpy(), vel.double().cpu().numpy())
        plan.close()
    assert np.abs(out["nufft"][0] - out["exact"][0]).max() < 1e-7
    assert _rel(out["nufft"][1], out["exact"][1]) < 1e-6


def test_auto_method_and_unsupported_grids(cuda_device):
    """The automatic choice agrees with the exact interpolant in both regimes;
    NUFFT is refused where its oversampled axis would exceed the transform
    lengths (N > 2048) and on LGL grids."""
    rng = np.random.default_rng(3)
    shape = (64, 64)
    f = torch.as_tensor(rng.standard_normal((1,) + shape), dtype=torch.float32, device=cuda_device).contiguous()
    plan = Plan(shape, (1.0, 1.0), device=cuda_device)
    for npts in (64, 8192):  # 64 * 4096 cells: exact; 8192 * 4096 > 2^24: NUFFT
        pts = torch.as_tensor(rng.uniform(0, 1, (2, npts)), dtype=torch.float64, device=cuda_device).contiguous()
        auto = plan.eval_points(f, pts).double().cpu().numpy()
        plan.tracer_method("exact")
        ex = plan.eval_points(f, pts).double().cpu().numpy()
        plan.tracer_method("auto")
        assert _rel(auto, ex) < 1e-6
    big = Plan((4096,), (1.0,), device=cuda_device)
    with pytest.raises(RuntimeError):
        big.tracer_method("nufft")
    lgl = Plan((17, 17), (2.0, 2.0), basis="legendre", device=cuda_device)
    with pytest.raises(RuntimeError):
        lgl.tracer_method("nufft")
    with pytest.raises(ValueError):
        plan.tracer_method("fast")
