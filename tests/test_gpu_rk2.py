"""scheme="rk2" (the midpoint method of every reference solver) on the GPU
against the reference's own runs (tests/golden/rk2.npz): 1D Sod with filter
cadence 2, 2D KHI, 3D TGV and 2D MHD Orszag-Tang, plus the LGL path against
the oracle."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FP = {"enabled": True, "p": 8, "alpha": 36.0}


def _errs(G, R):
    G = np.asarray(G, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    nc = G.shape[0]
    groups = ((slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8)) if nc == 8 else
              (slice(0, 1), slice(1, nc - 1), slice(nc - 1, nc)))
    floor = 1e-2 * np.linalg.norm(R)
    return [float(np.linalg.norm(G[g] - R[g]) / max(np.linalg.norm(R[g]), floor)) for g in groups]


def _run(plan, U0, nsteps, dt):
    import torch
    U = torch.as_tensor(np.ascontiguousarray(U0), dtype=torch.float32, device=plan.device).contiguous()
    for _ in range(nsteps):
        plan.step_(U, dt)
    return U.cpu().numpy()


def test_rk2_fourier_and_mhd_match_reference(cuda_device):
    from phrike_gb300.engine import Plan
    z = golden("rk2.npz")
    p1 = Plan((128,), (1.0,), filter_params=dict(FP, interval=2), scheme="rk2")
    assert max(_errs(_run(p1, z["sod_U0"], 5, 2e-4), z["sod_U"])) < 1e-5
    p2 = Plan((32, 32), (1.0, 1.0), filter_params=FP, scheme="rk2")
    assert max(_errs(_run(p2, z["khi_U0"], 4, 1e-3), z["khi_U"])) < 1e-5
    p3 = Plan((16, 16, 16), (2 * np.pi,) * 3, scheme="rk2")
    assert max(_errs(_run(p3, z["tgv_U0"], 3, 1e-3), z["tgv_U"])) < 1e-5
    pm = Plan((32, 32), (2 * np.pi,) * 2, gamma=5.0 / 3.0, filter_params=FP, equations="mhd", scheme="rk2")
    assert max(_errs(_run(pm, z["ot_U0"], 3, 2e-3), z["ot_U"])) < 1e-5


@pytest.mark.parametrize("case", ["khi", "tgv", "ot"])
def test_rk2_is_the_midpoint_method(case, cuda_device):
    """Longer steps, where RK2 and RK4 separate by far more than float32
    rounding: the GPU result sits on the oracle's RK2 trajectory."""
    from oracle import mhd as M
    from oracle import spectral as O
    from phrike_gb300 import problems
    from phrike_gb300.engine import Plan
    fbox = dict(dealias=True, filter_enabled=True)
    if case == "khi":
        U0, n, dt = problems.kelvin_helmholtz_2d(32, 32, U0=1.2, A=0.015), 20, 4e-3
        mk = lambda s: O.EulerSolver(O.FourierBox((32, 32), (1.0, 1.0), **fbox), scheme=s)  # noqa: E731
        plan = Plan((32, 32), (1.0, 1.0), filter_params=FP, scheme="rk2")
    elif case == "tgv":
        U0, n, dt = problems.taylor_green_3d(16), 10, 1e-2
        mk = lambda s: O.EulerSolver(O.FourierBox((16,) * 3, (2 * np.pi,) * 3, dealias=True), scheme=s)  # noqa: E731
        plan = Plan((16, 16, 16), (2 * np.pi,) * 3, scheme="rk2")
    else:
        U0, n, dt = problems.orszag_tang_2d(32, 32, gamma=5.0 / 3.0), 10, 1e-2
        mk = lambda s: M.MHDSolver2D(32, 32, filter_params=FP, scheme=s)  # noqa: E731
        plan = Plan((32, 32), (2 * np.pi,) * 2, gamma=5.0 / 3.0, filter_params=FP, equations="mhd", scheme="rk2")
    U0 = U0.astype(np.float32).astype(np.float64)
    if case == "ot":
        U0 = mk("rk2").project(U0)
    ref = {}
    for sch in ("rk2", "rk4"):
        so = mk(sch)
        U = U0.copy()
        for _ in range(n):
            U = so.step(U, dt)
        ref[sch] = U
    sep = max(_errs(ref["rk4"], ref["rk2"]))
    got = _run(plan, U0, n, dt)
    assert max(_errs(got, ref["rk2"])) < 0.2 * sep, (max(_errs(got, ref["rk2"])), sep)


def test_rk2_lgl_vs_oracle(cuda_device):
    from oracle import lgl as L
    from phrike_gb300 import problems
    from phrike_gb300.engine import Plan
    n = 33
    ax = L.LGLAxis(n, 2.0)
    U0 = problems.acoustic_pulse_lgl_2d(ax.x - 1.0, ax.x - 1.0, amp=0.2, width2=0.05)
    s = L.LGLSolver2D(n, n, scheme="rk2")
    R = U0.astype(np.float32).astype(np.float64)
    for _ in range(10):
        R = s.step(R, 1e-4)
    for prec in ("fp32", "bf16x3"):
        p = Plan((n, n), (2.0, 2.0), basis="legendre", gemm_precision=prec, scheme="rk2")
        assert max(_errs(_run(p, U0, 10, 1e-4), R)) < 2e-4, prec
