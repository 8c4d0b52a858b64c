"""Fourier axes of any 2^a 3^b 5^c length (the mixed-radix passes) against
the float64 oracle, whose NumPy transforms take any N as the reference's
grids do (phrike/grid.py:47-63, 87-115: k = fftfreq(N) * N).

* one-axis operators (derivative, filter, Laplacian) on 1D, 2D and 3D grids
  with N = 48, 96, 384, odd lengths (15, 45, 75) and mixed power-of-two and
  other axes: relative L2 <= 2e-6 on unit-variance random fields;
* right-hand sides: relative L2 per field <= 3e-4 (the float32 floor of the
  flux divergence, as for the power-of-two passes);
* steps: Kelvin-Helmholtz (2D, with the filter and gravity) within 1e-5 per
  conserved field, Taylor-Green (3D) within 5e-5 for runs of a few steps
  from rest, Sod (1D) on coarse grids within 1e-4 after 1000 steps (the
  power-of-two kernel's own float32 floor on that case is 2.2e-5) and within
  1e-5 on a CFL run;
* the reference's khi2d problem on its shipped 3840 x 2160 grid
  (configs/khi2d_4k.yaml) for three CFL steps against an oracle fixture,
  and through run_simulation with that config.
"""
import numpy as np
import pytest
import torch

import parity_cases as PC
from conftest import golden, rel_l2
from oracle import spectral as O
from phrike_gb300 import problems
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu

OP_TOL = 2e-6
RHS_TOL = 3e-4
STATE_TOL = 1e-5
SHORT_TOL = 5e-5
SOD_TOL = 1e-4
FILTER = {"enabled": True, "p": 8, "alpha": 36.0}


def dev(x, device):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device=device)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def field_errors(out, ref):
    nc = len(ref)
    norms = [np.linalg.norm(r) for r in ref]
    if nc >= 3:
        mv = float(np.sqrt(sum(norms[c] ** 2 for c in range(1, nc - 1))))
        for c in range(1, nc - 1):
            norms[c] = mv
    big = max(norms)
    return [np.linalg.norm(o - r) / (n if n > 1e-6 * big else big) for o, r, n in zip(out, ref, norms)]


OP_CASES = [
    ((48,), (1.0,)),
    ((96,), (2.0,)),
    ((384,), (1.0,)),
    ((45,), (1.0,)),
    ((6,), (1.0,)),
    ((96, 48), (1.0, 0.5)),
    ((384, 96), (2.0, 1.0)),
    ((64, 48), (1.0, 1.0)),
    ((75, 15), (1.0, 3.0)),
    ((2160, 40), (1.0, 0.2)),
    ((24, 36, 48), (2 * np.pi, np.pi, 2 * np.pi)),
    ((16, 30, 32), (1.0, 1.0, 1.0)),
]


@pytest.mark.parametrize("shape,lengths", OP_CASES)
@pytest.mark.parametrize("dealias,filt", [(True, True), (False, False), (True, False)])
def test_operators_vs_oracle(cuda_device, shape, lengths, dealias, filt):
    rng = np.random.default_rng(7 + sum(shape))
    nf = 3
    x = rng.standard_normal((nf,) + tuple(shape))
    box = O.FourierBox(tuple(shape), tuple(lengths), dealias=dealias, filter_enabled=filt)
    plan = Plan(shape, lengths, dealias=dealias, filter_params=FILTER if filt else None, device=cuda_device)
    xd = dev(x, cuda_device)
    nd = len(shape)
    for axis in range(nd):  # axis 0 = x = last array axis
        out = host(plan.derivative(xd, axis))
        ref = box.deriv(x, nd - 1 - axis)
        assert rel_l2(out, ref) < OP_TOL, (shape, axis, rel_l2(out, ref))
    out = host(plan.filter(xd))
    assert rel_l2(out, box.filt(x)) < OP_TOL, (shape, "filter", rel_l2(out, box.filt(x)))
    out = host(plan.laplacian(xd))
    assert rel_l2(out, box.laplacian(x)) < OP_TOL, (shape, "laplacian")
    # in place
    y = xd.clone()
    plan.derivative(y, 0, out=y)
    assert rel_l2(host(y), box.deriv(x, nd - 1)) < OP_TOL
    plan.close()


@pytest.mark.parametrize("N", [48, 96, 384, 128])
def test_sod_rhs_and_steps_vs_oracle(cuda_device, N):
    """1000 steps of dt = 2e-5 as the Sod workload, on coarse grids (the
    tanh edges 2-8 cells wide).  The float32 floor of this case is set by the
    edges' under-resolved modes: N = 128 on the power-of-two whole-step kernel
    measures 2.2e-5 (momentum), N = 48 / 96 / 384 on the mixed-radix passes
    1.5e-5 / 5.4e-5 / 2.3e-5, and a plain float32 restatement of the
    reference's step 1e-4; the bound is 1e-4.  (At the workload's N = 1024
    and width 0.005 the power-of-two kernel is within 1e-5.)"""
    U0 = problems.sod_smoothed(N, width=0.02)
    U0f = U0.astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True))
    plan = Plan((N,), (1.0,), filter_params=FILTER, device=cuda_device)
    U = dev(U0, cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, s.rhs(U0f))) < RHS_TOL
    ref = U0f
    for _ in range(1000):
        ref = s.step(ref, 2e-5)
    plan.run_(U, 1000, 2e-5)
    assert plan.status() == 0
    e = field_errors(host(U), ref)
    print(f"\nSod N={N} 1000 steps rel-L2 {e}")
    assert max(e) < SOD_TOL, e


def test_sod_cfl_run_vs_oracle(cuda_device):
    N = 96
    U0 = problems.sod_smoothed(N, width=0.02)
    U0f = U0.astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True), cfl=0.4)
    ref, tr, dts = s.run(U0f, 0.0, 0.02)
    plan = Plan((N,), (1.0,), filter_params=FILTER, cfl=0.4, device=cuda_device)
    U = dev(U0, cuda_device)
    f64 = dict(dtype=torch.float64, device=cuda_device)
    t, te = torch.zeros(1, **f64), torch.full((1,), 0.02, **f64)
    plan.run_cfl_(U, len(dts) + 5, t, te)
    assert abs(t.item() - tr) < 1e-12
    assert plan.steps_done()[0] == len(dts)
    e = field_errors(host(U), ref)
    assert max(e) < STATE_TOL, e


@pytest.mark.parametrize("ny,nx,grav", [(60, 48, None), (96, 80, (0.3, -1.0)), (48, 64, None)])
def test_khi_rhs_and_steps_vs_oracle(cuda_device, ny, nx, grav):
    U0 = problems.kelvin_helmholtz_2d(nx, ny, U0=1.0, A=0.01)
    U0f = U0.astype(np.float32).astype(np.float64)
    box = O.FourierBox((ny, nx), (1.0, 1.0), dealias=True, filter_enabled=True)
    s = O.EulerSolver(box, cfl=0.4, gravity=list(grav) if grav else None)
    plan = Plan((ny, nx), (1.0, 1.0), filter_params=FILTER, cfl=0.4,
                gravity=list(grav) if grav else None, device=cuda_device)
    U = dev(U0, cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, s.rhs(U0f))) < RHS_TOL
    ref = U0f
    dt = s.compute_dt(ref)
    for _ in range(20):
        ref = s.step(ref, dt)
    plan.run_(U, 20, dt)
    assert plan.status() == 0
    e = field_errors(host(U), ref)
    print(f"\nKHI {ny}x{nx} grav={grav} 20 steps rel-L2 {e}")
    assert max(e) < STATE_TOL, e
    speed = float(host(plan.max_wave_speed(dev(U0, cuda_device)))[0])
    assert abs(speed - O.max_wave_speed(U0f, 1.4)) / speed < 1e-6


@pytest.mark.parametrize("shape", [(24, 20, 18), (16, 16, 48), (12, 32, 16)])
def test_tgv_rhs_and_steps_vs_oracle(cuda_device, shape):
    Nz, Ny, Nx = shape
    U0 = problems.taylor_green_3d(Nx, Ny, Nz)
    U0f = U0.astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox(shape, (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    plan = Plan(shape, (2 * np.pi,) * 3, device=cuda_device)
    U = dev(U0, cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, s.rhs(U0f))) < RHS_TOL
    ref = U0f
    for _ in range(6):
        ref = s.step(ref, 1e-3)
    plan.run_(U, 6, 1e-3)
    e = field_errors(host(U), ref)
    print(f"\nTGV {shape} 6 steps rel-L2 {e}")
    assert max(e) < SHORT_TOL, e


def test_khi2d_4k_shipped_grid_vs_oracle(cuda_device):
    """configs/khi2d_4k.yaml: 3840 x 2160 (axes 2^8 3 5 and 2^4 3^3 5), the
    reference's khi2d initial state, filter p = 8, alpha = 36, three RK4 steps
    at the CFL step size; float64 oracle fixture on every 16th point."""
    z = golden("khi2d_4k_steps.npz")
    cfg = PC.khi4k_config()
    g = cfg["grid"]
    nx, ny = int(g["Nx"]), int(g["Ny"])
    plan = Plan((ny, nx), (float(g["Ly"]), float(g["Lx"])), filter_params=FILTER, cfl=0.25, device=cuda_device)
    U = dev(PC.khi4k_initial_state(cfg), cuda_device)
    for dt in z["dts"]:
        plan.step_(U, float(dt))
    assert plan.status() == 0
    out = PC.sub(host(U), int(z["stride"]))
    e = PC.field_errors(out, z["U"])
    print(f"\nkhi2d_4k 3 steps rel-L2 vector {e['vector']} component {e['component']}")
    assert max(e["vector"]) < STATE_TOL, e
    plan.close()


def test_khi2d_4k_config_through_run_simulation(cuda_device):
    """run_simulation("khi2d") with the khi2d_4k config keys, the end time cut
    to the fixture's three CFL steps.  The reference reads adaptive settings
    from integration.adaptive only (problems/base.py:111-125), so the config's
    top-level adaptive block leaves fixed RK4 steps (scheme rk78 falls back to
    RK4) at the CFL step size, as in the fixture."""
    from phrike_gb300 import run_simulation
    z = golden("khi2d_4k_steps.npz")
    cfg = PC.khi4k_config()
    t_end = float(np.sum(z["dts"]))
    cfg["integration"].update(t_end=t_end, output_interval=t_end, checkpoint_interval=0.0)
    cfg["adaptive"] = {"enabled": True, "scheme": "rk78", "rtol": 1e-6, "atol": 1e-8, "safety_factor": 0.5,
                       "min_dt_factor": 0.1, "max_dt_factor": 2.0, "max_rejections": 10, "fallback_scheme": "rk4"}
    solver, _ = run_simulation("khi2d", config=cfg, backend="gb300")
    assert abs(solver.t - t_end) < 1e-12
    out = PC.sub(solver.U.double().cpu().numpy(), int(z["stride"]))
    e = PC.field_errors(out, z["U"])
    print(f"\nkhi2d_4k through run_simulation rel-L2 vector {e['vector']}")
    assert max(e["vector"]) < STATE_TOL, e


def test_batched_mixed_radix_solves_equal_alone(cuda_device):
    """Three KHI solves in one batched plan give bitwise the states of the
    same solves run alone."""
    ny, nx = 60, 48
    amps = [0.01, 0.015, 0.02]
    alone = []
    for a in amps:
        p1 = Plan((ny, nx), (1.0, 1.0), filter_params=FILTER, device=cuda_device)
        U = dev(problems.kelvin_helmholtz_2d(nx, ny, U0=1.0, A=a), cuda_device)
        p1.run_(U, 10, 1e-3)
        alone.append(U)
    pb = Plan((ny, nx), (1.0, 1.0), filter_params=FILTER, nsolve=3, device=cuda_device)
    UB = dev(np.stack([problems.kelvin_helmholtz_2d(nx, ny, U0=1.0, A=a) for a in amps]), cuda_device)
    pb.run_(UB, 10, 1e-3)
    for i in range(3):
        assert torch.equal(UB[i], alone[i])


def test_power_of_two_and_mixed_radix_agree(cuda_device):
    """A 64 x 48 grid (x on the mixed-radix passes) steps like the oracle, and
    a 64 x 64 grid run on the power-of-two passes agrees with the oracle too:
    the two pass families implement one operator."""
    for nx in (48, 64):
        U0 = problems.kelvin_helmholtz_2d(nx, 64, U0=1.0, A=0.01)
        U0f = U0.astype(np.float32).astype(np.float64)
        s = O.EulerSolver(O.FourierBox((64, nx), (1.0, 1.0), dealias=True), cfl=0.4)
        ref = U0f
        for _ in range(5):
            ref = s.step(ref, 1e-3)
        plan = Plan((64, nx), (1.0, 1.0), device=cuda_device)
        U = dev(U0, cuda_device)
        plan.run_(U, 5, 1e-3)
        assert max(field_errors(host(U), ref)) < STATE_TOL
