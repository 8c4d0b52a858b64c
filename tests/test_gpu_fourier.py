"""GPU parity of the Fourier Euler path (C ABI through phrike_gb300.engine)
against the reference's golden vectors and the float64 oracle.

Tolerances: the CUDA path computes in float32 (fluxes, FFTs, RK stages),
the references in float64.
* one-axis operators on unit-variance random fields: relative L2 <= 2e-6;
* right-hand sides: relative L2 per field <= 3e-4.  This is the float32 floor
  of the algorithm itself: the reference's own formulas evaluated with
  float32 FFTs give 0.5-1.1e-4 on the same inputs (low-Mach cancellation in
  the flux divergence); fields that are identically zero in the reference
  are measured against the largest field of the same state;
* states: relative L2 per conserved field; momentum components are measured
  against the norm of the momentum vector field.  Full-length workload runs
  (Sod 1000 steps, Taylor-Green 200 steps, Kelvin-Helmholtz) must stay within
  1e-5, the acceptance bar.  Short golden runs (2-8 steps from rest) stay
  within 5e-5: their momentum is still ~1e-3 of its late-time size, so the
  float32 floor of the other fields dominates its relative error.
"""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2
from oracle import spectral as O
from phrike_gb300 import problems
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu

TAGS = ["d1f0", "d1f1", "d0f0", "d0f1"]


def dev(x, device):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device=device)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def field_errors(out, ref, momentum_vector=True):
    """Relative L2 error per conserved field.  Momentum components (1..nc-2)
    are scaled by the momentum vector norm; fields that vanish in the
    reference are scaled by the largest field norm of the same state."""
    nc = len(ref)
    norms = [np.linalg.norm(r) for r in ref]
    if momentum_vector and nc >= 3:
        mv = float(np.sqrt(sum(norms[c] ** 2 for c in range(1, nc - 1))))
        for c in range(1, nc - 1):
            norms[c] = mv
    big = max(norms)
    return [np.linalg.norm(o - r) / (n if n > 1e-6 * big else big) for o, r, n in zip(out, ref, norms)]


RHS_TOL = 3e-4
STATE_TOL = 1e-5
SHORT_TOL = 5e-5


@pytest.mark.parametrize("tag", TAGS)
def test_operators_vs_reference(cuda_device, tag):
    ops = golden("fourier_ops.npz")
    d, f = bool(int(tag[1])), bool(int(tag[3]))
    fp = {"enabled": f, "p": 8, "alpha": 36.0}
    cases = [
        ((64,), (1.0,), "g1", ["dx"]),
        ((16, 32), (0.5, 1.0), "g2", ["dx", "dy"]),
        ((16, 8, 16), (4 * np.pi, np.pi, 2 * np.pi), "g3", ["dx", "dy", "dz"]),
    ]
    for shape, lengths, g, names in cases:
        plan = Plan(shape, lengths, dealias=d, filter_params=fp, device=cuda_device)
        x = ops[f"{g}_{tag}_in"]
        xd = dev(x, cuda_device)
        for axis, nm in enumerate(names):
            out = host(plan.derivative(xd, axis))
            ref = ops[f"{g}_{tag}_{nm}"]
            # noise floor: float32 rounding of a unit-variance field
            assert rel_l2(out, ref) < 2e-6, (g, nm, rel_l2(out, ref))
        out = host(plan.filter(xd))
        assert rel_l2(out, ops[f"{g}_{tag}_filt"]) < 2e-6
        plan.close()


@pytest.mark.parametrize("N", [128, 1024])
def test_sod_rhs_and_steps_vs_reference(cuda_device, N):
    z = golden(f"sod1d_n{N}.npz")
    plan = Plan((N,), (1.0,), filter_params={"enabled": True, "p": 8, "alpha": 36.0}, device=cuda_device)
    U = dev(z["U0"], cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, z["rhs0"])) < RHS_TOL, field_errors(r, z["rhs0"])
    for _ in range(int(z["nsteps"])):
        plan.step_(U, float(z["dt"]))
    out = host(U)
    assert max(field_errors(out, z["U"])) < SHORT_TOL, field_errors(out, z["U"])


def test_sod_config_1000_steps_vs_oracle(cuda_device):
    """The 1D Sod workload at full size: N=1024, dt=2e-5, 1000 steps, one launch."""
    N = 1024
    U0 = problems.sod_smoothed(N)
    s = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True))
    ref = U0
    for _ in range(1000):
        ref = s.step(ref, 2e-5)
    plan = Plan((N,), (1.0,), filter_params={"enabled": True, "p": 8, "alpha": 36.0}, device=cuda_device)
    U = dev(U0, cuda_device)
    plan.run_(U, 1000, 2e-5)
    out = host(U)
    assert max(field_errors(out, ref)) < STATE_TOL, field_errors(out, ref)


@pytest.mark.parametrize("shape,nsteps", [((16, 16, 16), 3), ((32, 8, 16), 2)])
def test_tgv_rhs_and_steps_vs_reference(cuda_device, shape, nsteps):
    Nz, Ny, Nx = shape
    z = golden(f"tgv3d_{Nx}x{Ny}x{Nz}.npz")
    plan = Plan(shape, (2 * np.pi,) * 3, device=cuda_device)
    U = dev(z["U0"], cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, z["rhs0"])) < RHS_TOL, field_errors(r, z["rhs0"])
    for _ in range(nsteps):
        plan.step_(U, 1e-3)
    out = host(U)
    assert max(field_errors(out, z["U"])) < SHORT_TOL, field_errors(out, z["U"])
    speed = float(host(plan.max_wave_speed(dev(z["U0"], cuda_device)))[0])
    assert abs(speed - float(z["speed0"])) / float(z["speed0"]) < 1e-6


def test_tgv_64_multistep_vs_oracle(cuda_device):
    N = 64
    U0 = problems.taylor_green_3d(N)
    U0f = U0.astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox((N, N, N), (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    ref = U0f
    for _ in range(8):
        ref = s.step(ref, 1e-3)
    plan = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device)
    U = dev(U0, cuda_device)
    plan.run_(U, 8, 1e-3)
    out = host(U)
    assert max(field_errors(out, ref)) < SHORT_TOL, field_errors(out, ref)
    cons = host(plan.conserved(U))
    oc = O.conserved_sums(ref, 1.4)
    np.testing.assert_allclose(cons[0], oc["mass"], rtol=1e-6)
    np.testing.assert_allclose(cons[4], oc["energy"], rtol=1e-6)


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 16)])
def test_khi_rhs_and_cfl_steps_vs_reference(cuda_device, nx, ny):
    z = golden(f"khi2d_{nx}x{ny}.npz")
    plan = Plan((ny, nx), (1.0, 1.0), cfl=0.4, device=cuda_device)
    U = dev(z["U0"], cuda_device)
    r = host(plan.rhs(U))
    assert max(field_errors(r, z["rhs0"])) < RHS_TOL, field_errors(r, z["rhs0"])
    for dt in z["dts"]:
        plan.step_(U, float(dt))
    out = host(U)
    assert max(field_errors(out, z["U"])) < SHORT_TOL, field_errors(out, z["U"])


def test_khi_256_vs_oracle(cuda_device):
    N = 256
    U0 = problems.kelvin_helmholtz_2d(N, N, U0=1.0, A=0.01)
    U0f = U0.astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox((N, N), (1.0, 1.0), dealias=True), cfl=0.4)
    ref = U0f
    dt = s.compute_dt(ref)
    for _ in range(5):
        ref = s.step(ref, dt)
    plan = Plan((N, N), (1.0, 1.0), device=cuda_device)
    U = dev(U0, cuda_device)
    plan.run_(U, 5, dt)
    out = host(U)
    assert max(field_errors(out, ref)) < STATE_TOL, field_errors(out, ref)


def test_tgv_256_full_size_properties(cuda_device):
    """Full benchmark size: finite, mass conserved to float32 rounding, and the
    state the same whether stepped one call at a time or in one run: each call
    rebases the energy reference E_ref (E -> E - E_ref -> E), which moves E by
    an ulp (~1.5e-5 at E ~ 180) and the other fields through the energy flux,
    so the two agree to a few 1e-6 rather than bit for bit."""
    N = 256
    U0 = dev(problems.taylor_green_3d(N), cuda_device)
    plan = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device)
    m0 = host(plan.conserved(U0))
    U = U0.clone()
    plan.run_(U, 4, 1e-3)
    V = U0.clone()
    for _ in range(4):
        plan.step_(V, 1e-3)
    assert torch.isfinite(U).all()
    assert plan.status() == 0
    m1 = host(plan.conserved(U))
    assert abs(m1[0] - m0[0]) / m0[0] < 1e-6
    assert abs(m1[4] - m0[4]) / m0[4] < 1e-6
    torch.testing.assert_close(U, V, rtol=1e-6, atol=1e-5)


def test_tgv_200_steps_vs_oracle(cuda_device):
    """The Taylor-Green workload's full step count (200 steps, dt=1e-3) at 32^3:
    every conserved field within 1e-5 relative L2 of the float64 oracle."""
    N = 32
    U0 = problems.taylor_green_3d(N)
    s = O.EulerSolver(O.FourierBox((N, N, N), (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    ref = U0.astype(np.float32).astype(np.float64)
    for _ in range(200):
        ref = s.step(ref, 1e-3)
    plan = Plan((N, N, N), (2 * np.pi,) * 3, device=cuda_device)
    U = dev(U0, cuda_device)
    plan.run_(U, 200, 1e-3)
    out = host(U)
    assert plan.status() == 0
    assert max(field_errors(out, ref)) < STATE_TOL, field_errors(out, ref)
