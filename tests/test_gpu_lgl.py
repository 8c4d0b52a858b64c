"""LGL x LGL (2D Legendre-Gauss-Lobatto) path on the GPU against the oracle
and the reference's golden vectors: device construction of nodes, weights
and differentiation matrices (float64), walls, derivatives, filter, the
right-hand side and RK4 steps in every contraction precision, CFL runs and
batches.

Tolerances.  The state is float32, so even float64 contractions see the
float32 rounding of the input state (notably of E ~ 1.8 for the acoustic
pulse), amplified at the walls by the O(N^2) norm of D: that floor is about
3e-6 relative on the momentum right-hand side of the 17- and 33-point
fixtures.  Split bf16 x3 keeps about 16 significand bits of each operand, so
its momentum right-hand side sits near 2e-5.  The tensor-core and CUDA-core
forms of the split arithmetic differ only in float32 accumulation order
(about 2e-6 relative at 513 points).
"""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import lgl as L
from phrike_gb300 import problems

pytestmark = pytest.mark.gpu

GAMMA = 1.4
PRECS = ["fp32", "fp64", "bf16x3", "bf16x3_simt"]
RHS_TOL = {"fp64": 1e-5, "fp32": 1e-5, "bf16x3": 6e-5, "bf16x3_simt": 6e-5}


def _plan(nx, ny, prec="fp32", nsolve=1, filt=None, cfl=0.3):
    from phrike_gb300.engine import Plan
    return Plan((ny, nx), (2.0, 2.0), gamma=GAMMA, filter_params=filt, cfl=cfl, nsolve=nsolve,
                basis="legendre", gemm_precision=prec)


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


def _pulse(nx, ny, amp=0.01, width2=0.01):
    ax, ay = L.LGLAxis(nx, 2.0), L.LGLAxis(ny, 2.0)
    return problems.acoustic_pulse_lgl_2d(ax.x - 1.0, ay.x - 1.0, gamma=GAMMA, amp=amp, width2=width2)


def _field_errors(U, R):
    return [rel_l2(U[c], R[c]) for c in range(4)]


@pytest.mark.parametrize("n", [3, 4, 17, 64, 257, 513])
def test_lgl_build_matches_oracle(cuda_device, n):
    from phrike_gb300.engine import lgl_build
    x, w, D = lgl_build(n, 2.0)
    ax = L.LGLAxis(n, 2.0)
    np.testing.assert_allclose(x.cpu().numpy(), ax.x, rtol=0, atol=4e-16 * n)
    np.testing.assert_allclose(w.cpu().numpy(), ax.w_ref, rtol=2e-12, atol=0)
    Dg = D.cpu().numpy()
    assert np.abs(Dg - ax.D).max() <= 1e-10 * np.abs(ax.D).max()
    # derivative of a cubic is exact on n >= 4 nodes
    if n >= 4:
        xx = ax.x - 1.0
        np.testing.assert_allclose(Dg @ xx ** 3, 3 * xx ** 2, atol=1e-9 * n * n)


def test_lgl_walls_match_oracle(cuda_device):
    rng = np.random.default_rng(7)
    U = rng.uniform(0.5, 1.5, size=(4, 19, 23))
    p = _plan(23, 19)
    t = _dev(U)
    p.apply_boundary_conditions_(t)
    np.testing.assert_array_equal(t.cpu().numpy(), L.apply_wall_bc(U.astype(np.float32).copy()))


@pytest.mark.parametrize("prec", PRECS)
def test_lgl_derivatives_and_filter(cuda_device, prec):
    """dx1/dy1 and the nodal filter against the oracle applied to the same
    float32 inputs; one field carries a large constant offset (the pencil
    offset keeps its derivative accurate in the split modes)."""
    nx, ny = 65, 33
    ax, ay = L.LGLAxis(nx, 2.0), L.LGLAxis(ny, 2.0)
    X, Y = np.meshgrid(ax.x - 1.0, ay.x - 1.0, indexing="xy")
    f = np.stack([np.sin(2 * X) * np.cos(3 * Y), np.exp(X * Y), X ** 5 - Y ** 3,
                  1.0 + 0.01 * np.exp(-(X ** 2 + Y ** 2) / 0.05)]).astype(np.float32)
    f64 = f.astype(np.float64)
    p = _plan(nx, ny, prec, filt={"enabled": True, "p": 8, "alpha": 36.0})
    tol = {"fp64": 1e-7, "fp32": 3e-5, "bf16x3": 3e-3, "bf16x3_simt": 3e-3}[prec]
    dx = p.derivative(_dev(f), 0).cpu().numpy()
    dy = p.derivative(_dev(f), 1).cpu().numpy()
    ref_dx = f64 @ ax.D.T
    ref_dy = np.einsum("jk,cki->cji", ay.D, f64)
    for c in range(4):
        assert rel_l2(dx[c], ref_dx[c]) < tol, (c, rel_l2(dx[c], ref_dx[c]))
        assert rel_l2(dy[c], ref_dy[c]) < tol, (c, rel_l2(dy[c], ref_dy[c]))
    Fx, Fy = ax.nodal_filter(8, 36.0), ay.nodal_filter(8, 36.0)
    ff = p.filter(_dev(f)).cpu().numpy()
    ref = np.einsum("jk,cki->cji", Fy, f64 @ Fx.T)
    ftol = {"fp64": 1e-7, "fp32": 1e-6, "bf16x3": 3e-5, "bf16x3_simt": 3e-5}[prec]
    for c in range(4):
        assert rel_l2(ff[c], ref[c]) < ftol, (c, rel_l2(ff[c], ref[c]))
    # in-place derivative
    g = _dev(f)
    p.derivative(g, 1, out=g)
    assert rel_l2(g.cpu().numpy(), dy) < 1e-7


@pytest.mark.parametrize("nx,ny", [(17, 17), (33, 17)])
@pytest.mark.parametrize("prec", PRECS)
def test_lgl_rhs_and_steps_match_reference(cuda_device, nx, ny, prec):
    z = golden(f"lgl2d_{nx}x{ny}.npz")
    p = _plan(nx, ny, prec)
    U0 = _dev(z["U0"])
    rhs = p.rhs(U0).cpu().numpy()
    # momentum compared as a vector field; density and energy per field
    errs = [rel_l2(rhs[0], z["rhs0"][0]), rel_l2(rhs[1:3], z["rhs0"][1:3]), rel_l2(rhs[3], z["rhs0"][3])]
    assert max(errs) < RHS_TOL[prec], errs
    np.testing.assert_array_equal(U0.cpu().numpy(), z["U0"].astype(np.float32))  # rhs leaves U alone
    U = _dev(z["U0"])
    p.run_(U, int(z["nsteps"]), float(z["dt"]))
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], z["U"][0]), rel_l2(G[3], z["U"][3])) < 2e-7
    assert rel_l2(G[1:3], z["U"][1:3]) < RHS_TOL[prec]


@pytest.mark.parametrize("n", [17, 65, 257, 513])
def test_lgl_tensor_cores_match_cuda_core_split(cuda_device, n):
    """The tcgen05 split-bf16 x3 contractions against the same split
    arithmetic on CUDA cores, on a state with a velocity field that vanishes
    at the walls: they differ only in float32 accumulation order."""
    ax = L.LGLAxis(n, 2.0)
    x = ax.x - 1.0
    X, Y = np.meshgrid(x, x, indexing="xy")
    rho = 1.0 + 0.2 * np.exp(-(X ** 2 + Y ** 2) / 0.05)
    u = 0.3 * np.sin(np.pi * X) * np.cos(0.5 * np.pi * Y)
    v = -0.2 * np.cos(0.5 * np.pi * X) * np.sin(np.pi * Y)
    pr = rho ** GAMMA / GAMMA
    U0 = np.stack([rho, rho * u, rho * v, pr / (GAMMA - 1) + 0.5 * rho * (u * u + v * v)])
    r_tc = _plan(n, n, "bf16x3").rhs(_dev(U0)).cpu().numpy()
    r_cc = _plan(n, n, "bf16x3_simt").rhs(_dev(U0)).cpu().numpy()
    for c in range(4):
        assert rel_l2(r_tc[c], r_cc[c]) < 1e-5, (c, rel_l2(r_tc[c], r_cc[c]))
    Ua, Ub = _dev(U0), _dev(U0)
    pa, pb = _plan(n, n, "bf16x3"), _plan(n, n, "bf16x3_simt")
    pa.run_(Ua, 5, 1e-5)
    pb.run_(Ub, 5, 1e-5)
    Ga, Gb = Ua.cpu().numpy(), Ub.cpu().numpy()
    for c in range(4):
        assert rel_l2(Ga[c], Gb[c]) < 1e-6, (c, rel_l2(Ga[c], Gb[c]))
    assert pa.status() == 0


# Momentum after a run, against the float64 oracle started from the same
# float32 initial state (the engine's input).  FP64 and FP32 contractions sit
# at the float32-state floor; split-bf16 x3 keeps about 16 significand bits
# of each operand (measured 1.1e-5 at 65^2, 3.0e-5 at 257^2 and 4.6e-5 at
# 513^2 after 500 steps).
MOM_TOL = {"fp64": 1e-5, "fp32": 1e-5, "bf16x3": 6e-5, "bf16x3_simt": 6e-5}


def _oracle_steps(n, U0, nsteps, dt, **kw):
    s = L.LGLSolver2D(n, n, gamma=GAMMA, **kw)
    R = U0.astype(np.float32).astype(np.float64)
    for _ in range(nsteps):
        R = s.step(R, dt)
    return R


@pytest.mark.parametrize("prec", PRECS)
def test_lgl_acoustic_pulse_vs_oracle(cuda_device, prec):
    """The acoustic Gaussian pulse (amplitude 0.01, width^2 0.01) on 65 x 65
    LGL nodes, 500 steps of dt = 1e-5 (measured momentum 4.2e-7 for FP64 and
    FP32 contractions, 1.1e-5 for split-bf16 x3)."""
    n, nsteps, dt = 65, 500, 1e-5
    U0 = _pulse(n, n)
    R = _oracle_steps(n, U0, nsteps, dt)
    p = _plan(n, n, prec)
    U = _dev(U0)
    p.run_(U, nsteps, dt)
    G = U.cpu().numpy()
    assert rel_l2(G[0], R[0]) < 1e-6
    assert rel_l2(G[3], R[3]) < 1e-7
    tol = 2e-6 if prec in ("fp32", "fp64") else 3e-5
    assert rel_l2(G[1:3], R[1:3]) < tol, rel_l2(G[1:3], R[1:3])
    assert p.status() == 0


@pytest.mark.parametrize("n,prec", [(257, "fp32"), (257, "bf16x3"), (513, "fp32"), (513, "bf16x3")])
def test_lgl_workload_size_500_steps(cuda_device, n, prec):
    """The precision workload at its stated sizes: 257^2 and 513^2 nodes, 500
    steps of dt = 1e-5 (measured momentum: FP32 2.1e-6 and 6.1e-6,
    split-bf16 x3 3.0e-5 and 4.6e-5; density 6.4e-7, energy 4.4e-9)."""
    U0 = _pulse(n, n)
    R = _oracle_steps(n, U0, 500, 1e-5)
    p = _plan(n, n, prec)
    U = _dev(U0)
    p.run_(U, 500, 1e-5)
    G = U.cpu().numpy()
    e = (rel_l2(G[0], R[0]), rel_l2(G[1:3], R[1:3]), rel_l2(G[3], R[3]))
    print(f"\nLGL {n}^2 {prec} 500 steps: rho {e[0]:.2e} mom {e[1]:.2e} E {e[2]:.2e}")
    assert e[0] < 2e-6 and e[2] < 1e-7, e
    assert e[1] < MOM_TOL[prec], e
    assert p.status() == 0


def test_lgl_filter_in_step(cuda_device):
    n, nsteps, dt = 33, 20, 1e-4
    fp = {"enabled": True, "p": 8, "alpha": 36.0, "interval": 3}
    U0 = _pulse(n, n, amp=0.2, width2=0.05)
    R = _oracle_steps(n, U0, 0, dt)
    s = L.LGLSolver2D(n, n, gamma=GAMMA, filter_params=fp)
    for _ in range(nsteps):
        R = s.step(R, dt)
    p = _plan(n, n, "fp32", filt=fp)
    U = _dev(U0)
    for _ in range(nsteps):
        p.step_(U, dt)
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], R[0]), rel_l2(G[3], R[3])) < 2e-6
    assert rel_l2(G[1:3], R[1:3]) < 1e-5, rel_l2(G[1:3], R[1:3])


def test_lgl_cfl_run_vs_oracle(cuda_device):
    import torch
    n, t_end = 33, 0.02
    U0 = _pulse(n, n, amp=0.2, width2=0.05)
    s = L.LGLSolver2D(n, n, gamma=GAMMA, cfl=0.3)
    R, t, steps = U0.astype(np.float32).astype(np.float64), 0.0, 0
    while t < t_end - 1e-12:
        dt = min(s.compute_dt(R), t_end - t)
        R = s.step(R, dt)
        t += dt
        steps += 1
    p = _plan(n, n, "fp32", cfl=0.3)
    U = _dev(U0)
    tt = torch.zeros(1, dtype=torch.float64, device="cuda")
    te = torch.full((1,), t_end, dtype=torch.float64, device="cuda")
    p.run_cfl_(U, steps + 3, tt, te)
    assert abs(float(tt.item()) - t_end) < 1e-12
    assert p.steps_done() == [steps]
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], R[0]), rel_l2(G[3], R[3])) < 2e-6
    assert rel_l2(G[1:3], R[1:3]) < 1e-5, rel_l2(G[1:3], R[1:3])


def test_lgl_batch_matches_alone(cuda_device):
    import torch
    n, nsteps, dt = 41, 10, 2e-5
    states = [_pulse(n, n, amp=a, width2=w) for a, w in ((0.01, 0.01), (0.1, 0.02), (0.05, 0.05))]
    pb = _plan(n, n, "fp32", nsolve=3)
    Ub = _dev(np.stack(states))
    pb.run_(Ub, nsteps, dt)
    for i, st in enumerate(states):
        p1 = _plan(n, n, "fp32")
        U1 = _dev(st)
        p1.run_(U1, nsteps, dt)
        assert torch.equal(U1, Ub[i]), i


def test_lgl_properties_257(cuda_device):
    """Config-size grid (257 x 257, 50 steps of dt = 1e-5): mass is conserved
    to the quadrature accuracy, the pulse stays symmetric under x <-> y, the
    walls hold and nothing becomes non-finite."""
    import torch
    n = 257
    p = _plan(n, n, "bf16x3")
    U0 = _pulse(n, n)
    U = _dev(U0)
    p.run_(U, 50, 1e-5)
    G = U.cpu().numpy()
    assert np.isfinite(G).all()
    w = L.LGLAxis(n, 2.0).w_ref
    W = np.outer(w, w)
    m0, m1 = (W * U0[0]).sum(), (W * G[0].astype(np.float64)).sum()
    assert abs(m1 - m0) / m0 < 1e-6
    assert np.abs(G[0] - G[0].T).max() < 1e-5
    assert np.abs(G[1] - G[2].T).max() < 1e-5
    np.testing.assert_array_equal(G[1][:, 0], 0.0)
    np.testing.assert_array_equal(G[2][0, :], 0.0)
    assert p.status() == 0
    del torch


def test_tensor_core_n_tiles_give_the_same_bits(cuda_device):
    """The N tile of the tcgen05 contractions (64, 128, 176, 256 and the
    plan's own choice) changes which columns a CTA computes, not the dot
    product of any output value: two solves stepped five times end bitwise
    equal for every tile; the autotuner returns one of them."""
    import torch
    from phrike_gb300.autotune import tune_umma_n_tile
    from phrike_gb300.engine import Plan
    n = 65
    ax = L.LGLAxis(n, 2.0)
    U0 = problems.acoustic_pulse_lgl_2d(ax.x - 1.0, ax.x - 1.0, gamma=GAMMA)
    UB = torch.as_tensor(np.stack([U0, U0[:, ::-1, :].copy()]), dtype=torch.float32, device=cuda_device).contiguous()
    outs = []
    for nt in (None, 64, 128, 176, 256):
        plan = Plan((n, n), (2.0, 2.0), gamma=GAMMA, basis="legendre", gemm_precision="bf16x3", nsolve=2,
                    umma_n_tile=nt, device=cuda_device)
        V = UB.clone()
        plan.run_(V, 5, 1e-5)
        assert plan.status() == 0
        outs.append(V)
        plan.close()
    for V in outs[1:]:
        assert torch.equal(outs[0], V)
    best, times = tune_umma_n_tile((n, n), (2.0, 2.0), UB, nsolve=2, gamma=GAMMA, device=cuda_device)
    assert best in (64, 128, 176, 256) and set(times) == {64, 128, 176, 256}
    with pytest.raises(RuntimeError):
        Plan((n, n), (2.0, 2.0), basis="legendre", gemm_precision="bf16x3", umma_n_tile=96, device=cuda_device)
