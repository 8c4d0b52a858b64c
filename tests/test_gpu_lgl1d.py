"""1D Legendre-Gauss-Lobatto path on the GPU (one CTA per solve, whole RK
steps per launch) against the reference's golden vectors and the oracle:
the right-hand side with the boundary codes, RK4/RK2 steps with the nodal
filter, per-boundary/per-variable boundary maps and gravity, the boundary
kernel, derivative and filter, CFL runs and batches.

Tolerances.  The state is float32 with the energy held as E - E_ref.  The
derivative and the filter are summed as sum_j M_ij (u_j - u_i) (+ u_i for the
filter), so float32 rounding of M and u stays relative to u's variation: a
float32 emulation of 300 filter applications on the 33-node pulse gives
3e-7 relative against 5e-6 for the plain sum."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from lgl1d_cases import CASES, DT, LENGTH, NSTEPS, initial_state
from oracle import lgl as L

pytestmark = pytest.mark.gpu

GAMMA = 1.4
PRECS = ["fp32", "fp64"]


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


def _grid(tag, prec="fp32"):
    from phrike_gb300.grid import Grid1D
    c = CASES[tag]
    return Grid1D(N=c["n"], Lx=LENGTH, basis="legendre", bc=c["bc"], filter_params=c["filter_params"],
                  gemm_precision=prec)


def _solver(tag, prec="fp32", cfl=0.4):
    from phrike_gb300.equations import EulerEquations1D
    from phrike_gb300.solver import SpectralSolver1D
    c = CASES[tag]
    gc = {"enabled": True, "gx": c["gravity"]} if c["gravity"] is not None else None
    return SpectralSolver1D(_grid(tag, prec), EulerEquations1D(gamma=GAMMA), scheme=c["scheme"], cfl=cfl,
                            gravity_config=gc)


def _oracle(tag, cfl=0.4):
    c = CASES[tag]
    return L.LGLSolver1D(c["n"], LENGTH, gamma=GAMMA, filter_params=c["filter_params"], cfl=cfl,
                         bc=c["bc"] if c["bc"] is not None else "dirichlet", gravity=c["gravity"],
                         scheme=c["scheme"])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("tag", ["wall", "mixed"])
def test_lgl1d_rhs_and_steps_match_reference(cuda_device, tag, prec):
    z = golden("lgl1d.npz")
    s = _solver(tag, prec)
    np.testing.assert_allclose(s.grid.x.cpu().numpy(), z[f"{tag}_x"], rtol=0, atol=1e-14)
    U0 = _dev(z[f"{tag}_U0"])
    r = s.plan.rhs(U0).cpu().numpy()
    for k in range(3):
        assert rel_l2(r[k], z[f"{tag}_rhs0"][k]) < 1e-5, (k, rel_l2(r[k], z[f"{tag}_rhs0"][k]))
    np.testing.assert_array_equal(U0.cpu().numpy(), z[f"{tag}_U0"].astype(np.float32))  # rhs leaves U alone
    U = _dev(z[f"{tag}_U0"])
    for _ in range(NSTEPS):
        U = s.step(U, DT)
    G = U.cpu().numpy() if hasattr(U, "cpu") else np.asarray(U)
    assert rel_l2(G[0], z[f"{tag}_U"][0]) < 1e-6
    assert rel_l2(G[2], z[f"{tag}_U"][2]) < 1e-6
    assert rel_l2(G[1], z[f"{tag}_U"][1]) < 2e-5, rel_l2(G[1], z[f"{tag}_U"][1])
    assert abs(s.compute_dt(z[f"{tag}_U0"]) - float(z[f"{tag}_dt0"])) < 1e-5 * float(z[f"{tag}_dt0"])
    assert s.plan.status() == 0


@pytest.mark.parametrize("bc", ["dirichlet", "open", "periodic",
                                {"left": {"density": "neumann", "momentum": "wall", "pressure": "open"},
                                 "right": {"u": "open", "rho": "periodic"}}])
def test_lgl1d_boundary_kernel_matches_oracle(cuda_device, bc):
    from phrike_gb300.engine import Plan
    from phrike_gb300.grid import Grid1D
    rng = np.random.default_rng(11)
    U = rng.uniform(0.5, 1.5, size=(2, 3, 29))
    codes = L.bc_codes_1d(bc)
    g = Grid1D(N=29, Lx=1.0, basis="legendre", bc=bc)
    t = _dev(U[0])
    g.apply_boundary_conditions(t)
    np.testing.assert_array_equal(t.cpu().numpy(), L.apply_bc_1d(U[0].astype(np.float32).copy(), codes))
    # a batch of two solves through the plan
    p = Plan((29,), (1.0,), nsolve=2, basis="legendre", lgl_bc1d=codes.reshape(-1).tolist())
    t = _dev(U)
    p.apply_boundary_conditions_(t)
    want = np.stack([L.apply_bc_1d(u.astype(np.float32).copy(), codes) for u in U])
    np.testing.assert_array_equal(t.cpu().numpy(), want)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [5, 33, 257, 1025])
def test_lgl1d_derivative_and_filter(cuda_device, n, prec):
    from phrike_gb300.grid import Grid1D
    ax = L.LGLAxis(n, 2.0)
    x = ax.x - 1.0
    f = np.stack([np.sin(2 * x), np.exp(x), x ** 3 - x, 1.0 + 0.01 * np.exp(-x * x / 0.05)]).astype(np.float32)
    f64 = f.astype(np.float64)
    g = Grid1D(N=n, Lx=2.0, basis="legendre", filter_params={"enabled": True, "p": 8, "alpha": 36.0},
               gemm_precision=prec)
    d = g.dx1(_dev(f)).cpu().numpy()
    ref = f64 @ ax.D.T
    tol = {"fp64": 1e-7, "fp32": 3e-5}[prec] * max(1.0, n / 257)
    for c in range(4):
        assert rel_l2(d[c], ref[c]) < tol, (c, rel_l2(d[c], ref[c]))
    ff = g.apply_spectral_filter(_dev(f)).cpu().numpy()
    ref = f64 @ ax.nodal_filter(8, 36.0).T
    for c in range(4):
        assert rel_l2(ff[c], ref[c]) < {"fp64": 1e-7, "fp32": 2e-6}[prec], (c, rel_l2(ff[c], ref[c]))


@pytest.mark.parametrize("tag", ["wall", "mixed"])
def test_lgl1d_long_run_vs_oracle(cuda_device, tag):
    """200 steps of dt = 2e-4 against the float64 oracle."""
    s, o = _solver(tag), _oracle(tag)
    U0 = initial_state(L.LGLAxis(CASES[tag]["n"], LENGTH).x)
    R = U0.astype(np.float32).astype(np.float64)  # the oracle from the engine's float32 input
    for _ in range(200):
        R = o.step(R, DT)
    U = _dev(U0)
    s.plan.run_(U, 200, DT)
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], R[0]), rel_l2(G[2], R[2])) < 5e-6
    assert rel_l2(G[1], R[1]) < 1e-5, rel_l2(G[1], R[1])
    assert s.plan.status() == 0


def test_lgl1d_cfl_run_vs_oracle(cuda_device):
    import torch
    tag, t_end = "wall", 0.05
    s, o = _solver(tag, cfl=0.3), _oracle(tag, cfl=0.3)
    U0 = initial_state(o.ax.x)
    R, t, steps = U0.astype(np.float32).astype(np.float64), 0.0, 0
    while t < t_end - 1e-12:
        dt = min(o.compute_dt(R), t_end - t)
        R = o.step(R, dt)
        t += dt
        steps += 1
    U = _dev(U0)
    tt = torch.zeros(1, dtype=torch.float64, device="cuda")
    te = torch.full((1,), t_end, dtype=torch.float64, device="cuda")
    s.plan.run_cfl_(U, steps + 3, tt, te)
    assert abs(float(tt.item()) - t_end) < 1e-12
    assert s.plan.steps_done() == [steps]
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], R[0]), rel_l2(G[2], R[2])) < 5e-6
    assert rel_l2(G[1], R[1]) < 1e-5, rel_l2(G[1], R[1])


def test_lgl1d_batch_matches_alone(cuda_device):
    import torch
    from phrike_gb300.engine import Plan
    n, nsteps = 41, 10
    x = L.LGLAxis(n, LENGTH).x
    states = [initial_state(x) * a for a in (1.0, 1.1, 0.9)]
    fp = {"enabled": True, "p": 8, "alpha": 36.0, "interval": 3}
    codes = L.bc_codes_1d("dirichlet").reshape(-1).tolist()
    pb = Plan((n,), (LENGTH,), gamma=GAMMA, filter_params=fp, nsolve=3, basis="legendre", lgl_bc1d=codes)
    Ub = _dev(np.stack(states))
    pb.run_(Ub, nsteps, DT)
    for i, st in enumerate(states):
        p1 = Plan((n,), (LENGTH,), gamma=GAMMA, filter_params=fp, basis="legendre", lgl_bc1d=codes)
        U1 = _dev(st)
        p1.run_(U1, nsteps, DT)
        assert torch.equal(U1, Ub[i]), i


def test_lgl1d_large_grid_properties(cuda_device):
    """2048 nodes (the kernel's largest, float64 contractions: about 136 KB of
    shared memory per CTA): mass is conserved to quadrature accuracy, walls
    hold and nothing becomes non-finite over 20 steps."""
    from phrike_gb300.engine import Plan
    n = 2048
    ax = L.LGLAxis(n, LENGTH)
    U0 = initial_state(ax.x)
    p = Plan((n,), (LENGTH,), gamma=GAMMA, basis="legendre", gemm_precision="fp64",
             lgl_bc1d=L.bc_codes_1d("wall").reshape(-1).tolist())
    U = _dev(U0)
    p.run_(U, 20, 1e-7)
    G = U.cpu().numpy()
    assert np.isfinite(G).all()
    m0, m1 = (ax.w_ref * U0[0]).sum(), (ax.w_ref * G[0].astype(np.float64)).sum()
    assert abs(m1 - m0) / m0 < 1e-5
    assert G[1][0] == 0.0 and G[1][-1] == 0.0
    assert p.status() == 0


@pytest.mark.parametrize("n", [257, 513])
@pytest.mark.parametrize("tag", ["wall", "mixed"])
def test_lgl1d_cluster_form_vs_oracle(cuda_device, n, tag):
    """130..513 nodes in float32 run as a cluster of CTAs per solve (rows of D
    in each CTA's shared memory, the stage state exchanged through
    distributed shared memory): rhs, 20 steps and a CFL run against the
    float64 oracle with the case's boundary map, filter, scheme and gravity."""
    import torch
    from phrike_gb300.engine import Plan
    c = CASES[tag]
    codes = L.bc_codes_1d(c["bc"] if c["bc"] is not None else "dirichlet").reshape(-1).tolist()
    gravity = [c["gravity"]] if c["gravity"] is not None else None
    mk = lambda cfl=0.4: Plan((n,), (LENGTH,), gamma=GAMMA, filter_params=c["filter_params"], cfl=cfl,  # noqa: E731
                              basis="legendre", lgl_bc1d=codes, scheme=c["scheme"], gravity=gravity)
    o = L.LGLSolver1D(n, LENGTH, gamma=GAMMA, filter_params=c["filter_params"], cfl=0.4,
                      bc=c["bc"] if c["bc"] is not None else "dirichlet", gravity=c["gravity"], scheme=c["scheme"])
    U0 = initial_state(o.ax.x)
    r = mk().rhs(_dev(U0)).cpu().numpy()
    ro = o.rhs(U0.copy())
    for k in range(3):
        assert rel_l2(r[k], ro[k]) < 3e-5 * (n / 257), (k, rel_l2(r[k], ro[k]))
    dt = 0.2 * o.compute_dt(U0)
    R = U0.astype(np.float32).astype(np.float64)
    for _ in range(20):
        R = o.step(R, dt)
    p = mk()
    U = _dev(U0)
    p.run_(U, 20, dt)
    G = U.cpu().numpy()
    assert max(rel_l2(G[0], R[0]), rel_l2(G[2], R[2])) < 5e-6
    assert rel_l2(G[1], R[1]) < 1e-5, rel_l2(G[1], R[1])
    assert p.status() == 0
    # CFL loop to a short end time, and a batch of two that matches the solve alone
    t_end = 10 * o.compute_dt(U0)
    pb = Plan((n,), (LENGTH,), gamma=GAMMA, filter_params=c["filter_params"], cfl=0.4, basis="legendre",
              lgl_bc1d=codes, scheme=c["scheme"], gravity=gravity, nsolve=2)
    Ub = _dev(np.stack([U0, U0 * np.array([1.05, 1.0, 1.05])[:, None]]))
    tb = torch.zeros(2, dtype=torch.float64, device="cuda")
    pb.run_cfl_(Ub, 40, tb, torch.full((2,), t_end, dtype=torch.float64, device="cuda"))
    p1 = mk()
    U1 = _dev(U0)
    t1 = torch.zeros(1, dtype=torch.float64, device="cuda")
    p1.run_cfl_(U1, 40, t1, torch.full((1,), t_end, dtype=torch.float64, device="cuda"))
    assert torch.equal(U1, Ub[0]) and abs(float(t1.item()) - t_end) < 1e-12
    assert pb.steps_done()[0] == p1.steps_done()[0]
