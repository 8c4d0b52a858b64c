"""Adaptive embedded RK (rk23 / rk45 / the reference's 8-stage "rk78") on the
GPU against the oracle, which is pinned to the reference's own adaptive runs
(tests/golden/adaptive.npz).  The same initial state (float32-rounded) and the
same first dt go to both; the accept/reject sequence must be identical and the
final state agree to float32 accuracy.  Also: batched solves give bitwise the
same result as solves run alone, the output pause, and the solver API."""
import numpy as np
import pytest

import adaptive_cases as C
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _errs(G, R):
    """Relative L2 errors of density, momentum (vector), energy (and B), each
    against its group's norm with a floor of 1e-2 of the whole state's norm."""
    G = np.asarray(G, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    nc = G.shape[0]
    if nc == 8:
        groups = (slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8))
    else:
        nd = nc - 2
        groups = (slice(0, 1), slice(1, 1 + nd), slice(nd + 1, nd + 2))
    floor = 1e-2 * np.linalg.norm(R)
    return [float(np.linalg.norm(G[g] - R[g]) / max(np.linalg.norm(R[g]), floor)) for g in groups]


def _plan(tag, nsolve=1):
    from phrike_gb300.engine import Plan
    c = C.GPU_CASES[tag]
    nd = len(c["shape"])
    grav = c.get("gravity")
    return Plan(c["shape"], c["lengths"], gamma=5.0 / 3.0 if c["kind"] == "mhd" else 1.4, dealias=True,
                filter_params=C.FILTER if c["filt"] else None, cfl=c["cfl"],
                gravity=(list(grav) + [0.0] * (nd - len(grav))) if grav else None,
                equations="mhd" if c["kind"] == "mhd" else "euler", av_config=c.get("av"), nsolve=nsolve)


def _setup(tag):
    U0 = C.initial_state(tag).astype(np.float32).astype(np.float64)
    _, _, cdt, prep = C.oracle_case(tag)
    return U0, cdt(prep(U0))


def _vecs(plan, t_end, dt0, n=1):
    import torch
    f64 = dict(dtype=torch.float64, device=plan.device)
    return (torch.zeros(n, **f64), torch.full((n,), t_end, **f64), torch.full((n,), dt0, **f64),
            torch.zeros((n, 2), dtype=torch.int32, device=plan.device))


@pytest.mark.parametrize("tag", list(C.GPU_CASES))
def test_adaptive_attempts_match_oracle(tag, cuda_device):
    import torch
    from phrike_gb300.engine import Plan
    c = C.GPU_CASES[tag]
    U0, dt0 = _setup(tag)
    margins = []
    Uo, to, log, _, _ = C.run_oracle(tag, U0, margins=margins, dt0=dt0)
    assert min(margins) > 0.01, "case too close to the accept threshold for a float32 comparison"
    plan = _plan(tag)
    ad = Plan.adaptive_desc(dict(scheme=c["method"], **c["ctrl"]))
    U = torch.as_tensor(U0, dtype=torch.float32, device=cuda_device).contiguous()
    if c["kind"] == "mhd":
        plan.project_state_(U)  # the MHD run loop projects U0 first
    t, te, dtv, counts = _vecs(plan, c["t_end"], dt0)
    seq, dts = [], []
    for _ in range(len(log)):
        before = counts[0, 0].item()
        dts.append(min(dtv.item(), c["t_end"] - t.item()))
        plan.run_adaptive_(U, 1, ad, t, te, dtv, None, counts)
        seq.append(counts[0, 0].item() > before)
    assert seq == [ok for _, ok in log]
    assert counts[0].tolist() == [sum(ok for _, ok in log), sum(not ok for _, ok in log)]
    # dt_next scales as err^(-1/order) and err carries the float32 rounding of
    # the stage slopes, so step sizes agree to a few parts in 1e4
    # (the last attempt is cut to t_end - t, so it carries the accumulated drift of t)
    np.testing.assert_allclose(dts[:-1], [d for d, _ in log][:-1], rtol=c.get("dt_rtol", 5e-3))
    assert abs(t.item() - to) < 1e-6 * c["t_end"]
    errs = _errs(U.cpu().numpy(), Uo)
    assert max(errs) < 2e-5, errs
    # the run finished: further attempts do nothing
    plan.run_adaptive_(U, 3, ad, t, te, dtv, None, counts)
    assert counts[0].tolist() == [sum(ok for _, ok in log), sum(not ok for _, ok in log)]
    # one call with all attempts on the device gives the same state
    V = torch.as_tensor(U0, dtype=torch.float32, device=cuda_device).contiguous()
    if c["kind"] == "mhd":
        plan.project_state_(V)
    plan.adaptive_reset()
    t2, te2, dt2, counts2 = _vecs(plan, c["t_end"], dt0)
    plan.run_adaptive_(V, len(log) + 2, ad, t2, te2, dt2, None, counts2)
    assert counts2[0].tolist() == counts[0].tolist()
    # every call re-bases the energy-perturbation form, so calls of different
    # lengths agree to rounding only
    assert rel_l2(V.cpu().numpy(), U.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("tag", ["sod256_rk45", "khi32_rk23_grav"])
def test_adaptive_batch_equals_alone(tag, cuda_device):
    """Three solves with different end times in one batched plan: each ends
    bitwise equal to the same solve run alone (per-solve dt, decisions and
    stopping on the device)."""
    import torch
    from phrike_gb300.engine import Plan
    c = C.GPU_CASES[tag]
    U0, dt0 = _setup(tag)
    ad = Plan.adaptive_desc(dict(scheme=c["method"], **c["ctrl"]))
    ends = [c["t_end"], 0.5 * c["t_end"], 0.75 * c["t_end"]]
    alone = []
    for te_ in ends:
        p1 = _plan(tag)
        U = torch.as_tensor(U0, dtype=torch.float32, device=cuda_device).contiguous()
        t, te, dtv, counts = _vecs(p1, te_, dt0)
        p1.run_adaptive_(U, 200, ad, t, te, dtv, None, counts)
        alone.append((U.clone(), t.item(), counts[0].tolist()))
    pb = _plan(tag, nsolve=3)
    UB = torch.as_tensor(np.stack([U0] * 3), dtype=torch.float32, device=cuda_device).contiguous()
    t, _, dtv, counts = _vecs(pb, 0.0, dt0, 3)
    te = torch.tensor(ends, dtype=torch.float64, device=cuda_device)
    pb.run_adaptive_(UB, 200, ad, t, te, dtv, None, counts)
    for i, (U, ti, ci) in enumerate(alone):
        assert torch.equal(UB[i], U), i
        assert t[i].item() == ti and counts[i].tolist() == ci, i


def test_adaptive_output_pause(cuda_device):
    """With t_out a solve stops after the attempt that reaches it; resuming
    continues the same attempt sequence."""
    import torch
    from phrike_gb300.engine import Plan
    tag = "sod256_rk45"
    c = C.GPU_CASES[tag]
    U0, dt0 = _setup(tag)
    ad = Plan.adaptive_desc(dict(scheme=c["method"], **c["ctrl"]))
    plan = _plan(tag)
    U = torch.as_tensor(U0, dtype=torch.float32, device=cuda_device).contiguous()
    t, te, dtv, counts = _vecs(plan, c["t_end"], dt0)
    tout = torch.full((1,), 0.5 * c["t_end"], dtype=torch.float64, device=cuda_device)
    plan.run_adaptive_(U, 500, ad, t, te, dtv, tout, counts)
    tp = t.item()
    assert tp + 1e-12 >= 0.5 * c["t_end"] and tp < c["t_end"]
    # the attempt before the pause had not reached t_out: replay attempt by attempt
    V = torch.as_tensor(U0, dtype=torch.float32, device=cuda_device).contiguous()
    p2 = _plan(tag)
    t2, te2, dt2, counts2 = _vecs(p2, c["t_end"], dt0)
    while t2.item() + 1e-12 < 0.5 * c["t_end"]:
        p2.run_adaptive_(V, 1, ad, t2, te2, dt2, None, counts2)
    assert counts2.tolist() == counts.tolist()
    assert abs(t2.item() - tp) < 1e-5 * c["t_end"]
    assert rel_l2(V.cpu().numpy(), U.cpu().numpy()) < 1e-6
    plan.run_adaptive_(U, 500, ad, t, te, dtv, None, counts)
    assert abs(t.item() - c["t_end"]) < 1e-12


def test_solver_api_adaptive_run_matches_oracle(cuda_device):
    """SpectralSolver1D(adaptive_config=...).run: on_step sees every accepted
    attempt with the reference's step_count (rejections included) and dt;
    history outputs are recorded after the same attempts."""
    import torch
    from phrike_gb300 import Grid1D, EulerEquations1D
    from phrike_gb300.solver import SpectralSolver1D
    tag = "sod256_rk45"
    c = C.GPU_CASES[tag]
    grid = Grid1D(N=256, Lx=1.0, dealias=True, filter_params=C.FILTER)
    U0 = C.initial_state(tag).astype(np.float32).astype(np.float64)
    s = SpectralSolver1D(grid, EulerEquations1D(gamma=1.4), cfl=0.4,
                         adaptive_config=dict(enabled=True, scheme="rk45", **c["ctrl"]))
    dt0 = s.compute_dt(torch.as_tensor(U0, dtype=torch.float32, device=cuda_device))
    Uo, to, log, _, _ = C.run_oracle(tag, U0, dt0=dt0)
    seen = []
    hist = s.run(U0, 0.0, c["t_end"], output_interval=c["t_end"] / 3, on_step=lambda n, dt, U: seen.append((n, dt)))
    ref = C.accepted_steps(log)
    got = np.array(seen, dtype=np.float64).reshape(-1, 2)
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got[:, 0], ref[:, 0])
    np.testing.assert_allclose(got[:, 1], ref[:, 1], rtol=2e-3)
    assert abs(s.t - to) < 1e-9 and len(hist["time"]) >= 4
    assert max(_errs(s.U.cpu().numpy(), Uo)) < 2e-5
    # without on_step the attempts run in device chunks that pause at outputs
    s2 = SpectralSolver1D(grid, EulerEquations1D(gamma=1.4), cfl=0.4,
                          adaptive_config=dict(enabled=True, scheme="rk45", **c["ctrl"]))
    hist2 = s2.run(U0, 0.0, c["t_end"], output_interval=c["t_end"] / 3)
    np.testing.assert_allclose(hist2["time"], hist["time"], rtol=1e-5)
    assert rel_l2(s2.U.cpu().numpy(), s.U.cpu().numpy()) < 1e-6
