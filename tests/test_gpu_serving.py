"""The serving loop: continuous batching of a mixed request stream (Sod 1D,
KHI 2D, Orszag-Tang MHD, TGV 3D, 1D and 2D LGL acoustic) on one GPU.  Requests arrive
while others are running, are admitted into free slots of resident batched
plans, overlap on the device and retire at their end times.  Every result
must equal the same solve run alone (same kernels and arithmetic per slot):
the stated tolerance is zero, bit-identical states."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMALL = {"sod1d": [256, 512], "khi2d": [32, 64], "ot2d": [32, 64], "tgv3d": [16, 32], "lgl2d": [17, 33], "lgl1d": [17, 33]}


def _stream(count, seed=7, rate=400.0):
    from phrike_gb300.serving import request_stream
    return request_stream(count, rate=rate, seed=seed, t_end_range=(0.005, 0.03), families=SMALL)


def _check_alone(srv, reqs, device):
    from phrike_gb300.serving import run_alone
    for r in reqs:
        U, _ = run_alone(r, device, chunk=srv.chunk)
        got = srv.results[r.rid]
        assert np.array_equal(U.cpu().numpy(), got), (r.family, r.n, np.abs(U.cpu().numpy() - got).max())


def test_serving_results_equal_alone(cuda_device):
    from phrike_gb300.serving import Server
    reqs = _stream(20)
    srv = Server(cuda_device, chunk=5)
    stats = srv.serve(reqs, realtime=True, max_seconds=600)
    assert stats["requests"] == 20 and stats["status"] == 0
    assert stats["max_live_slots"] > 1  # requests overlapped on the device
    assert len(srv.results) == 20
    assert stats["latency_p50"] <= stats["latency_p95"] <= stats["latency_p99"]
    _check_alone(srv, reqs, cuda_device)


def test_serving_under_a_tight_hbm_budget(cuda_device):
    """With room for few groups, later requests wait for free slots and are
    admitted as earlier ones retire; results are unchanged."""
    from phrike_gb300.serving import Server, make_plan_bytes
    reqs = [r for r in _stream(16, seed=11) if r.family in ("khi2d", "sod1d")]
    one = max(make_plan_bytes(r.family, r.n, 2) + 4 * 4 * 2 * r.n ** 2 + 32 for r in reqs)
    srv = Server(cuda_device, chunk=5, budget_bytes=3 * one, slots=lambda f, n: 2)
    stats = srv.serve(reqs, realtime=False, max_seconds=600)
    assert stats["requests"] == len(reqs)
    assert srv.used <= 3 * one
    _check_alone(srv, reqs, cuda_device)


def test_serving_pause_and_resume(cuda_device, tmp_path):
    """A served solve paused at a chunk boundary (its Snapshot written to
    disk and read back) and resumed later in the mix ends bit-identical to the
    resumed solve run alone, and within float32 rounding of the solve run
    without the pause."""
    from conftest import rel_l2
    from phrike_gb300.io import Snapshot
    from phrike_gb300.serving import Request, Server, run_alone
    reqs = [Request(0, "khi2d", 64, 0.04, 0.0, {"U0": 1.1, "A": 0.012}),
            Request(1, "sod1d", 256, 0.03, 0.0), Request(2, "khi2d", 64, 0.02, 0.0, {"U0": 0.8, "A": 0.01})]
    srv = Server(cuda_device, chunk=5)
    srv.serve(reqs, realtime=False, pause_at={0: 0.015})
    assert 0 in srv.paused and 0 not in srv.results
    snap = srv.paused[0]
    assert 0.015 <= snap.t < 0.04
    snap = Snapshot.load(snap.save(str(tmp_path / "paused.npz")))
    later = [Request.resume(0, snap), Request(3, "khi2d", 64, 0.01, 0.0, {"U0": 1.3, "A": 0.02})]
    srv.serve(later, realtime=False)
    U, _ = run_alone(Request.resume(0, snap), cuda_device, chunk=srv.chunk)
    assert np.array_equal(srv.results[0], U.cpu().numpy())
    W, _ = run_alone(Request(9, "khi2d", 64, 0.04, 0.0, {"U0": 1.1, "A": 0.012}), cuda_device, chunk=srv.chunk)
    assert rel_l2(srv.results[0], W.cpu().numpy()) < 1e-5
