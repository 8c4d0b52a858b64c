"""The serving loop: continuous batching of a mixed request stream (Sod 1D,
KHI 2D, Orszag-Tang MHD, TGV 3D, LGL acoustic) on one GPU.  Requests arrive
while others are running, are admitted into free slots of resident batched
plans, overlap on the device and retire at their end times.  Every result
must equal the same solve run alone (same kernels and arithmetic per slot):
the stated tolerance is zero, bit-identical states."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMALL = {"sod1d": [256, 512], "khi2d": [32, 64], "ot2d": [32, 64], "tgv3d": [16, 32], "lgl2d": [17, 33]}


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
