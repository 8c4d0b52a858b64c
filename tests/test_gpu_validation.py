"""Accuracy of the plain form (bench.py validation_report): the 3D TGV
against the float64 oracle, conservation drift, the spectral-convergence
slope of the masked derivative and the RK4 temporal order on the exact
circularly polarized Alfven wave."""
import pytest

pytestmark = pytest.mark.gpu


def test_validation_report(cuda_device):
    from bench import validation_report
    r = validation_report(cuda_device, tgv_n=32, tgv_steps=50, drift_n=64, drift_steps=50)
    e = r["tgv_rel_l2"]
    assert max(e["rho"], e["mom"], e["E"]) < 1e-5, e
    d = r["tgv_drift"]
    assert d["mass"] < 1e-6 and d["energy"] < 1e-6 and d["momentum"] < 1e-6, d
    c = r["spectral_convergence"]
    for N in (8, 16, 32):  # above the float32 floor the GPU follows the float64 errors
        g, o = c["errors"][N]["gpu"], c["errors"][N]["oracle"]
        assert abs(g - o) < 0.02 * o + 3e-7, (N, g, o)
    assert abs(c["slope_16_32"]["gpu"] - c["slope_16_32"]["oracle"]) < 0.01
    assert c["errors"][128]["gpu"] < 3e-6  # the float32 floor of the derivative (measured 1.1e-6)
    o = r["rk4_order"]
    assert 3.8 < o["gpu_orders"][0] < 4.2, o
    assert abs(o["oracle_order"] - 4.0) < 0.05
