"""Parity at the workloads' stated sizes and end times against the float64
oracle (fixtures from tests/golden/make_large_parity.py, stored on a
sub-lattice; tests/parity_cases.py).

* Taylor-Green vortex, 128^3 and 256^3, 200 fixed steps of dt = 1e-3:
  relative L2 per conserved field within 1e-5, momentum against the
  momentum-vector norm.  Per component (each momentum component against its
  own norm) the z momentum, which the flow generates from zero, measures
  1.8e-5 at 128^3; the bound is 4e-5.
* Kelvin-Helmholtz, one ensemble draw per grid size (64^2 .. 512^2), CFL 0.4
  to t_end = 1.0 with the time loop on the device: within 1e-5 (momentum
  vector) at 64^2 to 256^2 (measured 8.5e-6, 2.1e-6, 3.1e-6).  At 512^2 the
  rolled-up shear layers amplify float32 rounding exponentially: measured
  5.7e-5, bound 1.2e-4.  Per component, the y momentum (the perturbation,
  1e-2 of the x momentum) measures 1e-4 to 1.9e-2 against its own norm.
"""
import numpy as np
import pytest
import torch

import parity_cases as PC
from conftest import golden
from phrike_gb300 import problems
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu

TGV_COMPONENT_TOL = 4e-5
KHI_TOL = {64: 1e-5, 128: 1e-5, 256: 1e-5, 512: 1.2e-4}


@pytest.mark.parametrize("n", [128, 256])
def test_tgv_workload_size_200_steps(cuda_device, n):
    z = golden(f"tgv3d_{n}_200.npz")
    plan = Plan((n, n, n), (2 * np.pi,) * 3, device=cuda_device)
    U = torch.as_tensor(problems.taylor_green_3d(n), dtype=torch.float32, device=cuda_device).contiguous()
    plan.run_(U, int(z["steps"]), float(z["dt"]))
    torch.cuda.synchronize()
    assert plan.status() == 0
    st = int(z["stride"])
    out = PC.sub(U.cpu().numpy(), st).astype(np.float64)
    e = PC.field_errors(out, z["U"])
    print(f"\nTGV {n}^3 200 steps rel-L2 vector {e['vector']} component {e['component']}")
    assert max(e["vector"]) < 1e-5, e
    assert max(e["component"]) < TGV_COMPONENT_TOL, e
    plan.close()


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_khi_ensemble_draw_to_t_end(cuda_device, n):
    z = golden("khi_c4_t1.npz")
    u0, amp = float(z[f"n{n}_u0"]), float(z[f"n{n}_amp"])
    plan = Plan((n, n), (1.0, 1.0), cfl=PC.KHI_CFL, device=cuda_device)
    U = torch.as_tensor(problems.kelvin_helmholtz_2d(n, n, U0=u0, A=amp), dtype=torch.float32,
                        device=cuda_device).contiguous()
    t = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    te = torch.full((1,), PC.KHI_T_END, dtype=torch.float64, device=cuda_device)
    nref = int(z[f"n{n}_steps"])
    plan.run_cfl_(U, nref + 64, t, te)
    torch.cuda.synchronize()
    assert abs(float(t.item()) - PC.KHI_T_END) < 1e-12
    assert plan.status() == 0
    steps = int(plan.steps_done()[0])
    assert abs(steps - nref) <= 1, (steps, nref)
    st = int(z[f"n{n}_stride"])
    out = PC.sub(U.cpu().numpy(), st).astype(np.float64)
    e = PC.field_errors(out, z[f"n{n}_U"])
    print(f"\nKHI {n}^2 t=1 ({steps} steps) rel-L2 vector {e['vector']} component {e['component']}")
    assert max(e["vector"]) < KHI_TOL[n], e
    plan.close()
