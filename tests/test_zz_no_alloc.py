"""The allocation-free right-hand side (ps_rhs_static) against the plan-based
one (ps_rhs), through the C ABI.

ps_rhs_static exists for callers that cannot allocate device memory at the
point where they evaluate a right-hand side (inside a stream capture, inside
a framework that owns every allocation, in an allocation-free loop).  It runs
the same pass kernels as ps_rhs with its scratch in a static device array, so
its output must match ps_rhs to float32 rounding (the spectral tables are built
on the device instead of the host; tolerance 1e-6 relative L2).  Two calls in
a row on different grids check that the shared array carries nothing stale
from the previous call.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from phrike_gb300 import _lib, problems
from phrike_gb300.engine import Plan

pytestmark = pytest.mark.gpu


def _desc(shape_xyz, lengths_xyz, filt=False):
    lib = _lib.load()
    d = _lib.PlanDesc()
    _lib.check(lib.ps_plan_desc_init(C.byref(d), len(shape_xyz)))
    for a, (n, L) in enumerate(zip(shape_xyz, lengths_xyz)):
        d.n[a] = n
        d.length[a] = L
    d.filter_enabled = 1 if filt else 0
    return d


def _static_rhs(desc, U):
    lib = _lib.load()
    out = torch.full_like(U, float("nan"))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ps_rhs_static(C.byref(desc), C.c_void_p(U.data_ptr()), C.c_void_p(out.data_ptr()), stream)
    _lib.check(rc)
    torch.cuda.synchronize()
    return out


def _rel(a, b):
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


def test_static_rhs_matches_plan_rhs_two_calls(cuda_device):
    # call 1: 3D Taylor-Green, 32 x 16 x 64 (x, y, z)
    U3 = torch.as_tensor(problems.taylor_green_3d(32, 16, 64), dtype=torch.float32,
                         device=cuda_device).contiguous()
    plan3 = Plan((64, 16, 32), (2 * np.pi,) * 3, device=cuda_device)
    ref3 = plan3.rhs(U3)
    got3 = _static_rhs(_desc((32, 16, 64), (2 * np.pi,) * 3), U3)
    assert torch.isfinite(got3).all()
    assert _rel(got3, ref3) < 1e-6
    # call 2: 2D Kelvin-Helmholtz 128^2 with the exponential filter on
    U2 = torch.as_tensor(problems.kelvin_helmholtz_2d(128, 128, U0=1.1, A=0.02), dtype=torch.float32,
                         device=cuda_device).contiguous()
    plan2 = Plan((128, 128), (1.0, 1.0), filter_params={"enabled": True, "p": 8, "alpha": 36.0},
                 device=cuda_device)
    ref2 = plan2.rhs(U2)
    got2 = _static_rhs(_desc((128, 128), (1.0, 1.0), filt=True), U2)
    assert torch.isfinite(got2).all()
    assert _rel(got2, ref2) < 1e-6
    # call 3: the first grid again, after the second overwrote the array
    got3b = _static_rhs(_desc((32, 16, 64), (2 * np.pi,) * 3), U3)
    assert _rel(got3b, ref3) < 1e-6
    plan3.close()
    plan2.close()


@pytest.mark.parametrize("nx,ny", [(1024, 64), (64, 1024), (512, 128)])
def test_static_rhs_long_pencils_at_the_limit(cuda_device, nx, ny):
    """Grids of exactly the cell limit whose long axis takes the grouped
    pencils (group twiddles built on the device), filter on, two calls."""
    U = torch.as_tensor(problems.kelvin_helmholtz_2d(nx, ny, U0=0.9, A=0.015), dtype=torch.float32,
                        device=cuda_device).contiguous()
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    plan = Plan((ny, nx), (1.0, 1.0), filter_params=fp, device=cuda_device)
    ref = plan.rhs(U)
    for _ in range(2):
        got = _static_rhs(_desc((nx, ny), (1.0, 1.0), filt=True), U)
        assert torch.isfinite(got).all()
        assert _rel(got, ref) < 1e-6, _rel(got, ref)
    plan.close()


def test_static_rhs_rejects_oversize_grid(cuda_device):
    lib = _lib.load()
    U = torch.zeros((5, 64, 64, 32), dtype=torch.float32, device=cuda_device)  # 131072 cells
    out = torch.empty_like(U)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ps_rhs_static(C.byref(_desc((32, 64, 64), (1.0,) * 3)), C.c_void_p(U.data_ptr()),
                           C.c_void_p(out.data_ptr()), stream)
    assert rc == 2
    assert b"static scratch limit" in lib.ps_last_error()
