"""run_simulation on the reference's own problems and shipped configs (grids
shrunk, end times cut to a few CFL steps), against the float64 oracle run
from the reference's initial state (tests/golden/problem_ics.npz).

Covered: sod (1D, sensor artificial viscosity, scheme rk45 without an
adaptive block, so fixed RK4 as in the reference), acoustic1d, alfven1d,
khi2d (scheme rk78 likewise), orszag_tang2d, tgv3d (its artificial
viscosity block ignored in 3D, as the reference's 3D solver does) and
turb3d.  Tolerance: relative L2 per conserved field 1e-5 (momentum against
the momentum-vector norm; fields that vanish against the state's largest
field)."""
import json

import numpy as np
import pytest

from conftest import golden
from oracle import mhd as M
from oracle import spectral as O
from phrike_gb300 import run_simulation

pytestmark = pytest.mark.gpu

Z = golden("problem_ics.npz")


def _case(name, fname):
    for i in range(int(Z["ncases"])):
        if str(Z[f"c{i}_name"]) == name and str(Z[f"c{i}_file"]) == fname:
            return json.loads(str(Z[f"c{i}_config"])), Z[f"c{i}_U0"]
    raise KeyError((name, fname))


def _errors(out, ref, mhd=False):
    groups = ([slice(0, 1), slice(1, 4), slice(4, 5), slice(5, 8)] if mhd else
              [slice(0, 1), slice(1, len(ref) - 1), slice(len(ref) - 1, len(ref))])
    big = max(np.linalg.norm(ref[g]) for g in groups)
    errs = []
    for g in groups:
        n = np.linalg.norm(ref[g])
        errs.append(float(np.linalg.norm(out[g] - ref[g]) / (n if n > 1e-6 * big else big)))
    return errs


def _fourier_box(cfg, shape, lengths):
    sf = cfg["integration"].get("spectral_filter", {}) or {}
    return O.FourierBox(shape, lengths, dealias=bool(cfg["grid"].get("dealias", True)),
                        filter_enabled=bool(sf.get("enabled", False)), filter_p=int(sf.get("p", 8)),
                        filter_alpha=float(sf.get("alpha", 36.0)))


def _run(name, cfg):
    solver, _ = run_simulation(name, config=cfg, backend="gb300")
    return solver.U.double().cpu().numpy(), solver.t


@pytest.mark.parametrize("name,fname,t_end", [
    ("sod", "sod.yaml", 2e-3),
    ("acoustic1d", "acoustic1d.yaml", 0.02),
    ("khi2d", "khi2d.yaml", 0.01),
    ("tgv3d", "tgv3d.yaml", 0.05),
    ("turb3d", "turb3d.yaml", 0.01),
])
def test_reference_euler_problem_runs_like_the_oracle(cuda_device, name, fname, t_end):
    cfg, U0 = _case(name, fname)
    cfg["integration"].update(t_end=t_end, output_interval=t_end, checkpoint_interval=0.0)
    cfg.pop("tracers", None)
    out, t = _run(name, cfg)
    g = cfg["grid"]
    gamma = float(cfg["physics"]["gamma"])
    av = cfg.get("artificial_viscosity") if (cfg.get("artificial_viscosity") or {}).get("enabled") else None
    if U0.ndim == 2:
        box = _fourier_box(cfg, (int(g["N"]),), (float(g["Lx"]),))
    elif U0.ndim == 3:
        box = _fourier_box(cfg, (int(g["Ny"]), int(g["Nx"])), (float(g["Ly"]), float(g["Lx"])))
    else:
        box = _fourier_box(cfg, (int(g["Nz"]), int(g["Ny"]), int(g["Nx"])),
                           (float(g["Lz"]), float(g["Ly"]), float(g["Lx"])))
        av = None  # the 3D solver passes no artificial viscosity (solver.py:1266, 1330-1337)
    interval = 5 if (av is not None and U0.ndim == 2) else 1  # 1D cadence with AV (solver.py:220-232)
    s = O.EulerSolver(box, gamma=gamma, cfl=float(cfg["integration"]["cfl"]), av=av, filter_interval=interval)
    ref, tr, dts = s.run(U0.astype(np.float32).astype(np.float64), 0.0, t_end)
    assert abs(t - tr) < 1e-12
    e = _errors(out, ref)
    print(f"\n{name} ({fname}), {len(dts)} steps: rel-L2 {e}")
    assert max(e) < 1e-5, e


@pytest.mark.parametrize("name,fname,t_end", [
    ("orszag_tang2d", "orszag_tang2d.yaml", 0.01),
    ("alfven1d", "alfven1d.yaml", 0.02),
])
def test_reference_mhd_problem_runs_like_the_oracle(cuda_device, name, fname, t_end):
    cfg, U0 = _case(name, fname)
    cfg["integration"].update(t_end=t_end, output_interval=t_end, checkpoint_interval=0.0)
    out, t = _run(name, cfg)
    g = cfg["grid"]
    gamma = float(cfg["physics"]["gamma"])
    sf = cfg["integration"].get("spectral_filter", {}) or {}
    mc = (cfg["physics"].get("mhd", {}) or {})
    kw = dict(gamma=gamma, filter_params=sf, cfl=float(cfg["integration"]["cfl"]),
              project_each_substage=bool(mc.get("project_each_substage", True)),
              divergence_clean=str(mc.get("divergence_clean", "projection")),
              resistivity=float(mc.get("resistivity", 0.0)), viscosity=float(mc.get("viscosity", 0.0)))
    if U0.ndim == 2:
        s = M.MHDSolver1D(int(g["N"]), lx=float(g["Lx"]), **kw)
    else:
        s = M.MHDSolver2D(int(g["Nx"]), int(g["Ny"]), lx=float(g["Lx"]), ly=float(g["Ly"]), **kw)
    R, tr, n = U0.astype(np.float32).astype(np.float64), 0.0, 0
    while tr < t_end - 1e-12:
        dt = min(s.compute_dt(R), t_end - tr)
        R = s.step(R, dt)
        tr += dt
        n += 1
    assert abs(t - tr) < 1e-12
    e = _errors(out, R, mhd=True)
    print(f"\n{name} ({fname}), {n} steps: rel-L2 {e}")
    assert max(e) < 1e-5, e


def test_lgl_problem_with_artificial_viscosity_is_refused(cuda_device):
    """Artificial viscosity on Legendre grids is not built: the shipped
    uniform_2d config, which enables it, raises instead of running without it."""
    cfg, _ = _case("uniform_2d", "uniform_2d_small.yaml")
    with pytest.raises(Exception, match="(?i)viscosity"):
        run_simulation("uniform_2d", config=cfg, backend="gb300")
