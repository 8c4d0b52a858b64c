"""Workload-size parity cases shared by the fixture generator
(tests/golden/make_large_parity.py) and the GPU tests
(tests/test_gpu_parity_full.py).

* Taylor-Green vortex at 128^3 and 256^3, 200 fixed steps of dt = 1e-3
  (the plain single-solve workload at its stated sizes);
* one Kelvin-Helmholtz solve per ensemble grid size (64^2 .. 512^2) run to
  t_end = 1.0 with CFL 0.4, the parameters drawn as the ensemble draws them;
* the reference's khi2d problem on its shipped 3840 x 2160 grid
  (configs/khi2d_4k.yaml: filter p = 8, alpha = 36, CFL 0.25), a few fixed
  RK4 steps at the CFL step size (mixed-radix axes 2^8 3 5 and 2^4 3^3 5).

The float64 oracle states are stored on a sub-lattice (every s-th point
along each axis) so that the fixtures stay small; the relative L2 error
over a regular sub-lattice of a smooth field estimates the full-grid error.
"""
import numpy as np

TGV_STEPS = 200
TGV_DT = 1e-3
TGV_STRIDE = {128: 4, 256: 8}

KHI_T_END = 1.0
KHI_CFL = 0.4
KHI_STRIDE = {64: 1, 128: 1, 256: 2, 512: 4}
ENSEMBLE_SEED = 20261203

KHI4K_STEPS = 3
KHI4K_STRIDE = 16


def khi4k_config():
    """The grid, physics, integration and initial-condition keys of the
    reference's configs/khi2d_4k.yaml (lines 4-28, 66-75)."""
    return {
        "problem": "khi2d",
        "grid": {"Nx": 3840, "Ny": 2160, "Lx": 1.77777777777777778, "Ly": 1.0, "dealias": True,
                 "precision": "single"},
        "physics": {"gamma": 1.4},
        "integration": {"t0": 0.0, "t_end": 5.0, "cfl": 0.25, "scheme": "rk78",
                        "spectral_filter": {"enabled": True, "p": 8, "alpha": 36.0}},
        "initial_conditions": {"rho_outer": 1.0, "rho_inner": 2.0, "u0": 1.0, "shear_thickness": 0.02,
                               "pressure_outer": 1.0, "pressure_inner": 1.0, "perturb_eps": 0.01,
                               "perturb_sigma": 0.02, "perturb_kx": 2},
    }


def khi4k_initial_state(cfg):
    """KHI2DProblem's initial state on the Fourier grid nodes (Grid2D:
    linspace(0, L, N, endpoint=False))."""
    from phrike_gb300 import problem_ics as IC
    g = cfg["grid"]
    nx, ny, lx, ly = int(g["Nx"]), int(g["Ny"]), float(g["Lx"]), float(g["Ly"])
    x = np.linspace(0.0, lx, nx, endpoint=False)
    y = np.linspace(0.0, ly, ny, endpoint=False)
    return IC.build("khi2d", cfg, float(cfg["physics"]["gamma"]), x, y, lengths=(lx, ly))


def khi_ensemble_draws(nsolve: int = 512, seed: int = ENSEMBLE_SEED):
    """(n, U0, A) for each solve of the KHI ensemble, in the ensemble's draw
    order: n uniform on {64, 128, 256, 512}, U0 ~ U[0.5, 1.5],
    A ~ U[0.005, 0.02]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nsolve):
        n = int(rng.choice([64, 128, 256, 512]))
        u0 = float(rng.uniform(0.5, 1.5))
        amp = float(rng.uniform(0.005, 0.02))
        out.append((n, u0, amp))
    return out


def khi_samples():
    """The first ensemble solve of every grid size: {n: (index, U0, A)}."""
    found = {}
    for i, (n, u0, amp) in enumerate(khi_ensemble_draws()):
        if n not in found:
            found[n] = (i, u0, amp)
    return dict(sorted(found.items()))


def sub(U: np.ndarray, stride: int) -> np.ndarray:
    """Every stride-th point along each spatial axis (leading component axis kept)."""
    sl = (slice(None),) + (slice(None, None, stride),) * (U.ndim - 1)
    return np.ascontiguousarray(U[sl])


def field_errors(out: np.ndarray, ref: np.ndarray):
    """Relative L2 error per conserved field, two ways:
    ``vector``: momentum components against the momentum-vector norm;
    ``component``: every field against its own norm."""
    nc = len(ref)
    norms = [float(np.linalg.norm(r)) for r in ref]
    mv = float(np.sqrt(sum(norms[c] ** 2 for c in range(1, nc - 1))))
    comp = [float(np.linalg.norm(o - r)) / n for o, r, n in zip(out, ref, norms)]
    vec = [float(np.linalg.norm(o - r)) / (mv if 0 < c < nc - 1 else n)
           for c, (o, r, n) in enumerate(zip(out, ref, norms))]
    return {"vector": vec, "component": comp}
