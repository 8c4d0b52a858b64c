"""3D MHD cases shared by the fixture generator, the oracle and GPU tests:
the circularly polarized Alfven wave (filter on, ideal, RK4) and a seeded
perturbed state with a divergent B on an anisotropic box (filter off,
resistive and viscous, RK2)."""
import numpy as np

GAMMA = 5.0 / 3.0
FILTER = {"enabled": True, "p": 8, "alpha": 36.0}
# name: (Nx, Ny, Nz, Lx, Ly, Lz, filter, mhd_config, scheme, dt, nsteps)
CASES = {
    "alfven": (32, 8, 8, 1.0, 1.0, 1.0, FILTER, {}, "rk4", 2e-3, 3),
    "turb": (16, 8, 32, 1.0, 0.5, 2.0, None, {"resistivity": 0.01, "viscosity": 0.02}, "rk2", 1e-3, 3),
}


def initial_state(name: str) -> np.ndarray:
    from phrike_gb300 import problems
    nx, ny, nz, lx, ly, lz = CASES[name][:6]
    if name == "alfven":
        return problems.alfven_cp_3d(nx, ny, nz, lx)
    rng = np.random.default_rng(31)
    z, y, x = np.meshgrid(*[np.linspace(0.0, L, n, endpoint=False) for n, L in ((nz, lz), (ny, ly), (nx, lx))],
                          indexing="ij")
    kx, ky, kz = 2 * np.pi / lx, 2 * np.pi / ly, 2 * np.pi / lz
    rho = 1.0 + 0.1 * np.sin(kx * x + 0.3) * np.cos(kz * z)
    ux = 0.2 * np.sin(ky * y + kz * z)
    uy = 0.15 * np.cos(kx * x - 2 * kz * z)
    uz = 0.1 * np.sin(kx * x + ky * y)
    p = 0.6 + 0.05 * np.cos(kx * x + ky * y + kz * z)
    Bx = 0.5 + 0.1 * np.sin(ky * y) + 0.05 * np.cos(kx * x)          # divergent part along x
    By = 0.2 * np.cos(kz * z + kx * x) + 0.03 * rng.standard_normal(x.shape) * 0.1
    Bz = 0.1 * np.sin(kx * x) + 0.04 * np.sin(kz * z)
    E = p / (GAMMA - 1.0) + 0.5 * rho * (ux * ux + uy * uy + uz * uz) + 0.5 * (Bx * Bx + By * By + Bz * Bz)
    return np.stack([rho, rho * ux, rho * uy, rho * uz, E, Bx, By, Bz])
