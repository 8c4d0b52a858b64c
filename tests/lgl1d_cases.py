"""1D Legendre cases shared by the oracle and GPU tests; they are the cases
tests/golden/make_golden.py ran through the reference (tests/golden/lgl1d.npz):
n LGL nodes on [0, 2], a Gaussian density/pressure pulse with a velocity bump,
five steps of dt = 2e-4."""
import numpy as np

CASES = {
    "wall": dict(n=33, filter_params={"enabled": True, "p": 8, "alpha": 36.0, "interval": 2}, bc=None,
                 scheme="rk4", gravity=None),
    "mixed": dict(n=41, filter_params=None,
                  bc={"left": {"density": "neumann", "momentum": "wall", "pressure": "open"}, "right": "neumann"},
                  scheme="rk2", gravity=-1.5),
}
LENGTH, DT, NSTEPS = 2.0, 2e-4, 5


def initial_state(x: np.ndarray) -> np.ndarray:
    rho = 1.0 + 0.2 * np.exp(-((x - 0.8) ** 2) / 0.02)
    p = rho ** 1.4 / 1.4
    u = 0.1 * np.sin(np.pi * x / 2.0) ** 2
    return np.stack([rho, rho * u, p / 0.4 + 0.5 * rho * u * u])
