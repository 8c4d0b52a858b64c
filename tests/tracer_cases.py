"""Tracer cases shared by the fixture generator, the oracle and GPU tests:
smooth seeded states on small periodic grids (dealias on with the filter,
and dealias off so the unpaired Nyquist mode takes part), seeded tracer
positions, a fixed state advected through STEPS leap-frog steps of DT, and a
field evaluated at the same points."""
import numpy as np

GAMMA = 1.4
DT, STEPS = 2e-3, 8

# name: (shape in array order (.., Ny, Nx), lengths in array order, dealias, filter, tracers)
CASES = {
    "d1": ((64,), (1.0,), True, {"enabled": True, "p": 8, "alpha": 36.0}, 50),
    "d1_nyq": ((32,), (2.0,), False, None, 20),
    "d2": ((16, 32), (0.5, 1.0), True, {"enabled": True, "p": 8, "alpha": 36.0}, 40),
    "d2_nyq": ((8, 16), (1.0, 1.5), False, None, 25),
    "d3": ((16, 8, 32), (1.5, 1.0, 2.0), True, {"enabled": True, "p": 8, "alpha": 36.0}, 30),
    "d3_nyq": ((8, 8, 16), (1.0, 1.0, 1.0), False, None, 17),
}


def coords(shape, lengths):
    """Node coordinates per array axis (endpoint excluded)."""
    return [np.linspace(0.0, L, n, endpoint=False) for n, L in zip(shape, lengths)]


def state(name: str) -> np.ndarray:
    """Conservative Euler state with a smooth velocity that has content
    above the 2/3 cut-off (so the mask matters)."""
    shape, lengths, _, _, _ = CASES[name]
    rng = np.random.default_rng(sum(map(ord, name)))
    mesh = np.meshgrid(*coords(shape, lengths), indexing="ij")
    nd = len(shape)
    rho = np.ones(shape)
    vel = []
    for a in range(nd):
        ph = rng.uniform(0, 2 * np.pi, size=3)
        u = np.zeros(shape)
        for k, amp in ((1, 0.3), (2, 0.1), (max(2, shape[a] // 2 - 1), 0.02)):
            for b in range(nd):
                u = u + amp / nd * np.sin(2 * np.pi * k * mesh[b] / lengths[b] + ph[b % 3] + a)
        vel.append(u)
    for b in range(nd):
        rho = rho + 0.1 * np.cos(2 * np.pi * mesh[b] / lengths[b] + 0.3 * b)
    p = np.ones(shape)
    E = p / (GAMMA - 1.0) + 0.5 * rho * sum(v * v for v in vel)
    return np.stack([rho] + [rho * v for v in vel] + [E])


def field(name: str) -> np.ndarray:
    """A scalar field with every mode present (random, seeded)."""
    shape = CASES[name][0]
    return np.random.default_rng(1000 + sum(map(ord, name))).standard_normal(shape)


def tracer_positions(name: str):
    """Seeded positions per spatial axis, x first (tracers take x0, y0, z0)."""
    shape, lengths, _, _, num = CASES[name]
    rng = np.random.default_rng(7 + len(name))
    xyz_lengths = list(reversed(lengths))
    return [rng.uniform(0.0, L, size=num) for L in xyz_lengths]
