"""Snapshot files and the serving loop's pause records on the host (no GPU):
the reference's .npz layout (phrike/io.py:32-236) written from a host state
and read back."""
import os
from types import SimpleNamespace

import numpy as np

from phrike_gb300 import io


def _state2d(rng, ny=8, nx=16):
    rho = 1.0 + 0.1 * rng.random((ny, nx))
    mx, my = 0.3 * rng.standard_normal((2, ny, nx))
    E = 2.5 + 0.5 * (mx * mx + my * my) / rho
    return np.stack([rho, mx, my, E])


def test_snapshot_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    U = _state2d(rng)
    grid = SimpleNamespace(x=np.linspace(0, 1, 16, endpoint=False), y=np.linspace(0, 0.5, 8, endpoint=False),
                           Nx=16, Ny=8, Lx=1.0, Ly=0.5)
    path = io.save_solution_snapshot(str(tmp_path), 0.125, U, grid, SimpleNamespace(gamma=1.4), tag="a")
    assert os.path.basename(path) == "snapshot_t0.125000_a.npz"
    with np.load(path, allow_pickle=True) as z:
        assert {"t", "U", "meta", "created", "x", "y", "rho", "ux", "uy", "p"} <= set(z.files)
        assert z["meta"].item() == {"Nx": 16, "Ny": 8, "Lx": 1.0, "Ly": 0.5, "gamma": 1.4}
    ck = io.load_checkpoint(path)
    assert ck["t"] == 0.125
    np.testing.assert_array_equal(ck["U"], U)
    np.testing.assert_array_equal(ck["y"], grid.y)
    pv = ck["primitive_vars"]
    np.testing.assert_allclose(pv["ux"], U[1] / U[0])
    np.testing.assert_allclose(pv["p"], 0.4 * (U[3] - 0.5 * (U[1] ** 2 + U[2] ** 2) / U[0]))


def test_mhd_and_1d_snapshots(tmp_path):
    rng = np.random.default_rng(2)
    n = 12
    U = np.concatenate([_state2d(rng, 1, n)[:1], 0.1 * rng.standard_normal((3, 1, n)),
                        3.0 + np.zeros((1, 1, n)), 0.2 * rng.standard_normal((3, 1, n))])[:, 0, :]
    U = np.repeat(U[:, None, :], 4, axis=1)  # (8, 4, 12)
    grid = SimpleNamespace(x=np.arange(n) / n, y=np.arange(4) / 4, Nx=n, Ny=4, Lx=1.0, Ly=1.0)
    path = io.save_solution_snapshot(str(tmp_path), 1.0, U, grid, SimpleNamespace(gamma=5.0 / 3.0))
    with np.load(path, allow_pickle=True) as z:
        assert z["meta"].item()["mhd"] is True
        assert {"Bx", "By", "Bz", "uz"} <= set(z.files)
        b2 = U[5] ** 2 + U[6] ** 2 + U[7] ** 2
        v2 = (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0] ** 2
        np.testing.assert_allclose(z["p"], (2.0 / 3.0) * (U[4] - 0.5 * U[0] * v2 - 0.5 * b2))
    U1 = _state2d(rng, 1, 32)[[0, 1, 3], 0, :]
    g1 = SimpleNamespace(x=np.arange(32) / 32, N=32, Lx=1.0)
    p1 = io.save_solution_snapshot(str(tmp_path), 0.5, U1, g1, SimpleNamespace(gamma=1.4))
    ck = io.load_checkpoint(p1)
    assert ck["meta"] == {"N": 32, "Lx": 1.0, "gamma": 1.4}
    assert set(ck["primitive_vars"]) == {"rho", "u", "p"}


def test_pause_record_round_trip(tmp_path):
    U = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    s = io.Snapshot("khi2d", 128, 0.25, 1.0, U, {"U0": 1.1, "A": 0.01})
    r = io.Snapshot.load(s.save(str(tmp_path / "pause.npz")))
    assert (r.family, r.n, r.t, r.t_end, r.params) == ("khi2d", 128, 0.25, 1.0, {"U0": 1.1, "A": 0.01})
    np.testing.assert_array_equal(r.U, U)
