"""Tracer construction from a config block on the host (no GPU): the
reference's layouts (phrike/problems/base.py:961-1021) restated with numpy
and compared position by position."""
from types import SimpleNamespace

import numpy as np

from phrike_gb300.tracers import FourierTracers1D, FourierTracers2D, FourierTracers3D, tracers_from_config


def _grid(shape, lengths, basis="fourier"):
    g = SimpleNamespace(_shape=tuple(shape), _basis=basis, Lx=lengths[0])
    if len(lengths) > 1:
        g.Ly = lengths[1]
    if len(lengths) > 2:
        g.Lz = lengths[2]
    return g


def test_random_layout_draws_axes_in_order():
    cfg = {"enabled": True, "num": 7, "layout": "random", "seed": 3, "mass": 2.0}
    tr = tracers_from_config(_grid((8, 16, 32), (1.0, 2.0, 3.0)), cfg)
    assert isinstance(tr, FourierTracers3D) and tr.mass == 2.0
    rng = np.random.default_rng(3)
    want = [rng.uniform(0.0, L, size=7) for L in (1.0, 2.0, 3.0)]
    for got, ref in zip((tr.x, tr.y, tr.z), want):
        np.testing.assert_array_equal(np.asarray(got), ref)


def test_uniform_layouts():
    tr = tracers_from_config(_grid((16, 32), (1.0, 0.5)), {"enabled": True, "num": 10, "layout": "uniform"})
    assert isinstance(tr, FourierTracers2D)
    n = 3  # round(sqrt(10)); the lattice has 9 < 10 points and is not padded
    xx, yy = np.meshgrid(np.linspace(0, 1.0, n, endpoint=False), np.linspace(0, 0.5, n, endpoint=False),
                         indexing="ij")
    np.testing.assert_array_equal(np.asarray(tr.x), xx.ravel())
    np.testing.assert_array_equal(np.asarray(tr.y), yy.ravel())
    tr = tracers_from_config(_grid((8, 8, 8), (1.0, 1.0, 1.0)), {"enabled": True, "num": 6, "layout": "UNIFORM"})
    assert isinstance(tr, FourierTracers3D) and np.asarray(tr.x).size == 6  # 2^3 lattice cut to num
    tr = tracers_from_config(_grid((64,), (2.0,)), {"enabled": True, "num": 5, "layout": "uniform"})
    assert isinstance(tr, FourierTracers1D)
    np.testing.assert_array_equal(np.asarray(tr.x), np.linspace(0, 2.0, 5, endpoint=False))


def test_disabled_or_not_fourier():
    assert tracers_from_config(_grid((16, 16), (1.0, 1.0)), {"enabled": False, "num": 4}) is None
    assert tracers_from_config(_grid((16, 16), (1.0, 1.0)), {}) is None
    assert tracers_from_config(_grid((17, 17), (2.0, 2.0), basis="legendre"), {"enabled": True}) is None
