"""Host logic of the serving loop that needs no GPU: the seeded request
stream, the families' grids and initial states, and the scratch bytes that
HBM admission charges per group (through ps_batch_scratch_bytes, which
allocates nothing)."""
import numpy as np
import pytest

from phrike_gb300 import serving


def test_request_stream_is_seeded_and_well_formed():
    a = serving.request_stream(200, rate=200.0, seed=7)
    b = serving.request_stream(200, rate=200.0, seed=7)
    c = serving.request_stream(200, rate=200.0, seed=8)
    key = lambda rs: [(r.family, r.n, r.t_end, r.arrival, tuple(sorted(r.params.items()))) for r in rs]
    assert key(a) == key(b)
    assert key(a) != key(c)
    arrivals = np.array([r.arrival for r in a])
    assert np.all(np.diff(arrivals) > 0)
    # mean gap of a Poisson stream at 200/s, within a loose band for 200 draws
    assert 0.5 / 200 < float(np.mean(np.diff(arrivals))) < 2.0 / 200
    sizes = {"sod1d": {256, 512, 1024, 2048, 4096}, "khi2d": {128, 256, 512, 1024}, "ot2d": {128, 256, 512},
             "tgv3d": {32, 64, 128}, "lgl2d": {65, 129, 257, 513}, "lgl1d": {65, 129, 257, 513}}
    assert {r.family for r in a} == set(sizes)
    for r in a:
        assert r.n in sizes[r.family]
        assert 0.1 <= r.t_end <= 1.0
        assert r.shape == (r.n,) * serving.FAMILIES[r.family]["ndim"]
        if r.family == "khi2d":
            assert 0.5 <= r.params["U0"] <= 1.5 and 0.005 <= r.params["A"] <= 0.02


@pytest.mark.parametrize("family,n", [("sod1d", 256), ("khi2d", 128), ("ot2d", 64), ("tgv3d", 16)])
def test_fourier_family_initial_states(family, n):
    r = serving.Request(0, family, n, 0.5, params={"U0": 1.2, "A": 0.01} if family == "khi2d" else {})
    U = r.initial_state()
    ncomp = {"sod1d": 3, "khi2d": 4, "ot2d": 8, "tgv3d": 5}[family]
    assert U.shape == (ncomp,) + r.shape
    assert np.isfinite(U).all() and (U[0] > 0).all()
    assert r.initial_state() is U  # built once
    assert len(serving.family_lengths(family, n)) == len(r.shape)


def test_group_bytes_grow_with_slots_and_include_the_split_buffer(built_lib):
    """Per slot a 512^2 group is charged its state-sized scratch (plus 32
    bytes of per-solve scalars); the tables are charged once."""
    cells = 512 * 512
    one = serving.make_plan_bytes("khi2d", 512, 1)
    four = serving.make_plan_bytes("khi2d", 512, 4)
    # 2D Euler from 256 rows: G (8) + acc (4) + Us (4) + the right-hand side (4)
    assert (four - one) == 3 * ((8 + 4 + 4 + 4) * cells * 4 + 32)
    one = serving.make_plan_bytes("ot2d", 512, 1)
    two = serving.make_plan_bytes("ot2d", 512, 2)
    # 2D MHD: G (16) + acc (8) + Us (8) + half spectra (3) + the right-hand side (8)
    assert (two - one) == (16 + 8 + 8 + 3 + 8) * cells * 4 + 32
