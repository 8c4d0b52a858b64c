"""Initial states of the reference's registered problems, built from the
reference's own shipped configs (grids shrunk), against the reference's
create_initial_conditions on the same node coordinates
(tests/golden/problem_ics.npz, written by make_golden.py problems)."""
import json

import numpy as np
import pytest

from conftest import golden
from phrike_gb300 import problem_ics
from phrike_gb300.config import load_yaml

Z = golden("problem_ics.npz")
CASES = list(range(int(Z["ncases"])))


@pytest.mark.parametrize("i", CASES, ids=[f"{str(Z[f'c{i}_name'])}-{str(Z[f'c{i}_file'])}" for i in CASES])
def test_initial_state_matches_reference(i):
    name = str(Z[f"c{i}_name"])
    cfg = json.loads(str(Z[f"c{i}_config"]))
    coords = {ax: Z[f"c{i}_{ax}"] for ax in ("x", "y", "z") if f"c{i}_{ax}" in Z.files}
    U = problem_ics.build(name, cfg, float(Z[f"c{i}_gamma"]), coords["x"], coords.get("y"), coords.get("z"),
                          lengths=list(Z[f"c{i}_L"]), legendre=bool(int(Z[f"c{i}_legendre"])))
    ref = Z[f"c{i}_U0"]
    assert U.shape == ref.shape
    np.testing.assert_allclose(U, ref, rtol=0, atol=1e-13 * float(np.abs(ref).max()))


def test_every_registered_problem_has_a_builder_and_a_case():
    names = {str(Z[f"c{i}_name"]) for i in CASES}
    assert names == set(problem_ics.PROBLEMS)


def test_yaml_subset_reader():
    text = """# comment
problem: khi2d
grid:
  Nx: 512     # trailing comment
  Lx: 1.0
  dealias: true
  precision: "double"
integration:
  rtol: 1e-6
  spectral_filter:
    enabled: false
    p: 8
  empty:
initial_conditions: {}
smoothing:
  variables: ["density", velocity, 'pressure']
"""
    d = load_yaml(text)
    assert d == {"problem": "khi2d",
                 "grid": {"Nx": 512, "Lx": 1.0, "dealias": True, "precision": "double"},
                 "integration": {"rtol": 1e-6, "spectral_filter": {"enabled": False, "p": 8}, "empty": None},
                 "initial_conditions": {},
                 "smoothing": {"variables": ["density", "velocity", "pressure"]}}
    with pytest.raises(ValueError):
        load_yaml("a:\n  - 1\n  - 2\n")
