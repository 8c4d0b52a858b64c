"""Host-side behaviour of the reference-shaped API (no GPU needed)."""
import json

import pytest

import phrike_gb300
from phrike_gb300 import _load_config


def test_backend_and_problem_validation():
    with pytest.raises(ValueError, match="backend"):
        phrike_gb300.run_simulation("sod", config={}, backend="numpy")
    with pytest.raises(ValueError, match="unknown problem"):
        phrike_gb300.run_simulation("nope", config={}, backend="gb300")


def test_config_loading_json(tmp_path):
    cfg = {"grid": {"N": 64}, "integration": {"t_end": 0.1}}
    p = tmp_path / "c.json"
    p.write_text(json.dumps(cfg))
    assert _load_config(str(p), None) == cfg
    assert _load_config(None, {"a": 1}) == {"a": 1}


def test_lazy_exports():
    from phrike_gb300 import grid
    assert phrike_gb300.Grid3D is grid.Grid3D
    with pytest.raises(ValueError, match="backend 'gb300'"):
        grid._check_backend("torch")
