"""SimConfig / load_config semantics (the reference's ConfigParsingTests and
single-device BadConfigTests, unit_tests/test_distributed_solver.py:423-562)."""
import json
import os

import numpy as np
import pytest

from ns_solver_jax_differential_distributed_gb300 import SimConfig, load_config, make_advection_scheme
from ns_solver_jax_differential_distributed_gb300.solver import make_grid


@pytest.mark.parametrize("kw", [dict(N=-1), dict(N=0), dict(nu=0.0), dict(nu=-0.001),
                                dict(advection_scheme="quickscheme"), dict(advection_scheme="")])
def test_bad_config_raises(kw):
    with pytest.raises(ValueError):
        SimConfig(**kw)


def test_make_advection_scheme_unknown():
    with pytest.raises(ValueError):
        make_advection_scheme("lax-wendroff")


def _write(tmp_path, payload):
    p = tmp_path / "cfg.json"
    p.write_text(json.dumps(payload))
    return str(p)


def test_none_and_missing_path_defaults():
    assert load_config(None).N == 128
    assert load_config("/nonexistent/path/does_not_exist.json").N == 128


def test_overrides_and_defaults(tmp_path):
    cfg = load_config(_write(tmp_path, {"N": 64, "nu": 0.005, "t": 1.0, "advection_scheme": "upwind"}))
    assert (cfg.N, cfg.advection_scheme) == (64, "upwind")
    assert cfg.nu == pytest.approx(0.005) and cfg.t == pytest.approx(1.0)
    cfg = load_config(_write(tmp_path, {"N": 32}))
    assert cfg.N == 32 and cfg.nu == pytest.approx(SimConfig().nu)


def test_unknown_fields_ignored_and_bad_scheme(tmp_path):
    assert load_config(_write(tmp_path, {"N": 48, "unknown_parameter": 999})).N == 48
    with pytest.raises(ValueError):
        load_config(_write(tmp_path, {"advection_scheme": "invalid"}))


def test_theta0_loaded(tmp_path):
    cfg = load_config(_write(tmp_path, {"theta0": [0.3, 0.7]}))
    np.testing.assert_allclose(np.asarray(cfg.theta0), [0.3, 0.7], atol=1e-6)


def test_steps_dx_dt():
    cfg = SimConfig(N=32, t=0.5)
    assert cfg.steps == int(np.ceil(cfg.t / cfg.dt)) and cfg.steps > 0
    assert SimConfig(N=64, L=2.0).dx == pytest.approx(2.0 / 64)
    cfg = SimConfig(N=64, nu=0.01, cfl=0.4, v_max=1.0)
    assert cfg.dt <= cfg.cfl * cfg.dx / cfg.v_max + 1e-12
    assert cfg.dt <= cfg.dx ** 2 / (4.0 * cfg.nu) + 1e-12


def test_reference_sample_configs_dt_steps(golden):
    """dt/steps of the studies' configs equal the values the reference saved."""
    for row in golden["studies"]["viscosity"]:
        cfg = SimConfig(N=128, nu=row["nu"])
        assert cfg.dt == row["dt_saved"] and cfg.steps == row["steps"]


def test_make_grid_matches_linspace():
    g = make_grid(64, 2 * np.pi)
    x = np.linspace(0, 2 * np.pi, 64, endpoint=False, dtype=np.float32)
    np.testing.assert_allclose(g.X[:, 0].numpy(), x, rtol=0, atol=1e-6)
    assert g.dx == pytest.approx(2 * np.pi / 64)
