"""The golden pins have power: a mistake planted in the oracle (on the CPU)
makes the comparison with the reference's shipped outputs fail, at the same
metric and tolerance as tests/test_oracle_golden.py.

Planted, one at a time: the sign of the pressure gradient in the projection
(NS_solver.py:696-697), the forcing's period-1 wrap (NS_solver.py:626), the
objective accumulated on the state after the step instead of before it
(NS_solver.py:742-750), and the discrete symbol sin(k dx)/dx in place of the
continuous |k| in the Poisson solve (NS_solver.py:517-527).  The zero initial
state of every shipped output leaves advection unexercised, so an advection
mistake is not detectable this way; the finite-difference and float64
autograd checks of the gradient cover it."""
import math
import os

import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.conftest import rel_l2

SPEED_TOL = 5e-7   # test_speed_field_N128
J_TOL = 1e-6       # test_scheme_study_objective_energy_speed
CAUGHT = 5         # a planted mistake must miss the golden by this factor at least


def _caught(err: float, tol: float) -> bool:
    # a non-finite result fails the golden comparison as well
    return not np.isfinite(err) or err > CAUGHT * tol


def _speed_field_error(golden) -> float:
    f = golden["speed_fields"][0]
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", f["file"]))
    cfg = O.OracleConfig(N=128, L=1.0, nu=f["nu"], dt=f["dt"], steps=f["steps"])
    _, u = O.rollout(np.zeros((2, 128, 128), np.float32), np.array(f["theta"], np.float32), cfg)
    return rel_l2(ref, np.sqrt(u[0].astype(np.float64) ** 2 + u[1].astype(np.float64) ** 2))


def _scheme_row(golden):
    return next(r for r in golden["studies"]["scheme"] if r["steps"] <= 800)


def _objective_error(golden, rollout=None) -> float:
    row = _scheme_row(golden)
    cfg = O.OracleConfig(N=row["N"], L=row["L"], nu=row["nu"], dt=row["dt"], steps=row["steps"],
                         scheme=row["scheme"])
    J, _ = (rollout or O.rollout)(np.zeros((2, row["N"], row["N"]), np.float32),
                                  np.array(row["theta"], np.float32), cfg)
    return abs(float(J) / row["objective"] - 1)


def test_unplanted_oracle_passes(golden):
    assert _speed_field_error(golden) < SPEED_TOL
    assert _objective_error(golden) < J_TOL


def test_pressure_gradient_sign_is_caught(golden, monkeypatch):
    # planted in the pressure itself: the projection then adds dt grad p
    # (flipping grad would flip the divergence too, and the two cancel)
    real = O.poisson_solve
    monkeypatch.setattr(O, "poisson_solve", lambda rhs, dx, inv_k2=None: -real(rhs, dx, inv_k2))
    with np.errstate(all="ignore"):  # the planted projection amplifies the field until it overflows
        assert _caught(_speed_field_error(golden), SPEED_TOL)


def test_missing_forcing_wrap_is_caught(golden, monkeypatch):
    def fx_unwrapped(theta, t, cfg, dtype=np.float32):
        th = np.asarray(theta, dtype=dtype)
        t, twopi = dtype(t), dtype(2.0 * math.pi)
        mu = dtype(cfg.mu0) + np.sin(twopi * th[0] * t, dtype=dtype)
        c = np.cos(twopi * th[1] * t, dtype=dtype)
        sig = dtype(cfg.sigma0) + c * c
        d = (O.grid_x(cfg.N, cfg.L, dtype) - mu).astype(dtype)  # no period-1 wrap
        return (dtype(cfg.C) * np.exp(-(d * d) / (dtype(2.0) * sig * sig))).astype(dtype)

    monkeypatch.setattr(O, "forcing_fx", fx_unwrapped)
    assert _caught(_objective_error(golden), J_TOL)


def test_objective_after_the_step_is_caught(golden):
    def rollout_late_J(u0, theta, cfg):
        dtype = u0.dtype.type
        th, nu = O._split_theta(theta, cfg, dtype)
        inv_k2 = O.poisson_inv_k2(cfg.N, cfg.dx, dtype)
        dt, dx2 = dtype(cfg.dt), dtype(cfg.dx ** 2)
        u, J = u0.copy(), dtype(0.0)
        for i in range(cfg.steps):
            f = O.full_forcing(th, dtype(dtype(i) * dt), cfg, dtype)
            u = O.projector_step(u, f, cfg, nu=nu, inv_k2=inv_k2)
            J = dtype(J + dt * np.sum(u * f, dtype=dtype) * dx2)  # planted: the state after the step
        return J, u

    assert _caught(_objective_error(golden, rollout_late_J), J_TOL)


def test_discrete_poisson_symbol_is_caught(golden, monkeypatch):
    def inv_s2(N, dx, dtype=np.float32):
        k = 2.0 * np.pi * np.fft.fftfreq(N, d=dx)
        s = np.sin(k * dx) / dx
        s2 = s[:, None] ** 2 + s[None, :] ** 2
        out = np.zeros_like(s2)
        np.divide(1.0, s2, out=out, where=s2 > 0)
        return out.astype(dtype)

    monkeypatch.setattr(O, "poisson_inv_k2", inv_s2)
    assert _caught(_speed_field_error(golden), SPEED_TOL)
