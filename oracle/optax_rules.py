"""Update rules of the optimisers the reference's optimisation study uses
(TEST INFRASTRUCTURE: only tests import this module).

The reference drives `SingleCoreNSSolver.jit_gradient` with optax 0.2.4
(requirements.txt:16) in `ParameterOptimizationStudy` (studies.py:864-934):
`optax.adam(lr)`, `optax.sgd(lr)`, `optax.rmsprop(lr)` with their default
hyper-parameters, applied by `optax.apply_updates` (studies.py:896-900).
optax is not installed here; this module restates the published update rules
of that version in float32 NumPy, in the order the library evaluates them:

* sgd:     u = g * (-lr)
* adam:    m = (1-b1) g + b1 m;  v = (1-b2) g^2 + b2 v;  t = t + 1;
           m_hat = m / (1 - b1^t);  v_hat = v / (1 - b2^t);
           u = (m_hat / (sqrt(v_hat + eps_root) + eps)) * (-lr)
           (b1 = 0.9, b2 = 0.999, eps = 1e-8, eps_root = 0)
* rmsprop: v = (1-decay) g^2 + decay v;  u = (g * rsqrt(v + eps)) * (-lr)
           (decay = 0.9, eps = 1e-8 inside the square root, initial v = 0)
* apply:   theta = theta + u

The rules are pinned by the reference's shipped trajectories
(result/optimization_study_results.npz, extracted to tests/golden/): the
first step of each optimiser from the JAX gradient the SGD trajectory encodes.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

F32 = np.float32


@dataclass
class OptState:
    mu: np.ndarray
    nu: np.ndarray
    count: int = 0


@dataclass(frozen=True)
class Rule:
    kind: str          # "sgd" | "adam" | "rmsprop"
    lr: float
    b1: float = 0.9
    b2: float = 0.999
    eps: float = 1e-8
    eps_root: float = 0.0
    decay: float = 0.9


def init(theta: np.ndarray) -> OptState:
    z = np.zeros_like(np.asarray(theta, F32))
    return OptState(z.copy(), z.copy(), 0)


def update(rule: Rule, g: np.ndarray, st: OptState) -> tuple[np.ndarray, OptState]:
    """(updates, new state) for gradient g, float32 throughout."""
    g = np.asarray(g, F32)
    lr = F32(rule.lr)
    if rule.kind == "sgd":
        return g * (-lr), st
    if rule.kind == "adam":
        mu = F32(1.0 - rule.b1) * g + F32(rule.b1) * st.mu
        nu = F32(1.0 - rule.b2) * (g * g) + F32(rule.b2) * st.nu
        t = st.count + 1
        mu_hat = mu / F32(1.0 - rule.b1 ** t)
        nu_hat = nu / F32(1.0 - rule.b2 ** t)
        u = (mu_hat / (np.sqrt(nu_hat + F32(rule.eps_root)) + F32(rule.eps))) * (-lr)
        return u.astype(F32), OptState(mu, nu, t)
    if rule.kind == "rmsprop":
        nu = F32(1.0 - rule.decay) * (g * g) + F32(rule.decay) * st.nu
        u = (g * (F32(1.0) / np.sqrt(nu + F32(rule.eps)))) * (-lr)
        return u.astype(F32), OptState(st.mu, nu, st.count + 1)
    raise ValueError(rule.kind)


def apply(theta: np.ndarray, u: np.ndarray) -> np.ndarray:
    return (np.asarray(theta, F32) + u).astype(F32)
