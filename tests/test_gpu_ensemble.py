"""Ensembles of uneven grid sizes: every member's result equals its own plain
rollout bit for bit (the batched launches and graph chunks change nothing
about a member's arithmetic), and a member matches the oracle."""
import math

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from tests.conftest import rel_l2
from ns_solver_jax_differential_distributed_gb300.workloads import ensemble as make_ensemble

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ens_mod(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import ensemble
    return ensemble


def _specs(ens_mod, count=14, sizes=(16, 32, 64, 128), probs=(0.3, 0.3, 0.3, 0.1), scheme="central"):
    members = make_ensemble(count=count, steps=1, sizes=sizes, probs=probs, seed=7, scheme=scheme)
    specs = ens_mod.from_workload(members, scheme=scheme)
    return specs


@pytest.mark.parametrize("chunk", [0, 8])
@pytest.mark.parametrize("scheme", ["central", "upwind"])
def test_ensemble_equals_sequential(ens_mod, chunk, scheme):
    specs = _specs(ens_mod, scheme=scheme)
    ens = ens_mod.Ensemble(specs, steps=37, chunk=chunk)
    J, us = ens.run()
    J = J.clone()
    us = [u.clone() for u in us]
    Js, uss = ens.run_sequential()
    assert torch.equal(J, Js)
    for a, b in zip(us, uss):
        assert torch.equal(a, b)
    # a second run of the same ensemble (cached graph) gives the same bits
    J2, us2 = ens.run()
    assert torch.equal(J2, J) and all(torch.equal(a, b) for a, b in zip(us2, us))


@pytest.mark.parametrize("slice_steps", [1, 5, 16])
def test_ensemble_advance_slices_equal_sequential(ens_mod, slice_steps):
    """Advancing in slices (continuous batching) gives the same bits."""
    specs = _specs(ens_mod, count=9)
    ens = ens_mod.Ensemble(specs, steps=23, chunk=0)
    J, us = ens.run_advance(slice_steps)
    J = J.clone()
    us = [u.clone() for u in us]
    Js, uss = ens.run_sequential()
    assert torch.equal(J, Js)
    assert all(torch.equal(a, b) for a, b in zip(us, uss))


def test_ensemble_member_matches_oracle(ens_mod):
    specs = _specs(ens_mod, count=6, sizes=(32, 64), probs=(0.5, 0.5))
    ens = ens_mod.Ensemble(specs, steps=20, chunk=4)
    J, us = ens.run()
    for k in (0, len(specs) - 1):
        s = specs[k]
        cfg = O.OracleConfig(N=s.N, L=s.L, nu=s.nu, dt=s.dt, steps=20, scheme=s.scheme)
        J32, u32 = O.rollout(s.u0, s.theta, cfg)
        assert rel_l2(u32, us[k].cpu().numpy()) < 1e-5
        assert abs(float(J[k]) - float(J32)) <= 1e-4 * abs(float(J32)) + 1e-9


def test_ensemble_single_step_and_one_member(ens_mod):
    specs = _specs(ens_mod, count=1, sizes=(64,), probs=(1.0,))
    for steps in (1, 2, 3):
        ens = ens_mod.Ensemble(specs, steps=steps, chunk=2)
        J, us = ens.run()
        Js, uss = ens.run_sequential()
        assert torch.equal(J, Js) and torch.equal(us[0], uss[0])


def test_ensemble_rejects_a_field_of_the_wrong_size(ens_mod):
    """Members reach the kernels as bare pointers, so a u0 whose shape is not
    (2, N, N) is refused before anything is allocated or launched."""
    import dataclasses
    specs = _specs(ens_mod, count=3, sizes=(32, 64), probs=(0.5, 0.5))
    bad = dataclasses.replace(specs[1], u0=np.zeros((2, specs[1].N // 2, specs[1].N // 2), np.float32))
    with pytest.raises(ValueError, match="member 1: u0 must have shape"):
        ens_mod.Ensemble([specs[0], bad, specs[2]], steps=2)
