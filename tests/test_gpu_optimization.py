"""The device optimisation loop (nsgb_optimize, ParameterOptimizationStudy)
against the reference's own optimisation study: the four 100-step optimiser
trajectories it ships (result/optimization_study_results.npz, extracted to
tests/golden/reference_results.json), run from the same configuration (N=128,
L=1, nu=0.01, dt from SimConfig, 328 steps, central, zero initial state,
theta0 = [1, 0.5]).  The gradient differs from JAX's by float32 rounding (the
FFTs and the fused step round differently), which the 100-step trajectories
carry; the tolerances bound that drift."""
import math
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def study_results(cuda_lib, golden):
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    from ns_solver_jax_differential_distributed_gb300 import optimization as opt
    g = golden["studies"]["optimizers"]
    grid = nsgb.make_grid(g["N"], L=g["L"])
    phys = nsgb.Phys(nu=g["nu"], mu0=0.5, sigma0=0.1, C=1.0)
    solver = nsgb.SingleCoreNSSolver(grid, phys, nsgb.Time(dt=g["dt"], steps=g["steps"]), g["scheme"])
    study = opt.ParameterOptimizationStudy(solver.jit_objective, solver.jit_gradient, theta0=g["theta"],
                                           optim_steps=g["optim_steps"])
    return study, study.run_all(), {r["name"]: r for r in g["runs"]}


# Bounds per optimiser: (max rel error of J, max |error| of B, of A).  SGD
# follows the reference's steps themselves, so its whole trajectory matches.
# dJ/dA is 2.6e-5 at theta0 and about 1e-6 after a few steps, the size of
# float32 gradient noise; Adam and RMSprop divide each update by a running
# gradient magnitude, so a noise-sized A gradient still moves A by about lr
# per step with a noise-dependent sign, and the A component of their
# trajectories is not reproducible by any float32 gradient (J hardly depends
# on A, so the objectives still agree).  B is compared tightly for all.  The
# reference's own RMSprop trajectory settles at B = 0.64856 by step 60 and
# then, with its second moment decayed onto noise-sized gradients, kicks out
# to 0.663 at step 77: from there the path depends on gradient noise, so
# RMSprop is held tightly over its first 70 steps and loosely after.
BOUNDS = {"Adam (lr=0.01)": (1e-5, 1e-4, 0.1), "Adam (lr=0.001)": (1e-5, 1e-5, 0.01),
          "SGD (lr=0.1)": (1e-5, 1e-6, 1e-6), "RMSprop (lr=0.01)": (2e-3, 5e-2, 0.1)}
STABLE_STEPS = {"RMSprop (lr=0.01)": 70}


@pytest.mark.parametrize("name", list(BOUNDS))
def test_trajectory_matches_reference(study_results, name):
    _, res, gold = study_results
    ours, ref = res[name], gold[name]
    J = np.asarray(ours["history"]["objectives"], np.float64)
    Jr = np.asarray(ref["objectives"], np.float64)
    P = np.asarray(ours["history"]["parameters"], np.float64)
    Pr = np.asarray(ref["parameters"], np.float64)
    dJ = np.abs(J - Jr) / np.abs(Jr)
    dA, dB = np.abs(P[:, 0] - Pr[:, 0]).max(), np.abs(P[:, 1] - Pr[:, 1]).max()
    print(f"{name}: max rel dJ {dJ.max():.2e} (first {dJ[0]:.2e}), max |dB| {dB:.2e}, max |dA| {dA:.2e}, "
          f"improvement {ours['improvement']:.6f} vs {ref['improvement']:.6f}")
    bJ, bB, bA = BOUNDS[name]
    assert dJ[0] < 2e-6           # J(theta0): the forward alone
    if name in STABLE_STEPS:
        k = STABLE_STEPS[name] + 1
        print(f"  first {k - 1} steps: max rel dJ {dJ[:k].max():.2e}, max |dB| "
              f"{np.abs(P[:k, 1] - Pr[:k, 1]).max():.2e}")
        assert dJ[:k].max() < 1e-5
        assert np.abs(P[:k, 1] - Pr[:k, 1]).max() < 1e-4
    assert dJ.max() < bJ
    assert dB < bB
    assert dA < bA
    assert abs(ours["improvement"] - ref["improvement"]) < 10 * bJ


def test_save_results_layout(study_results, tmp_path):
    study, _, gold = study_results
    path = os.path.join(tmp_path, "opt.npz")
    study.save_results(path)
    d = np.load(path)
    keys = {f"{n}_{k}" for n in gold for k in ("obj_initial", "obj_final", "improvement", "steps", "objectives",
                                               "parameters")}
    assert set(d.files) == keys
    assert d["SGD (lr=0.1)_parameters"].shape == (101, 2)
    assert d["SGD (lr=0.1)_steps"].dtype == np.int32


def test_optimize_sgd_matches_host_loop(cuda_lib):
    """Three SGD steps of nsgb_optimize equal a host loop of jit_gradient and
    the restated update rule, from a seeded state (bitwise: same kernels)."""
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    from ns_solver_jax_differential_distributed_gb300 import _native
    from oracle import optax_rules as R
    N, L, nu, dt, steps = 64, 2 * math.pi, 1e-3, 1e-3, 20
    solver = nsgb.SingleCoreNSSolver(nsgb.make_grid(N, L), nsgb.Phys(nu=nu, mu0=0.5, sigma0=0.1, C=1.0),
                                     nsgb.Time(dt=dt, steps=steps),
                                     "upwind", checkpoint_every=7)
    th0 = torch.tensor([0.9, 0.45, 2e-3], device="cuda")
    spec = _native.Optimizer(_native.OPT_SGD, 0.05, 0.9, 0.999, 1e-8, 0.0, 0.9)
    J, P = _native.optimize(th0, steps, 7, N, L, nu, dt, 1, spec, 3)
    th = th0.cpu().numpy()
    for k in range(3):
        Jk, g = solver.gradient(torch.zeros(2, N, N, device="cuda"), torch.from_numpy(th).cuda())
        assert float(Jk) == float(J[k])
        u, _ = R.update(R.Rule("sgd", 0.05), g.cpu().numpy(), R.init(th))
        th = R.apply(th, u)
        assert np.array_equal(P[k + 1].cpu().numpy(), th)


def test_overlapped_loops_equal_one_by_one(study_results):
    """run_all enqueues the four loops from four host threads onto four
    streams; each loop's objectives and parameters equal its own loop run
    alone (bitwise: each has its own workspace and the same kernels)."""
    study, res, _ = study_results
    for cfg in study.optim_configs:
        alone = study._run_single_optimizer(cfg["name"], cfg["optimizer"])
        assert np.array_equal(alone["history"]["objectives"], res[cfg["name"]]["history"]["objectives"])
        assert np.array_equal(alone["history"]["parameters"], res[cfg["name"]]["history"]["parameters"])


def test_overlapped_loops_raise_on_the_callers_thread(study_results):
    """An error while one loop is enqueued (on its own thread) is raised to
    the caller of run_all, after the other loops' threads have finished."""
    from ns_solver_jax_differential_distributed_gb300 import optimization as opt
    study = study_results[0]

    class Broken:
        def native(self):
            raise RuntimeError("broken optimiser spec")

    cfgs = [study.optim_configs[0], {"name": "broken", "optimizer": Broken()}]
    mixed = opt.ParameterOptimizationStudy(study.objective, study.grad_jax, [1.0, 0.5], optim_configs=cfgs,
                                           optim_steps=2)
    with pytest.raises(RuntimeError, match="broken optimiser spec"):
        mixed.run_all()
    torch.cuda.synchronize()
