"""The reference's research studies (studies.py) run through this package
and compared with the results the reference shipped: the viscosity sweep and
the scheme comparison (objective, kinetic energy, maximum speed, dt; zero
initial state, N=128, L=1) and the gradient benchmark's finite-difference
error sweep, plus the .npz layouts of their save_results."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def studies(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import studies as S
    return S


def test_viscosity_study(studies, golden, tmp_path):
    st = studies.ViscosityStudy()
    res = st.run_sweep()
    rows = {r["nu"]: r for r in golden["studies"]["viscosity"]}
    for nu, r in res.items():
        g = rows[round(nu, 6)]
        assert abs(r["dt"] - g["dt_saved"]) <= 1e-9 * g["dt_saved"]
        assert abs(r["objective"] / g["objective"] - 1) < 2e-5, (nu, r["objective"], g["objective"])
        assert abs(r["kinetic_energy"] / g["kinetic_energy"] - 1) < 2e-5
        assert r["vorticity"].shape == (128, 128)
    path = os.path.join(tmp_path, "visc.npz")
    st.save_results(path)
    d = np.load(path)
    assert set(d.files) == {f"nu_{nu:.4f}_{k}" for nu in res for k in ("objective", "kinetic_energy", "dt")}
    assert abs(float(d["nu_0.0100_objective"]) / rows[0.01]["objective"] - 1) < 2e-5


def test_scheme_comparison_study(studies, golden, tmp_path):
    st = studies.SchemeComparisonStudy()
    res = st.run_comparison(np.array([1.0, 0.5], np.float32))
    rows = {(r["scheme"], r["nu"]): r for r in golden["studies"]["scheme"]}
    for scheme, sr in res.items():
        for nu, r in sr.items():
            g = rows[(scheme, round(nu, 6))]
            assert abs(r["objective"] / g["objective"] - 1) < 2e-5, (scheme, nu, r["objective"], g["objective"])
            assert abs(r["kinetic_energy"] / g["kinetic_energy"] - 1) < 2e-5
            assert abs(r["max_velocity"] / g["max_velocity"] - 1) < 2e-5
            h = r["convergence_history"]
            assert len(h) == g["steps"] and h[0]["objective"] == 0.0
    path = os.path.join(tmp_path, "scheme.npz")
    st.save_results(path)
    assert len(np.load(path).files) == 2 * 3 * 4


def test_gradient_benchmark(studies, golden, tmp_path):
    """Where the finite-difference error is truncation (step >= 1e-2) it is a
    property of the objective, so its sweep reproduces the reference's; below
    that it is float32 noise and only its size is comparable."""
    import math
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    g = golden["studies"]["gradient_benchmark"]
    solver = nsgb.SingleCoreNSSolver(nsgb.make_grid(g["N"], g["L"]), nsgb.Phys(nu=g["nu"], mu0=0.5, sigma0=0.1,
                                                                              C=1.0),
                                     nsgb.Time(dt=g["dt"], steps=g["steps"]), g["scheme"])
    pv = [np.array(v, np.float32) for v in g["param_vectors"]]
    bm = studies.GradientBenchmark(solver.jit_objective, solver.jit_gradient, param_vectors=pv, jax_timing_runs=3)
    res = bm.run_all()
    for i, r in res.items():
        eps = sorted(r["epsilon_sweep"])
        rel = np.array([r["epsilon_sweep"][e]["rel_error"] for e in eps])
        ref = np.array(g["rel_errors"][i])
        assert np.allclose(eps, g["epsilons"], rtol=1e-6)
        big = np.array(eps) >= 1e-2
        print(i, "large-step rel errors", rel[big], "reference", ref[big], "best", rel.min(), ref.min(),
              "grad s", r["time_jax_exec_mean"])
        assert np.allclose(rel[big], ref[big], rtol=5e-2)
        assert rel.min() < 10 * ref.min() + 1e-4
    path = os.path.join(tmp_path, "grad.npz")
    bm.save_results(path)
    assert len(np.load(path).files) == 3 * 8
