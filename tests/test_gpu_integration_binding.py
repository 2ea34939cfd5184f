"""The reference-side ctypes binding printed in INTEGRATION.md runs as
written: its rollout matches the oracle and the package's own rollout (to
rounding: it creates a plan with the default launch shapes, the package's
plans may carry tuned ones)."""
import math
import os
import re

import numpy as np
import pytest
import torch

from oracle import ns_oracle as O
from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _binding_source() -> str:
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        blocks = re.findall(r"```python\n(.*?)```", f.read(), re.S)
    return next(b for b in blocks if "ctypes.CDLL" in b)


def test_documented_binding_runs_and_matches(cuda_lib, monkeypatch):
    import ns_solver_jax_differential_distributed_gb300 as nsgb
    monkeypatch.chdir(ROOT)  # the binding loads the library by its in-tree path
    ns = {}
    exec(compile(_binding_source(), "INTEGRATION.md", "exec"), ns)
    N, L, nu, dt, steps = 64, 2 * math.pi, 1e-3, 1e-3, 40
    u0 = spectral_u0(N, 8, 3)
    th = np.array([1.0, 0.5], np.float32)
    J, uf = ns["rollout"](torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda(), L, nu, dt, steps)
    torch.cuda.synchronize()
    J32, u32 = O.rollout(u0, th, O.OracleConfig(N=N, L=L, nu=nu, dt=dt, steps=steps))
    assert O.rel_l2(u32, uf.cpu().numpy()) < 1e-5
    assert abs(float(J) - float(J32)) <= 1e-5 * abs(float(J32))
    s = nsgb.SingleCoreNSSolver(nsgb.make_grid(N, L), nsgb.Phys(nu=nu, mu0=0.5, sigma0=0.1, C=1.0),
                                nsgb.Time(dt=dt, steps=steps), "central")
    Jp, ufp = s.rollout(torch.from_numpy(u0).cuda(), torch.from_numpy(th).cuda())
    assert O.rel_l2(ufp.cpu().numpy(), uf.cpu().numpy()) < 1e-6
    assert abs(float(J) - float(Jp)) <= 1e-6 * abs(float(Jp))
