"""Solves launched at the same time from several host threads, each thread on
its own CUDA stream, give the same bits as the same solves run one after
another.  The threads use different grid sizes with row-streaming launch
shapes, so the same kernels are launched with different shared-memory sizes
concurrently (the serving loop's gradient workers do this)."""
import math
import threading

import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L = 2 * math.pi
NU, DT = 1e-3, 1e-3
# row-streaming bands (width, rows) per N: shared memory grows with both
SHAPES = {256: (256, 16), 512: (512, 24), 1024: (1024, 12)}
JOBS = [(N, kind) for N in SHAPES for kind in ("rollout", "graph", "grad")]


@pytest.fixture(scope="module")
def nat(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    return _native


@pytest.fixture(scope="module")
def rows_plans(nat):
    old = {}
    for N, (tw, th) in SHAPES.items():
        plan = nat.get_plan(N, L, torch.device("cuda"))
        old[N] = plan.tiles()
        plan.set_tiles(tw, th, old[N][2], old[N][3])
    yield
    for N, t in old.items():
        nat.get_plan(N, L, torch.device("cuda")).set_tiles(*t)


def _run(nat, job):
    N, kind = job
    u0 = torch.from_numpy(spectral_u0(N, 8, N)).cuda()
    th = torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda")
    if kind == "grad":
        J, g, uf, _ = nat.rollout_grad_raw(u0, th, 12, 4, L, NU, DT, "central", own_workspace=True)
        out = (J.cpu(), g.cpu(), uf.cpu())
    else:
        # graph chunks of 16 steps start from 33 steps
        steps = 36 if kind == "graph" else 12
        J, uf = nat.op_rollout(u0, th, steps, L, NU, DT, 1, 0.5, 0.1, 1.0, kind == "graph")
        out = (J.cpu(), uf.cpu())
    torch.cuda.current_stream().synchronize()
    return out


def test_concurrent_threads_match_sequential(nat, rows_plans):
    seq = {job: _run(nat, job) for job in JOBS}
    errors = []

    def worker(k):
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                for rep in range(3):
                    for i in range(len(JOBS)):
                        job = JOBS[(i + 3 * k + rep) % len(JOBS)]
                        got = _run(nat, job)
                        for a, b in zip(got, seq[job]):
                            if not torch.equal(a, b):
                                errors.append((k, rep, job, (a - b).abs().max().item()))
        except Exception as exc:
            errors.append((k, repr(exc)))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:5]


def test_concurrent_gradient_batches(nat):
    """Gradient batches advanced from two host threads at once (each on its
    own stream; their size groups fork onto the library's branch streams,
    whose pool is shared) give the bits of the same batches run alone."""
    from ns_solver_jax_differential_distributed_gb300 import ensemble

    def batch(seed):
        gb = ensemble.GradientBatch()
        ids = []
        for k, N in enumerate((64, 128, 64, 256)):
            u0 = torch.from_numpy(spectral_u0(N, 8, seed + k)).cuda()
            th = torch.tensor([0.9, 0.4, 2e-3], dtype=torch.float32, device="cuda")
            ids.append(gb.add(u0, th, 10, 3, L, NU, 0.4 / N, "upwind"))
        gb.run(7)
        torch.cuda.current_stream().synchronize()
        return [tuple(t.cpu() for t in gb.result(i)) for i in ids]

    alone = {seed: batch(seed) for seed in (0, 100)}
    errors = []

    def worker(seed):
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                for _ in range(3):
                    got = batch(seed)
                    for a, b in zip(got, alone[seed]):
                        if not (torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])):
                            errors.append((seed, a, b))
        except Exception as exc:
            errors.append((seed, repr(exc)))

    threads = [threading.Thread(target=worker, args=(s,)) for s in (0, 100)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:3]
