"""The persistent ensemble launch (nsgb_ensemble_persistent): one cooperative
launch advances every member of an uneven ensemble through all its steps.
Fields equal the graph-chunked ensemble and the members' solo rollouts bit
for bit (radix-16 transforms); J agrees to rounding (its partials follow the
persistent launch's 64 x 16 tiling); repeated launches give the same bits."""
import math

import numpy as np
import pytest
import torch

from ns_solver_jax_differential_distributed_gb300.workloads import spectral_u0

pytestmark = pytest.mark.gpu

L = 2 * math.pi
SIZES = [64, 128, 256, 512, 1024, 64, 128, 2048, 4096]
SCHEMES = ["central", "upwind", "upwind", "central", "upwind", "central", "central", "upwind", "upwind"]


@pytest.fixture(scope="module")
def mods(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native, ensemble
    return _native, ensemble


@pytest.fixture
def radix16(mods):
    _native, _ = mods
    plans = {N: _native.get_plan(N, L, torch.device("cuda")) for N in set(SIZES)}
    old = {N: p.fft_radix() for N, p in plans.items()}
    for p in plans.values():
        p.set_fft_radix(16, 16)
    yield
    for N, p in plans.items():
        p.set_fft_radix(*old[N])


def _specs(ensemble):
    out = []
    for k, (N, scheme) in enumerate(zip(SIZES, SCHEMES)):
        nu = 1e-3
        dx = L / N
        dt = float(np.float32(min(0.4 * dx / 4.0, dx * dx / (4 * nu))))
        th = np.array([0.9 + 0.01 * k, 0.45, nu], np.float32)
        out.append(ensemble.SolveSpec(N, spectral_u0(N, min(8, N // 4), k), th, nu, dt, scheme, L))
    return out


def test_persistent_equals_chunked_and_solo(mods, radix16):
    _native, ensemble = mods
    steps = 21
    ens = ensemble.Ensemble(_specs(ensemble), steps=steps, chunk=16)
    Jp, up = ens.run_persistent()
    Jp, up = Jp.clone(), [u.clone() for u in up]
    Jr, ur = ens.run()
    Jr, ur = Jr.clone(), [u.clone() for u in ur]
    Js, us = ens.run_sequential()
    torch.cuda.synchronize()
    for k in range(len(SIZES)):
        assert torch.isfinite(up[k]).all()
        assert torch.equal(up[k], ur[k]), (k, SIZES[k], (up[k] - ur[k]).abs().max().item())
        assert torch.equal(up[k], us[k]), k
    rel = ((Jp.double() - Jr.double()).abs() / Jr.double().abs().clamp_min(1e-12)).max().item()
    assert rel < 1e-5 or (Jp.double() - Jr.double()).abs().max().item() < 1e-9, (Jp, Jr)
    Jq, uq = ens.run_persistent()
    torch.cuda.synchronize()
    assert torch.equal(Jq, Jp) and all(torch.equal(a, b) for a, b in zip(uq, up))


def test_unsupported_size_rejected(mods):
    _native, ensemble = mods
    N = 32
    spec = ensemble.SolveSpec(N, spectral_u0(N, 4, 0), np.array([1.0, 0.5, 1e-3], np.float32), 1e-3, 1e-3,
                              "central", L)
    ens = ensemble.Ensemble([spec], steps=4, chunk=0)
    with pytest.raises(_native.NativeError):
        ens.run_persistent()


def test_table_uploading_calls_refuse_capture(mods):
    """The ensemble calls upload their member tables from host memory that
    does not outlive the call, so inside a stream capture they return
    NSGB_ERR_INVALID_ARG and enqueue nothing."""
    import ctypes
    _native, ensemble = mods
    N = 64
    spec = ensemble.SolveSpec(N, spectral_u0(N, 8, 0), np.array([1.0, 0.5, 1e-3], np.float32), 1e-3, 1e-3,
                              "central", L)
    ens = ensemble.Ensemble([spec], steps=4, chunk=0)
    lib = _native.lib()
    need = lib.nsgb_ensemble_persistent_workspace_bytes(ens._members, 1)
    pws = torch.empty(need, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            st = ctypes.c_void_p(s.cuda_stream)
            rcs = [lib.nsgb_ensemble_rollout(ens._members, 1, 0, ens.workspace.data_ptr(), ens.workspace.numel(), st),
                   lib.nsgb_ensemble_advance(ens._members, 1, 2, ens.workspace.data_ptr(), ens.workspace.numel(), st),
                   lib.nsgb_ensemble_persistent(ens._members, 1, pws.data_ptr(), pws.numel(), st)]
        finally:
            g.capture_end()
    assert rcs == [1, 1, 1], rcs
