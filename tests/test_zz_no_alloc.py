"""nsgb_poisson_noalloc: the spectral Poisson solve for callers that cannot
allocate device memory when they solve (a fixed device-memory budget they
cannot grow, loops where a cudaMalloc that may synchronise the device is not
acceptable, plain C FFI hosts that cannot own a plan and a workspace).  Its
scratch is a static device array shared by all calls, so the tests check
consecutive calls (different sizes and inputs) against the plan-and-workspace
entry point nsgb_poisson, through the C ABI.  The same kernels and the same
tables run in both, so the results must agree to the bit: a stale table or a
race on the shared arrays would show as a difference.  This file is collected
last, and passes alone in a fresh process as well."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

LX = 2 * math.pi


def _rhs(N, seed):
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.standard_normal((N, N)).astype(np.float32)).cuda()


def _reference(lib, _native, N, rhs, st):
    plan = _native.get_plan(N, LX, "cuda")
    ws = torch.empty(lib.nsgb_poisson_workspace_bytes(plan.handle), dtype=torch.uint8, device="cuda")
    p = torch.empty_like(rhs)
    assert lib.nsgb_poisson(plan.handle, rhs.data_ptr(), p.data_ptr(), ws.data_ptr(), ws.numel(), st) == 0
    torch.cuda.synchronize()
    return p


def test_noalloc_matches_poisson_on_consecutive_calls(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    st = torch.cuda.current_stream().cuda_stream
    # calls in a row; the second changes N, so the shared tables and the
    # shared spectrum are reused with new contents
    for call, (N, seed) in enumerate(((256, 0), (64, 1), (256, 2))):
        rhs = _rhs(N, seed)
        p_ref = _reference(lib, _native, N, rhs, st)
        p_na = torch.empty_like(rhs)
        assert lib.nsgb_poisson_noalloc(N, LX, rhs.data_ptr(), p_na.data_ptr(), st) == 0, \
            lib.nsgb_last_error().decode()
        torch.cuda.synchronize()
        assert torch.equal(p_na, p_ref), (call, N)


def test_noalloc_queued_calls_of_different_sizes(cuda_lib):
    """Three calls queued on one stream before a single synchronisation: each
    call's table upload must not be overwritten by the next call's host-side
    refill while it is still queued."""
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    st = torch.cuda.current_stream().cuda_stream
    cases = ((256, 10), (64, 11), (256, 12))
    rhs = [_rhs(N, seed) for N, seed in cases]
    refs = [_reference(lib, _native, N, r, st) for (N, _), r in zip(cases, rhs)]
    outs = [torch.empty_like(r) for r in rhs]
    for (N, _), r, o in zip(cases, rhs, outs):
        assert lib.nsgb_poisson_noalloc(N, LX, r.data_ptr(), o.data_ptr(), st) == 0, \
            lib.nsgb_last_error().decode()
    torch.cuda.synchronize()
    for k, (o, p) in enumerate(zip(outs, refs)):
        assert torch.equal(o, p), k


def test_noalloc_refuses_a_capturing_stream(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    rhs = _rhs(64, 4)
    out = torch.empty_like(rhs)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        assert lib.nsgb_poisson_noalloc(64, LX, rhs.data_ptr(), out.data_ptr(), s.cuda_stream) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = lib.nsgb_poisson_noalloc(64, LX, rhs.data_ptr(), out.data_ptr(), s.cuda_stream)
        msg = lib.nsgb_last_error()
        out.add_(0.0)  # the captured graph is not empty
    assert rc == 1 and b"capturing" in msg, (rc, msg)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    rhs = _rhs(64, 3)
    assert lib.nsgb_poisson_noalloc(2048, 1.0, rhs.data_ptr(), rhs.data_ptr(), None) == 2
    assert b"1024" in lib.nsgb_last_error()
    assert lib.nsgb_poisson_noalloc(100, 1.0, rhs.data_ptr(), rhs.data_ptr(), None) == 2
