"""nsgb_poisson_noalloc: the spectral Poisson solve for callers that cannot
allocate device memory when they solve (a fixed device-memory budget they
cannot grow, loops where a cudaMalloc that may synchronise the device is not
acceptable, plain C FFI hosts that cannot own a plan and a workspace).  Its
scratch is a static device array shared by all calls, so the test checks two
calls in a row (different sizes and inputs) against the plan-and-workspace
entry point nsgb_poisson, through the C ABI.  It lives in a file of its own
that pytest collects last, and passes alone in a fresh process as well."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rhs(N, seed):
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.standard_normal((N, N)).astype(np.float32)).cuda()


def test_noalloc_matches_poisson_on_consecutive_calls(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    st = torch.cuda.current_stream().cuda_stream
    Lx = 2 * math.pi
    # two calls in a row; the second changes N, so the shared tables and the
    # shared spectrum are reused with new contents
    for call, (N, seed) in enumerate(((256, 0), (64, 1), (256, 2))):
        plan = _native.get_plan(N, Lx, "cuda")
        ws = torch.empty(lib.nsgb_poisson_workspace_bytes(plan.handle), dtype=torch.uint8, device="cuda")
        rhs = _rhs(N, seed)
        p_ref, p_na = torch.empty_like(rhs), torch.empty_like(rhs)
        assert lib.nsgb_poisson(plan.handle, rhs.data_ptr(), p_ref.data_ptr(), ws.data_ptr(), ws.numel(), st) == 0
        assert lib.nsgb_poisson_noalloc(N, Lx, rhs.data_ptr(), p_na.data_ptr(), st) == 0, \
            lib.nsgb_last_error().decode()
        torch.cuda.synchronize()
        # the Poisson parity tolerance of the other tests; the same kernels and
        # tables make the results agree to the bit in practice
        rel = float((p_na.double() - p_ref.double()).norm() / p_ref.double().norm())
        assert rel < 2e-6, (call, N, rel)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    from ns_solver_jax_differential_distributed_gb300 import _native
    lib = _native.lib()
    rhs = _rhs(64, 3)
    assert lib.nsgb_poisson_noalloc(2048, 1.0, rhs.data_ptr(), rhs.data_ptr(), None) == 2
    assert b"1024" in lib.nsgb_last_error()
    assert lib.nsgb_poisson_noalloc(100, 1.0, rhs.data_ptr(), rhs.data_ptr(), None) == 2
