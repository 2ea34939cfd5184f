"""The C-ABI library loads and exports every entry point that include/nsgb.h
declares; argument errors are reported without touching a GPU."""
import ctypes
import os
import re

import pytest

from ns_solver_jax_differential_distributed_gb300 import _build, _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "nsgb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nsgb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return ctypes.CDLL(_build.LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "nsgb_rollout" in names and "nsgb_rollout_grad" in names and len(names) >= 18


def test_every_declared_symbol_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_version_and_argument_errors(lib):
    L = _native.lib()
    assert L.nsgb_version() == 10000
    h = ctypes.c_void_p()
    for N in (100, 8, 16384, 0, -4):
        assert L.nsgb_plan_create(N, 1.0, ctypes.byref(h)) == 2  # NSGB_ERR_UNSUPPORTED_N
        assert b"unsupported" in L.nsgb_last_error()
    assert L.nsgb_plan_create(64, -1.0, ctypes.byref(h)) == 1
    assert L.nsgb_plan_create(64, 1.0, None) == 1
    assert L.nsgb_rollout(None, None, None, None, 2, 1, None, None, None, 0, 0, None) == 1
    assert b"plan" in L.nsgb_last_error()
    assert L.nsgb_poisson_workspace_bytes(None) == 0
    # launch-tuning and measurement entry points refuse a NULL plan before
    # touching the device
    out = (ctypes.c_int * 2)()
    assert L.nsgb_plan_set_adjoint_tiles(None, 64, 16) == 1
    assert L.nsgb_plan_get_adjoint_tiles(None, out) == 1
    assert L.nsgb_plan_set_fft_radix(None, 16, 16) == 1
    outf = (ctypes.c_float * 4)()
    assert L.nsgb_time_step_pipeline(None, None, None, None, 2, 4, None, 0, outf, None) == 1
    assert b"plan" in L.nsgb_last_error()
    assert L.nsgb_rollout_grad(None, None, None, None, 2, 4, 1, 3, None, None, None, None, None, 0, None) == 1
    assert L.nsgb_rollout_grad_workspace_bytes(None, 4, 1) == 0


def test_misaligned_field_rejected_before_launch(lib):
    """Step kernels read fields as float4 groups: a pointer that is not
    16-byte aligned is refused at the boundary (checked before the plan is
    used, so a placeholder plan handle suffices here)."""
    L = _native.lib()
    dummy_plan = ctypes.create_string_buffer(64)
    ph = _native.make_phys(1.0, 0.01, 1e-3, "central")
    theta = ctypes.create_string_buffer(16)
    rc = L.nsgb_rollout(ctypes.addressof(dummy_plan), ctypes.byref(ph), 0x1004, ctypes.addressof(theta), 2, 1,
                        0x2000, 0x3000, 0x4000, 1 << 20, 0, None)
    assert rc == 1 and b"16-byte aligned" in L.nsgb_last_error()


def _grad_ops(steps, every):
    """Operations of a gradient solve: forward steps, then per checkpoint
    segment its recomputed steps (none for one step) and adjoint steps."""
    segs = [min(every, steps - s0) for s0 in range(0, steps, every)]
    return steps + sum(1 if n == 1 else 2 * n for n in segs)


def test_grad_batch_schedule_and_arguments(lib):
    L = _native.lib()
    for steps, every in [(1, 1), (5, 1), (10, 4), (12, 4), (7, 50), (1000, 50), (999, 7)]:
        assert L.nsgb_grad_ops(steps, every) == _grad_ops(steps, every)
    assert L.nsgb_grad_ops(0, 1) == 0 and L.nsgb_grad_ops(4, 0) == 0
    assert L.nsgb_grad_batch_workspace_bytes(0, 8) == 0
    assert L.nsgb_grad_batch_workspace_bytes(3, 8) > 0
    assert L.nsgb_grad_batch_advance(None, 1, 4, None, 0, None) == 1
    assert b"empty" in L.nsgb_last_error()


def test_ensemble_entry_points_refuse_bad_members(lib):
    """The ensemble calls check their member tables before any device work:
    an empty table, a NULL plan and steps out of range come back as
    NSGB_ERR_INVALID_ARG with a message (no GPU is touched)."""
    L = _native.lib()
    assert L.nsgb_ensemble_workspace_bytes(None, 0) == 0
    assert L.nsgb_ensemble_persistent_workspace_bytes(None, 0) == 0
    for call in (lambda: L.nsgb_ensemble_advance(None, 0, 4, None, 0, None),
                 lambda: L.nsgb_ensemble_rollout(None, 0, 8, None, 0, None),
                 lambda: L.nsgb_ensemble_persistent(None, 0, None, 0, None)):
        assert call() == 1 and b"empty" in L.nsgb_last_error()
    m = (_native.Member * 1)()
    m[0].plan = None
    m[0].phys = _native.make_phys(1.0, 0.01, 1e-3, "central")
    assert L.nsgb_ensemble_advance(m, 1, 4, None, 0, None) == 1
    assert b"plan is NULL" in L.nsgb_last_error()
    gm = (_native.GradMember * 1)()
    assert L.nsgb_grad_batch_advance(gm, 1, 4, None, 0, None) == 1
