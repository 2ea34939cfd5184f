"""The reference's CLI and profiler contracts (unit_tests/test_distributed_solver.py
ProfilerAPITests :569-626 and RunnerArgParseTests :629-685) against this
package's runner and profiler; host-only, no GPU."""
import pytest

from ns_solver_jax_differential_distributed_gb300.profile_stages import (
    ProfileSummary, SolverKernelProfiler, benchmark_callable)
from ns_solver_jax_differential_distributed_gb300.runner import build_parser


def test_benchmark_callable_returns_profile_summary():
    r = SolverKernelProfiler.benchmark_callable("dummy", lambda: sum(range(100)), warmup=1, runs=3)
    assert isinstance(r, ProfileSummary) and r.label == "dummy" and r.mean_sec > 0.0


def test_benchmark_callable_min_le_mean_le_max():
    r = benchmark_callable("order", lambda: sum(range(100)), warmup=0, runs=5)
    assert r.min_sec <= r.mean_sec <= r.max_sec


def test_benchmark_callable_respects_run_count():
    log = []
    SolverKernelProfiler.benchmark_callable("count", lambda: log.append(1), warmup=2, runs=5)
    assert len(log) == 7


def test_benchmark_callable_zero_warmup_and_args():
    r = benchmark_callable("args", lambda a, b: a + b, 1, 2, warmup=0, runs=2)
    assert isinstance(r, ProfileSummary)


def test_profile_summary_fields():
    s = ProfileSummary(label="s", mean_sec=0.5, min_sec=0.4, max_sec=0.6, std_sec=0.05)
    assert (s.label, s.mean_sec, s.min_sec, s.max_sec, s.std_sec) == ("s", 0.5, 0.4, 0.6, 0.05)


def test_empty_args_give_defaults():
    a = build_parser().parse_args([])
    assert a.config is None and a.profile is False and a.profile_warmup == 1 and a.profile_runs == 5


def test_combined_flags():
    a = build_parser().parse_args(["--config", "my.json", "--profile", "--profile-warmup", "2",
                                   "--profile-runs", "8"])
    assert (a.config, a.profile, a.profile_warmup, a.profile_runs) == ("my.json", True, 2, 8)


@pytest.mark.parametrize("argv", [["--profile-warmup", "notanint"], ["--profile-runs", "3.5"]])
def test_integer_flags_reject_non_integers(argv):
    with pytest.raises(SystemExit):
        build_parser().parse_args(argv)
