"""Parameter optimisation on the device: the reference's
``ParameterOptimizationStudy`` (studies.py:864-934) with its optax optimisers
(studies.py:879-884, optax 0.2.4) restated as one C-ABI call per optimiser
(``nsgb_optimize``): every step is the discrete-adjoint gradient of the
solver's objective followed by a one-launch optimiser update, all ordered on
the CUDA stream, so the 100-step loop never returns to the host.

Usage mirrors studies.py:

    solver = SingleCoreNSSolver(grid, phys, time, advection_scheme="central")
    study = ParameterOptimizationStudy(solver.jit_objective, solver.jit_gradient,
                                       theta0=[1.0, 0.5], optim_steps=100)
    study.run_all()
    study.save_results("optimization_study_results.npz")

``adam``, ``sgd`` and ``rmsprop`` take the optax arguments of the same name.
Plotting (``plot_convergence``) is not provided: the package has no plotting
dependency.
"""
from __future__ import annotations

import logging
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np
import torch

from . import _native
from .solver import SingleCoreNSSolver

logger = logging.getLogger(__name__)


@dataclass(frozen=True)
class OptimizerSpec:
    """One optimiser: ``kind`` is "sgd", "adam" or "rmsprop"; the remaining
    fields are optax 0.2.4's hyper-parameters and defaults."""
    kind: str
    learning_rate: float
    b1: float = 0.9
    b2: float = 0.999
    eps: float = 1e-8
    eps_root: float = 0.0
    decay: float = 0.9

    def native(self) -> _native.Optimizer:
        kinds = {"sgd": _native.OPT_SGD, "adam": _native.OPT_ADAM, "rmsprop": _native.OPT_RMSPROP}
        if self.kind not in kinds:
            raise ValueError(f"unknown optimizer {self.kind!r}")
        return _native.Optimizer(kinds[self.kind], float(self.learning_rate), float(self.b1), float(self.b2),
                                 float(self.eps), float(self.eps_root), float(self.decay))


def sgd(learning_rate: float) -> OptimizerSpec:
    """optax.sgd(learning_rate): theta -= lr * g."""
    return OptimizerSpec("sgd", learning_rate)


def adam(learning_rate: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8,
         eps_root: float = 0.0) -> OptimizerSpec:
    """optax.adam(learning_rate, b1, b2, eps, eps_root)."""
    return OptimizerSpec("adam", learning_rate, b1=b1, b2=b2, eps=eps, eps_root=eps_root)


def rmsprop(learning_rate: float, decay: float = 0.9, eps: float = 1e-8) -> OptimizerSpec:
    """optax.rmsprop(learning_rate, decay, eps) (eps inside the square root,
    zero initial scale, no momentum)."""
    return OptimizerSpec("rmsprop", learning_rate, decay=decay, eps=eps)


def default_configs() -> list:
    """The four optimisers of the reference study (studies.py:879-884)."""
    return [
        {"name": "Adam (lr=0.01)", "optimizer": adam(learning_rate=0.01)},
        {"name": "Adam (lr=0.001)", "optimizer": adam(learning_rate=0.001)},
        {"name": "SGD (lr=0.1)", "optimizer": sgd(learning_rate=0.1)},
        {"name": "RMSprop (lr=0.01)", "optimizer": rmsprop(learning_rate=0.01)},
    ]


class ParameterOptimizationStudy:
    """Compare optimisers on the same objective (studies.py:864-934).

    ``objective`` and ``grad_jax`` are a ``SingleCoreNSSolver``'s
    ``jit_objective`` and ``jit_gradient`` (J and dJ/dtheta from the zero
    initial state, NS_solver.py:724-725, 752-756); the study runs on that
    solver's device with its grid, physics, time stepping and checkpoint
    policy."""

    def __init__(self, objective: Callable, grad_jax: Callable, theta0, optim_configs: Optional[list] = None,
                 optim_steps: int = 100):
        solver = getattr(grad_jax, "__self__", None)
        if not isinstance(solver, SingleCoreNSSolver) or getattr(objective, "__self__", None) is not solver:
            raise TypeError("ParameterOptimizationStudy needs the jit_objective and jit_gradient of one "
                            "SingleCoreNSSolver")
        self.objective = objective
        self.grad_jax = grad_jax
        self.solver = solver
        self.theta0 = torch.as_tensor(np.asarray(theta0, np.float32))
        if self.theta0.numel() not in (2, 3):
            raise ValueError(f"theta0 must have 2 or 3 entries, got {self.theta0.numel()}")
        self.optim_steps = int(optim_steps)
        self.optim_configs = optim_configs or default_configs()
        self.results: dict = {}
        logger.info(f"ParameterOptimizationStudy initialized: {len(self.optim_configs)} optimizers, "
                    f"{self.optim_steps} steps")

    def _launch_optimizer(self, optimizer: OptimizerSpec):
        """Enqueue one optimiser's whole loop on the current stream; device
        tensors (objectives, parameters)."""
        s = self.solver
        g, ph = s.grid, s.phys
        return _native.optimize(
            self.theta0.to(s.device), int(s.time.steps), s._every(), g.N, float(g.L), float(ph.nu),
            float(s.time.dt), s._scheme_id, optimizer.native(), self.optim_steps, u0=None,
            mu0=float(ph.mu0), sigma0=float(ph.sigma0), C=float(ph.C))

    def _run_single_optimizer(self, name: str, optimizer: OptimizerSpec) -> dict:
        return self._collect(name, *self._launch_optimizer(optimizer))

    def _collect(self, name: str, objectives, parameters) -> dict:
        objectives = objectives.cpu().numpy()
        parameters = parameters.cpu().numpy()
        obj_initial = float(objectives[0])
        obj_final = float(objectives[-1])
        improvement = float((obj_initial - obj_final) / (obj_initial + 1e-20))
        logger.info(f"{name}: initial={obj_initial:.6e}, final={obj_final:.6e}, improvement={improvement*100:.3f}%")
        return {
            "obj_initial": obj_initial,
            "obj_final": obj_final,
            "improvement": improvement,
            "history": {
                "steps": np.arange(self.optim_steps + 1, dtype=np.int32),
                "objectives": objectives,
                "parameters": parameters,
            },
        }

    def run_all(self) -> dict:
        """Every optimiser's loop, each enqueued by its own host thread on its
        own CUDA stream, so the loops overlap on the device (they share
        nothing: each has its own workspace and graph; one thread alone
        would wait for the launch queue it fills); results equal running them
        one by one."""
        import threading
        logger.info(f"Testing {len(self.optim_configs)} optimizer configurations over {self.optim_steps} steps")
        dev = self.solver.device
        cur = torch.cuda.current_stream(dev)
        sides = [torch.cuda.Stream(dev) for _ in self.optim_configs]
        outs = [None] * len(sides)
        errors = []

        def enqueue(k, cfg):
            try:
                torch.cuda.set_device(dev)
                with torch.cuda.stream(sides[k]):
                    outs[k] = self._launch_optimizer(cfg["optimizer"])
            except Exception as exc:  # re-raised on the caller's thread
                errors.append(exc)

        for side in sides:
            side.wait_stream(cur)
        threads = [threading.Thread(target=enqueue, args=(k, cfg)) for k, cfg in enumerate(self.optim_configs)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        results = {}
        for cfg, side, out in zip(self.optim_configs, sides, outs):
            cur.wait_stream(side)
            for t in out:
                t.record_stream(cur)
            results[cfg["name"]] = self._collect(cfg["name"], *out)
        self.results = results
        return results

    def save_results(self, filename: str = "result/optimization_study_results.npz") -> None:
        """The reference's npz layout (studies.py:948-963)."""
        if not self.results:
            logger.warning("No optimization results to save")
            return
        data = {}
        for name, r in self.results.items():
            data[f"{name}_obj_initial"] = r["obj_initial"]
            data[f"{name}_obj_final"] = r["obj_final"]
            data[f"{name}_improvement"] = r["improvement"]
            data[f"{name}_steps"] = np.array(r["history"]["steps"])
            data[f"{name}_objectives"] = np.array(r["history"]["objectives"])
            data[f"{name}_parameters"] = np.array(r["history"]["parameters"])
        np.savez(filename, **data)
        logger.info(f"Saved to {filename}")
