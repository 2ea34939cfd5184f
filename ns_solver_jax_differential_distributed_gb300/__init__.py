"""GB300-native single-device Chorin-projection Navier-Stokes solver.

A drop-in for the single-device path of the JAX reference solver
(helmhlotz/ns_solver_jax_differential_distributed): the same classes and
methods (``SingleCoreNSSolver.rollout``, ``jit_gradient``, the
``DifferentialOps`` / ``AdvectionScheme`` / ``SpectralPoissonSolver`` /
``ChorinProjector`` strategies), backed by hand-written sm_103a CUDA kernels
behind a C ABI (``include/nsgb.h``).
"""
from .solver import (  # noqa: F401
    CONFIG, AdvectionScheme, CentralAdvection, ChorinProjector, DifferentialOps,
    GaussianForcingField, Grid, PeriodicDifferentialOps, Phys, SimConfig, SingleCoreNSSolver,
    SpectralPoissonSolver, Time, UpwindAdvection, load_config, make_advection_scheme, make_grid,
    setup_logger,
)

__version__ = "1.0.0"
