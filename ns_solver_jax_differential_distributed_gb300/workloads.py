"""Seeded synthetic inputs and the named workloads of the solver's benchmarks.

The reference has no dataset: its runs start from zero velocity.  The
workloads here use a divergence-free random initial condition instead, so
that advection and the pressure solve are exercised:

* u0: a streamfunction with complex Gaussian Fourier coefficients
  (a + ib)/sqrt(2), a, b ~ N(0,1), amplitude |k|^-3 for 1 <= |k| <= K and
  zero elsewhere (integer wavenumbers of the [0, 2 pi]^2 torus), turned into
  u = (d psi/dy, -d psi/dx) spectrally and scaled to rms speed 1; computed in
  float64 and rounded to float32.  Seed = solve index.
* theta: [A, B, nu] = [1.0, 0.5, nu_default] * (1 + 0.2 U(-1, 1)), the
  reference's forcing parameters (NS_solver.py:63-64) plus the viscosity.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

TWO_PI = 2.0 * math.pi


def spectral_u0(N: int, K: int, seed: int = 0) -> np.ndarray:
    """(2, N, N) float32 divergence-free velocity with rms speed 1."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(N, 1.0 / N)
    ky = np.fft.rfftfreq(N, 1.0 / N)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    kmag = np.sqrt(KX * KX + KY * KY)
    a = rng.standard_normal(KX.shape)
    b = rng.standard_normal(KX.shape)
    amp = np.where((kmag >= 1) & (kmag <= K), np.power(np.maximum(kmag, 1.0), -3.0), 0.0)
    psi_hat = (a + 1j * b) / math.sqrt(2.0) * amp
    ux = np.fft.irfft2(1j * KY * psi_hat, s=(N, N))
    uy = np.fft.irfft2(-1j * KX * psi_hat, s=(N, N))
    rms = math.sqrt(float(np.mean(ux * ux + uy * uy)))
    if rms == 0:
        raise ValueError("empty spectrum: K must be >= 1")
    return np.stack([ux / rms, uy / rms]).astype(np.float32)


def theta_draw(nu_default: float, seed: int = 0, spread: float = 0.2) -> np.ndarray:
    """[A, B, nu] uniformly within +-spread of [1.0, 0.5, nu_default]."""
    rng = np.random.default_rng(seed)
    base = np.array([1.0, 0.5, nu_default], dtype=np.float64)
    return (base * (1.0 + spread * rng.uniform(-1.0, 1.0, size=3))).astype(np.float32)


@dataclass(frozen=True)
class PlainWorkload:
    """A single solve on [0, L]^2."""
    name: str
    N: int
    steps: int
    dt: float
    nu: float
    scheme: str
    K: int
    L: float = TWO_PI
    seed: int = 0

    def u0(self) -> np.ndarray:
        return spectral_u0(self.N, self.K, self.seed)

    def theta(self) -> np.ndarray:
        return theta_draw(self.nu, self.seed)

    @property
    def cell_steps(self) -> int:
        return self.N * self.N * self.steps


# Small parity case (runs on CPU in the reference), the headline throughput
# case (both schemes) and the differentiation case.
PLAIN_SMALL = PlainWorkload("plain-N128-central", 128, 100, 1e-3, 1e-3, "central", 8)
PLAIN_SCALE_CENTRAL = PlainWorkload("plain-N4096-central", 4096, 200, 2.5e-4, 1e-4, "central", 32)
PLAIN_SCALE_UPWIND = PlainWorkload("plain-N4096-upwind", 4096, 200, 2.5e-4, 1e-4, "upwind", 32)
GRAD_N1024 = PlainWorkload("grad-N1024-upwind", 1024, 1000, 1e-3, 5e-4, "upwind", 32)
GRAD_CHECKPOINT_EVERY = 50


@dataclass(frozen=True)
class EnsembleMember:
    index: int
    N: int
    steps: int
    dt: float
    nu: float
    theta: np.ndarray = field(repr=False, compare=False)
    scheme: str = "central"
    L: float = TWO_PI
    K: int = 32

    def u0(self) -> np.ndarray:
        return spectral_u0(self.N, self.K, self.index)


def ensemble(count: int = 256, steps: int = 500, seed: int = 1234, dt: float = 1e-3,
             sizes=(64, 128, 256, 512), probs=(0.4, 0.3, 0.2, 0.1),
             scheme: str = "central") -> list:
    """Ensemble of independent solves of uneven size: N drawn from `sizes`
    with `probs`, nu log-uniform in [1e-4, 1e-2], theta within +-20% of the
    defaults (seed = solve index), u0 seeded by the solve index."""
    rng = np.random.default_rng(seed)
    Ns = rng.choice(np.asarray(sizes), size=count, p=np.asarray(probs))
    nus = np.exp(rng.uniform(math.log(1e-4), math.log(1e-2), size=count))
    out = []
    for i in range(count):
        th = theta_draw(float(nus[i]), seed=i)
        th[2] = np.float32(nus[i])  # per-solve nu is the drawn value itself
        out.append(EnsembleMember(i, int(Ns[i]), steps, dt, float(nus[i]), th, scheme))
    return out
