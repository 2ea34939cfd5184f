"""Seeded input generators: determinism, rms 1, spectral divergence-freeness."""
import numpy as np

from ns_solver_jax_differential_distributed_gb300.workloads import (
    PLAIN_SCALE_CENTRAL, PLAIN_SMALL, ensemble, spectral_u0, theta_draw)


def test_u0_deterministic_rms_and_solenoidal():
    a = spectral_u0(64, 8, 0)
    b = spectral_u0(64, 8, 0)
    assert a.dtype == np.float32 and a.shape == (2, 64, 64)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, spectral_u0(64, 8, 1))
    assert abs(np.sqrt(np.mean(a[0].astype(np.float64) ** 2 + a[1] ** 2)) - 1) < 1e-6
    ux, uy = np.fft.fft2(a[0].astype(np.float64)), np.fft.fft2(a[1].astype(np.float64))
    k = np.fft.fftfreq(64, 1 / 64)
    KX, KY = np.meshgrid(k, k, indexing="ij")
    div = KX * ux + KY * uy
    assert np.max(np.abs(div)) / np.max(np.abs(ux)) < 1e-5


def test_u0_band_limited():
    u = spectral_u0(128, 8, 3).astype(np.float64)
    spec = np.abs(np.fft.fft2(u[0]))
    k = np.fft.fftfreq(128, 1 / 128)
    KX, KY = np.meshgrid(k, k, indexing="ij")
    assert spec[np.sqrt(KX ** 2 + KY ** 2) > 8.5].max() < 1e-9 * spec.max()


def test_theta_draw_within_20pct():
    th = theta_draw(1e-3, 0)
    base = np.array([1.0, 0.5, 1e-3])
    assert th.shape == (3,) and np.all(np.abs(th / base - 1) <= 0.2 + 1e-6)
    assert np.array_equal(th, theta_draw(1e-3, 0))


def test_named_workloads():
    assert PLAIN_SMALL.N == 128 and PLAIN_SMALL.steps == 100 and PLAIN_SMALL.K == 8
    assert PLAIN_SCALE_CENTRAL.cell_steps == 4096 * 4096 * 200


def test_ensemble_distribution():
    ens = ensemble()
    assert len(ens) == 256
    Ns = np.array([m.N for m in ens])
    assert set(Ns) <= {64, 128, 256, 512}
    frac = [np.mean(Ns == n) for n in (64, 128, 256, 512)]
    assert abs(frac[0] - 0.4) < 0.1 and abs(frac[3] - 0.1) < 0.06
    nus = np.array([m.nu for m in ens])
    assert nus.min() >= 1e-4 and nus.max() <= 1e-2
    assert [m.N for m in ensemble()] == list(Ns)
