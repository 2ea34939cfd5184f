"""Autograd twin of the reference rollout (TEST INFRASTRUCTURE, CPU only).

The reference differentiates its rollout with ``jax.grad`` (NS_solver.py:725).
JAX is not available here, so this module restates the same algorithm as
``ns_oracle`` in torch (CPU, float64 by default) and lets torch's reverse-mode
autograd differentiate it.  It is the stand-in for the reference's JAX
gradient in the adjoint parity tests: like JAX, torch takes the derivative of
``round`` as 0 and of ``where`` through the selected branch only.

Only the tests may import it; the product never does.
"""
from __future__ import annotations

import math

import torch


def _roll(f, shift, dim):
    return torch.roll(f, shifts=shift, dims=dim)


def grad(f, dx):
    h = 2 * dx
    return (_roll(f, -1, 0) - _roll(f, 1, 0)) / h, (_roll(f, -1, 1) - _roll(f, 1, 1)) / h


def laplacian(f, dx):
    return (_roll(f, 1, 0) + _roll(f, -1, 0) + _roll(f, -1, 1) + _roll(f, 1, 1) - 4 * f) / (dx ** 2)


def advect(f, ux, uy, dx, scheme):
    if scheme == "central":
        fx, fy = grad(f, dx)
        return -(ux * fx + uy * fy)
    dfx = torch.where(ux >= 0, f - _roll(f, 1, 0), _roll(f, -1, 0) - f) / dx
    dfy = torch.where(uy >= 0, f - _roll(f, 1, 1), _roll(f, -1, 1) - f) / dx
    return -(ux * dfx + uy * dfy)


def inv_k2(N, dx, dtype):
    m = torch.cat([torch.arange(0, N // 2), torch.arange(-(N // 2), 0)]).to(dtype)
    k = m / (dx * N) * 2 * math.pi
    KX, KY = torch.meshgrid(k, k, indexing="ij")
    k2 = KX * KX + KY * KY
    return torch.where(k2 == 0, torch.zeros_like(k2), 1.0 / torch.where(k2 == 0, torch.ones_like(k2), k2))


def poisson(rhs, ik2):
    p_hat = -torch.fft.fft2(rhs) * ik2
    mask = torch.ones_like(ik2)
    mask[0, 0] = 0
    return torch.fft.ifft2(p_hat * mask).real


def forcing_fx(theta, t, N, L, mu0=0.5, sigma0=0.1, C=1.0, dtype=torch.float64):
    A, B = theta[0], theta[1]
    x = L * (torch.arange(N, dtype=dtype) / N)
    mu = mu0 + torch.sin(2 * math.pi * A * t)
    sig = sigma0 + torch.cos(2 * math.pi * B * t) ** 2
    r = x - mu
    d = r - torch.round(r)
    return C * torch.exp(-(d * d) / (2 * sig * sig))


def rollout(u0, theta, N, L, dt, steps, scheme, nu=None, mu0=0.5, sigma0=0.1, C=1.0):
    """(J, u_final) of SingleCoreNSSolver.rollout (NS_solver.py:732-750);
    theta = [A, B] or [A, B, nu]."""
    dtype = u0.dtype
    dx = L / N
    ik2 = inv_k2(N, dx, dtype)
    nu_v = theta[2] if theta.numel() == 3 else nu
    u = u0
    J = torch.zeros((), dtype=dtype)
    for i in range(steps):
        t = i * dt
        fx = forcing_fx(theta, t, N, L, mu0, sigma0, C, dtype)
        f0 = fx[:, None].expand(N, N)
        J = J + dt * torch.sum(u[0] * f0) * dx ** 2
        ux, uy = u[0], u[1]
        ux_s = ux + dt * (nu_v * laplacian(ux, dx) + advect(ux, ux, uy, dx, scheme) + f0)
        uy_s = uy + dt * (nu_v * laplacian(uy, dx) + advect(uy, ux, uy, dx, scheme))
        gx, _ = grad(ux_s, dx)
        _, gy = grad(uy_s, dx)
        p = poisson((gx + gy) / dt, ik2)
        px, py = grad(p, dx)
        u = torch.stack([ux_s - dt * px, uy_s - dt * py])
    return J, u


def gradient(u0, theta, N, L, dt, steps, scheme, nu=None, wrt_u0=False):
    """dJ/dtheta (and dJ/du0) by reverse-mode autograd in float64."""
    th = torch.as_tensor(theta, dtype=torch.float64).clone().requires_grad_(True)
    u = torch.as_tensor(u0, dtype=torch.float64).clone().requires_grad_(wrt_u0)
    J, _ = rollout(u, th, N, L, dt, steps, scheme, nu=nu)
    J.backward()
    if wrt_u0:
        return float(J), th.grad.numpy().copy(), u.grad.numpy().copy()
    return float(J), th.grad.numpy().copy()
