"""Seeded synthetic inputs for the Poisson solver.

Manufactured solution on [-pi, pi]^3 with n_a interior points per axis,
h_a = 2 pi / (n_a + 1), x_j = -pi + j h_a:

    u = sum_{m=1..terms} a_m sin(k1_m (x+pi)/2) sin(k2_m (y+pi)/2) sin(k3_m (z+pi)/2)

Each term is a DST-I basis vector (sin(k j pi/(n+1)) at x_j), so the 7-point
Laplacian acts on it by its eigenvalue -(lx(k1)+ly(k2)+lz(k3)) with
l(k) = 4/h^2 sin^2(k pi / (2(n+1))); f is built that way (the discrete
Laplacian of u) and `noise` adds N(0, noise^2) white noise to f.  Integer k's
are uniform in [1, kmax] and a_m ~ N(0,1), all from the seed.
"""
from __future__ import annotations

import math

import numpy as np


def grid_h(n: int) -> float:
    return 2 * math.pi / (n + 1)


def solver_args(nx: int, ny: int, nz: int):
    """(dx, dy, dz, lx, ly, lz, nx, ny, nz) of LaplCube for the box."""
    hx, hy, hz = grid_h(nx), grid_h(ny), grid_h(nz)
    return hx, hy, hz, (nx + 1) * hx, (ny + 1) * hy, (nz + 1) * hz, nx, ny, nz


def params(seed: int, kmax, terms: int = 8):
    """k's (terms x 3: kx, ky, kz) and amplitudes.  kmax: int or (kx, ky, kz)."""
    rng = np.random.default_rng(seed)
    km = np.broadcast_to(np.asarray(kmax, dtype=np.int64), (3,))
    ks = np.stack([rng.integers(1, km[a] + 1, size=terms) for a in range(3)], axis=1)
    amp = rng.standard_normal(terms)
    return ks, amp


def _lam(k, n):
    h = grid_h(n)
    return 4.0 / (h * h) * np.sin(k * math.pi / (2 * (n + 1))) ** 2


def _basis(k, n):
    j = np.arange(1, n + 1)
    return np.sin(k * j * math.pi / (n + 1))


def manufactured(nx: int, ny: int, nz: int, seed: int, kmax, terms: int = 8, noise: float = 0.0):
    """(f, u) as float64 arrays of shape (nz, ny, nx)."""
    ks, amp = params(seed, kmax, terms)
    u = np.zeros((nz, ny, nx))
    f = np.zeros((nz, ny, nx))
    for m in range(terms):
        kx, ky, kz = ks[m]
        t = amp[m] * np.einsum("i,k,j->ikj", _basis(kz, nz), _basis(ky, ny), _basis(kx, nx))
        u += t
        f -= (_lam(kx, nx) + _lam(ky, ny) + _lam(kz, nz)) * t
    if noise:
        rng = np.random.default_rng(seed + 7919)
        f += rng.normal(0.0, noise, f.shape)
    return f, u


def manufactured_torch(nx: int, ny: int, nz: int, seed: int, kmax, terms: int = 8, noise: float = 0.0,
                       device="cuda"):
    """The same f (and u) built on a device with torch; the noise comes from a
    torch generator seeded with the same seed (so it differs from the numpy
    version's noise, but is reproducible on a given device)."""
    import torch
    ks, amp = params(seed, kmax, terms)
    u = torch.zeros((nz, ny, nx), dtype=torch.float64, device=device)
    f = torch.zeros_like(u)
    for m in range(terms):
        kx, ky, kz = (int(v) for v in ks[m])
        bz = torch.from_numpy(_basis(kz, nz)).to(device)
        by = torch.from_numpy(_basis(ky, ny)).to(device)
        bx = torch.from_numpy(_basis(kx, nx)).to(device)
        t = float(amp[m]) * bz[:, None, None] * by[None, :, None] * bx[None, None, :]
        u += t
        f -= float(_lam(kx, nx) + _lam(ky, ny) + _lam(kz, nz)) * t
    if noise:
        g = torch.Generator(device=device)
        g.manual_seed(seed + 7919)
        f += noise * torch.randn(f.shape, generator=g, dtype=torch.float64, device=device)
    return f, u


def random_sizes(count: int, seed: int, choices=(31, 63, 127)):
    """count (nx, ny, nz) triples drawn independently from choices."""
    rng = np.random.default_rng(seed)
    return [tuple(int(c) for c in rng.choice(choices, size=3)) for _ in range(count)]


def uneven_batch_torch(count: int, seed: int, choices=(31, 63, 127), device="cuda"):
    """The uneven batch's right-hand sides: count volumes whose sizes per axis
    are drawn from choices (random_sizes), volume i manufactured like the
    single solves (8 terms, no noise) with k along each axis uniform in
    [1, (n+1)/4] for that axis's n, seeded by seed and i.  Returns (shapes,
    f list, u list) of float64 device tensors of shape (nz, ny, nx)."""
    shapes = random_sizes(count, seed)
    fs, us = [], []
    for i, (nx, ny, nz) in enumerate(shapes):
        f, u = manufactured_torch(nx, ny, nz, seed=seed * 100003 + i,
                                  kmax=((nx + 1) // 4, (ny + 1) // 4, (nz + 1) // 4), device=device)
        fs.append(f)
        us.append(u)
    return shapes, fs, us
