"""Seeded synthetic inputs with the shapes of the reference's experiments.

The reference has no datasets: its drivers build analytic fields
(experiments/run-compact.py:30-40, run-adi.py:41-44).  These generators give
the same kinds of inputs, deterministic per seed, built directly on the GPU.
"""
import math

import numpy as np

COMPACT_COEFFS = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)  # experiments/run-compact.py:48


def fourier_modes(ndim, seed=0, modes=8, kmax=16):
    """(amplitudes ~ N(0,1), integer wavevectors in [1, kmax], phases U(0,1))."""
    rng = np.random.default_rng(seed)
    amps, ks, phases = [], [], []
    for _ in range(modes):
        ks.append(rng.integers(1, kmax + 1, size=ndim))
        phases.append(rng.random())
        amps.append(rng.normal())
    return np.array(amps), np.array(ks), np.array(phases)


def fourier_field(shape, seed=0, modes=8, kmax=16, device="cuda", dtype=None):
    """f = sum_m A_m sin(2 pi (k_m . x + phi_m)) on the unit cube/square grid
    with len(shape) axes (C order, last axis fastest), float64 on `device`."""
    import torch

    dtype = dtype or torch.float64
    amps, ks, phases = fourier_modes(len(shape), seed, modes, kmax)
    axes = [torch.linspace(0, 1, s, dtype=dtype, device=device) for s in shape]
    f = torch.zeros(shape, dtype=dtype, device=device)
    for a, k, p in zip(amps, ks, phases):
        arg = None
        for d, (kk, ax) in enumerate(zip(k, axes)):
            view = [1] * len(shape)
            view[d] = shape[d]
            term = (2 * math.pi * float(kk)) * ax.view(view)
            arg = term if arg is None else arg + term
        f += float(a) * torch.sin(arg + 2 * math.pi * float(p))
    return f


def fourier_block(shape, lo, hi, seed=0, modes=8, kmax=16):
    """NumPy block [lo[d], hi[d]) of fourier_field(shape, seed) (same modes,
    same grid), for host code that holds only part of a field."""
    amps, ks, phases = fourier_modes(len(shape), seed, modes, kmax)
    axes = [np.linspace(0, 1, s)[a:b] for s, a, b in zip(shape, lo, hi)]
    f = np.zeros([b - a for a, b in zip(lo, hi)])
    for a, k, p in zip(amps, ks, phases):
        arg = 2 * math.pi * float(p)
        for d, (kk, ax) in enumerate(zip(k, axes)):
            view = [1] * len(shape)
            view[d] = ax.size
            arg = arg + (2 * math.pi * float(kk)) * ax.reshape(view)
        f += float(a) * np.sin(arg)
    return f


def gaussians_2d(N, seed=0, count=16, wmin=0.02, wmax=0.1, device="cuda"):
    """Sum of `count` Gaussians, centres U(0,1)^2, widths U(wmin, wmax), with
    zero Dirichlet boundary (the ADI initial condition)."""
    import torch

    rng = np.random.default_rng(seed)
    g = torch.linspace(0, 1, N, dtype=torch.float64, device=device)
    y, x = torch.meshgrid(g, g, indexing="ij")
    u = torch.zeros((N, N), dtype=torch.float64, device=device)
    for _ in range(count):
        cx, cy = rng.random(2)
        w = rng.uniform(wmin, wmax)
        u += torch.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * w * w))
    u[0, :] = 0
    u[-1, :] = 0
    u[:, 0] = 0
    u[:, -1] = 0
    return u


def uneven_batch(count=4096, nmin=32, nmax=8192, seed=0):
    """Lengths log-uniform in [nmin, nmax]; interior b = 1, a, c ~ U(0.1, 0.3);
    the first and last two rows random and diagonally dominant; RHS ~ N(0,1).
    Returns (lengths, rows) where rows[s] = (a, b, c) arrays of length n_s."""
    rng = np.random.default_rng(seed)
    lengths = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=count)).astype(np.int64)
    lengths = np.clip(lengths, nmin, nmax)
    systems = []
    for n in lengths:
        a_i, c_i = rng.uniform(0.1, 0.3, size=2)
        head = []
        tail = []
        for _ in range(2):
            aa, cc = rng.uniform(-0.4, 0.4, size=2)
            head.append((aa, abs(aa) + abs(cc) + rng.uniform(0.5, 1.5), cc))
            aa, cc = rng.uniform(-0.4, 0.4, size=2)
            tail.append((aa, abs(aa) + abs(cc) + rng.uniform(0.5, 1.5), cc))
        systems.append(((float(a_i), 1.0, float(c_i)), head, tail))
    return lengths, systems
