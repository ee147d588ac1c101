"""Seeded synthetic workloads with the shapes and distributions of the benchmark configs.

* ``gaussian_mixture``: a mixture of 5 isotropic Gaussians, centres uniform
  in [-3, 3]^2, sigma uniform in [0.1, 1.0], equal weights (the
  5-Gaussian example of datashader's getting-started guide, regenerated here).
* ``pyramid_points``: points in [0, 1)^2, half uniform and half from 20
  Gaussians with sigma in [1e-3, 1e-1] (clipped into the unit square).
* ``time_series``: n series of m vertices, x = linspace(0, 1), y = cumsum of
  N(0, 0.01) steps, laid out like utils.dataframe_from_multiple_sequences
  (utils.py:485-515): a NaN row after each series.

Each generator has a numpy form (small sizes, host) and a torch form that
draws directly on the GPU (large sizes); both are deterministic for a seed
but they do not produce the same numbers as each other.
"""
from __future__ import annotations

import numpy as np


def _mixture_params(rng, k, lo, hi, slo, shi):
    centres = rng.uniform(lo, hi, size=(k, 2))
    sigmas = rng.uniform(slo, shi, size=k)
    return centres, sigmas


def gaussian_mixture_np(n, seed=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    centres, sigmas = _mixture_params(rng, 5, -3.0, 3.0, 0.1, 1.0)
    comp = rng.integers(0, 5, size=n)
    xy = rng.standard_normal((n, 2)) * sigmas[comp, None] + centres[comp]
    return xy[:, 0].astype(dtype), xy[:, 1].astype(dtype)


def gaussian_mixture_torch(n, seed=0, dtype=None, device="cuda", chunk=1 << 26):
    import torch
    dtype = dtype or torch.float32
    rng = np.random.default_rng(seed)
    centres, sigmas = _mixture_params(rng, 5, -3.0, 3.0, 0.1, 1.0)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    c = torch.tensor(centres, dtype=torch.float64, device=device)
    s = torch.tensor(sigmas, dtype=torch.float64, device=device)
    x = torch.empty(n, dtype=dtype, device=device)
    y = torch.empty(n, dtype=dtype, device=device)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        comp = torch.randint(0, 5, (b - a,), generator=g, device=device)
        z = torch.randn((b - a, 2), generator=g, device=device, dtype=torch.float64)
        xy = z * s[comp, None] + c[comp]
        x[a:b] = xy[:, 0].to(dtype)
        y[a:b] = xy[:, 1].to(dtype)
    return x, y


def lognormal_torch(n, seed=1, device="cuda", chunk=1 << 26):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    v = torch.empty(n, dtype=torch.float64, device=device)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        v[a:b] = torch.randn(b - a, generator=g, device=device, dtype=torch.float64).exp_()
    return v


def categories_torch(n, k, seed=2, device="cuda", dtype=None):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    return torch.randint(0, k, (n,), generator=g, device=device, dtype=dtype or torch.int8)


def pyramid_points_np(n, seed=0, dtype=np.float32):
    rng = np.random.default_rng(seed)
    centres, sigmas = _mixture_params(rng, 20, 0.0, 1.0, 1e-3, 1e-1)
    nu = n // 2
    xy = np.empty((n, 2))
    xy[:nu] = rng.uniform(0.0, 1.0, size=(nu, 2))
    comp = rng.integers(0, 20, size=n - nu)
    xy[nu:] = rng.standard_normal((n - nu, 2)) * sigmas[comp, None] + centres[comp]
    np.clip(xy, 0.0, np.nextafter(1.0, 0.0), out=xy)
    return xy[:, 0].astype(dtype), xy[:, 1].astype(dtype)


def pyramid_points_torch(n, seed=0, device="cuda", chunk=1 << 26):
    import torch
    rng = np.random.default_rng(seed)
    centres, sigmas = _mixture_params(rng, 20, 0.0, 1.0, 1e-3, 1e-1)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    c = torch.tensor(centres, dtype=torch.float64, device=device)
    s = torch.tensor(sigmas, dtype=torch.float64, device=device)
    x = torch.empty(n, dtype=torch.float32, device=device)
    y = torch.empty(n, dtype=torch.float32, device=device)
    nu = n // 2
    top = float(np.nextafter(np.float32(1.0), np.float32(0.0)))
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        m = b - a
        u = torch.rand((m, 2), generator=g, device=device, dtype=torch.float64)
        comp = torch.randint(0, 20, (m,), generator=g, device=device)
        z = torch.randn((m, 2), generator=g, device=device, dtype=torch.float64) * s[comp, None] + c[comp]
        rows = torch.arange(a, b, device=device)
        xy = torch.where((rows < nu)[:, None], u, z).clamp_(0.0, top)
        x[a:b] = xy[:, 0].to(torch.float32).clamp_(0.0, top)
        y[a:b] = xy[:, 1].to(torch.float32).clamp_(0.0, top)
    return x, y


def time_series_np(nseries, length, seed=0, step=0.01):
    """x, y (float64) with NaN separators, and v (uniform [0, 1)) per vertex."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, length)
    ys = np.cumsum(rng.normal(0.0, step, size=(nseries, length)), axis=1)
    x = np.zeros(length + 1)
    x[-1] = np.nan
    x[:-1] = xs
    x = np.tile(x, nseries)
    y = np.zeros((nseries, length + 1))
    y[:, -1] = np.nan
    y[:, :-1] = ys
    v = rng.uniform(0.0, 1.0, size=x.shape[0])
    return x, y.ravel(), v, ys
