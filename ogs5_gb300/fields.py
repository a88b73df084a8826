"""Seeded log-normal conductivity fields for the synthetic decks.

OGS-5 reads element-wise heterogeneous permeability from a
``$PERMEABILITY_DISTRIBUTION`` file (CMediumProperties::
SetDistributedELEProperties, FEM/rf_mmp_new.cpp:5725).  Here the field is
generated in memory: ln K is a stationary Gaussian random field with
exponential covariance  C(r) = var * exp(-|r| / ell)  on the element-centre
grid, sampled by circulant embedding on a grid twice the size in every
direction (FFT), negative embedding eigenvalues clipped to zero.
"""
from __future__ import annotations

import numpy as np


def gaussian_random_field(shape, var: float, ell: float, seed: int) -> np.ndarray:
    """Zero-mean GRF on a regular grid of cell centres (unit spacing)."""
    shape = tuple(int(s) for s in shape)
    ext = tuple(2 * s for s in shape)
    axes = [np.minimum(np.arange(m), m - np.arange(m)).astype(np.float64) for m in ext]
    grids = np.meshgrid(*axes, indexing="ij")
    r = np.sqrt(sum(g * g for g in grids))
    cov = var * np.exp(-r / ell)
    lam = np.fft.fftn(cov).real
    lam = np.clip(lam, 0.0, None)
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(ext) + 1j * rng.standard_normal(ext)
    f = np.fft.ifftn(np.sqrt(lam / np.prod(ext)) * noise * np.prod(ext)).real
    sl = tuple(slice(0, s) for s in shape)
    return np.ascontiguousarray(f[sl])


def lognormal_k(shape, mean_ln: float, var: float, ell: float, seed: int) -> np.ndarray:
    """Element-wise K = exp(mean_ln + GRF), flattened x-fastest like the meshes."""
    g = gaussian_random_field(shape[::-1], var, ell, seed)  # (nz, ny, nx) order
    return np.exp(mean_ln + g).ravel().astype(np.float64)


def lognormal_k_device(shape, mean_ln: float, var: float, ell: float, seed: int, device="cuda"):
    """lognormal_k computed with torch on a device (same construction, torch's
    random stream: the values differ from the numpy version, the
    distribution does not).  Returns a flattened float64 tensor."""
    import torch

    sh = tuple(int(s) for s in shape[::-1])  # (nz, ny, nx)
    ext = tuple(2 * s for s in sh)
    axes = [torch.minimum(torch.arange(m, device=device), m - torch.arange(m, device=device)).double()
            for m in ext]
    grids = torch.meshgrid(*axes, indexing="ij")
    r = torch.sqrt(sum(g * g for g in grids))
    lam = torch.fft.fftn(var * torch.exp(-r / ell)).real.clamp_min(0.0)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    n = 1
    for m in ext:
        n *= m
    noise = torch.complex(torch.randn(ext, generator=gen, device=device, dtype=torch.float64),
                          torch.randn(ext, generator=gen, device=device, dtype=torch.float64))
    f = torch.fft.ifftn(torch.sqrt(lam / n) * noise * n).real
    f = f[tuple(slice(0, m) for m in sh)]
    return torch.exp(mean_ln + f).reshape(-1).contiguous()
