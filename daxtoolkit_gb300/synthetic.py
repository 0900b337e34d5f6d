"""Seeded synthetic point fields on the unit cube (no datasets are shipped).

* ``sphere_field``: ||p - (0.5, 0.5, 0.5)|| + amp * U(-1, 1) noise (the 64^3
  sphere case).
* ``blob_field``: sum of isotropic Gaussian blobs, amplitude 1,
  f(p) = sum_b exp(-||p - c_b||^2 / (2 sigma_b^2)), evaluated per axis as the
  product exp(-(x - cx)^2/(2s^2)) exp(-(y - cy)^2/(2s^2)) exp(-(z - cz)^2/(2s^2))
  (mathematically the same function), centres U[0.1, 0.9]^3 and sigma
  U[0.05, 0.15] drawn from numpy's PCG64 with the given seed; optional
  uniform noise.

Coordinates are i / (n - 1) per axis.  Generation runs in float64 with torch on
the requested device and is cast to float32 once; the returned tensor is the
single copy of the field that every consumer (GPU kernels, CPU baselines via a
host copy) reads.
"""
import numpy as np
import torch


def blob_params(nblobs, seed):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.1, 0.9, size=(nblobs, 3))
    sigmas = rng.uniform(0.05, 0.15, size=nblobs)
    return centres, sigmas


def _axis(n, device):
    return torch.arange(n, dtype=torch.float64, device=device) / max(n - 1, 1)


def blob_field(dims, nblobs=8, seed=20260101, noise=0.0, device="cpu"):
    nx, ny, nz = dims
    centres, sigmas = blob_params(nblobs, seed)
    x, y, z = _axis(nx, device), _axis(ny, device), _axis(nz, device)
    out = torch.zeros((nz, ny, nx), dtype=torch.float32, device=device)
    for b in range(nblobs):
        s2 = 2.0 * sigmas[b] ** 2
        gx = torch.exp(-(x - centres[b, 0]) ** 2 / s2)
        gy = torch.exp(-(y - centres[b, 1]) ** 2 / s2)
        gz = torch.exp(-(z - centres[b, 2]) ** 2 / s2)
        for k0 in range(0, nz, 64):  # bounded temporaries
            k1 = min(nz, k0 + 64)
            out[k0:k1] += (gz[k0:k1, None, None] * gy[None, :, None] * gx[None, None, :]).float()
    if noise:
        g = torch.Generator(device="cpu").manual_seed(seed + 1)
        out += (noise * (2 * torch.rand((nz, ny, nx), generator=g) - 1)).to(device)
    return out.reshape(-1).contiguous()


def sphere_field(dims, noise=0.01, seed=1234, device="cpu"):
    nx, ny, nz = dims
    x, y, z = _axis(nx, "cpu"), _axis(ny, "cpu"), _axis(nz, "cpu")
    r = torch.sqrt((x[None, None, :] - 0.5) ** 2 + (y[None, :, None] - 0.5) ** 2 +
                   (z[:, None, None] - 0.5) ** 2)
    g = torch.Generator(device="cpu").manual_seed(seed)
    f = r + noise * (2 * torch.rand((nz, ny, nx), generator=g, dtype=torch.float64) - 1)
    return f.float().reshape(-1).contiguous().to(device)


def batch_grid_dims(count, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return [tuple(int(v) for v in rng.integers(lo, hi + 1, size=3)) for _ in range(count)]


def batch_isovalues(count, lo, hi, seed):
    rng = np.random.default_rng(seed + 7)
    return [float(v) for v in rng.uniform(lo, hi, size=count)]
