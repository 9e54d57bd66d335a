"""Seeded synthetic pressure fields and their material-acceleration inputs.

The benchmark cases are analytic pressure fields p; the solver input is a = -grad(p)/rho
(the reference integrates grad p = -rho a, K:1816) plus i.i.d. Gaussian noise of standard
deviation frac * max|grad p| per component.  Volumes are float32 with shape (nz, ny, nx).
"""
from __future__ import annotations

import numpy as np


def _grid(dims):
    nx, ny, nz = dims
    k, j, i = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    return i, j, k


def _finish(p, gx, gy, gz, rho, noise, seed, dims, spacing, mask=None, name=""):
    gmax = float(np.sqrt(gx * gx + gy * gy + gz * gz).max())
    rng = np.random.default_rng(seed)
    ax = -gx / rho
    ay = -gy / rho
    az = -gz / rho
    if noise > 0:
        s = noise * gmax / rho
        ax = ax + rng.normal(0.0, s, ax.shape)
        ay = ay + rng.normal(0.0, s, ay.shape)
        az = az + rng.normal(0.0, s, az.shape)
    nx, ny, nz = dims
    return {
        "name": name,
        "dims": (nx, ny, nz),
        "spacing": tuple(float(s) for s in spacing),
        "rho": float(rho),
        "ax": ax.astype(np.float32),
        "ay": ay.astype(np.float32),
        "az": az.astype(np.float32),
        "p_true": p,
        "mask": (np.ones(p.shape, np.float32) if mask is None else mask.astype(np.float32)),
    }


def gaussian(n=32, sigma_cells=6.0, spacing=1e-3, noise=0.05, seed=0, rho=1.0):
    """p = exp(-r^2 / (2 sigma^2)) centred in an n^3 grid."""
    dims = (n, n, n)
    i, j, k = _grid(dims)
    c = (n - 1) / 2.0
    X, Y, Z = (i - c) * spacing, (j - c) * spacing, (k - c) * spacing
    s = sigma_cells * spacing
    p = np.exp(-(X * X + Y * Y + Z * Z) / (2 * s * s))
    return _finish(p, -p * X / (s * s), -p * Y / (s * s), -p * Z / (s * s), rho, noise, seed, dims,
                   (spacing,) * 3, name="gaussian%d" % n)


def taylor_green(n=128, noise=0.10, seed=0, rho=1.0):
    """p = (cos 2x + cos 2y)(cos 2z + 2) / 16 on [0, 2 pi)^3."""
    dims = (n, n, n)
    h = 2 * np.pi / n
    i, j, k = _grid(dims)
    x, y, z = i * h, j * h, k * h
    A = np.cos(2 * x) + np.cos(2 * y)
    B = np.cos(2 * z) + 2
    p = A * B / 16.0
    gx = -2 * np.sin(2 * x) * B / 16.0
    gy = -2 * np.sin(2 * y) * B / 16.0
    gz = A * (-2 * np.sin(2 * z)) / 16.0
    return _finish(p, gx, gy, gz, rho, noise, seed, dims, (h, h, h), name="taylor_green%d" % n)


def blobs(n=256, count=8, sigma_range=(8.0, 24.0), noise=0.05, seed=0, rho=1.0, spacing=1e-3,
          sphere_radius=None, dims=None):
    """Sum of `count` Gaussian blobs (sigma ~ U[sigma_range] cells, amplitude ~ N(0,1)),
    optionally with a spherical obstacle of radius `sphere_radius` cells at the centre that
    is masked out (mask = 0)."""
    dims = tuple(dims) if dims is not None else (n, n, n)
    nx, ny, nz = dims
    rng = np.random.default_rng(seed + 1000)
    i, j, k = _grid(dims)
    p = np.zeros(i.shape)
    gx = np.zeros(i.shape)
    gy = np.zeros(i.shape)
    gz = np.zeros(i.shape)
    for _ in range(count):
        s = rng.uniform(*sigma_range)
        a = rng.normal(0.0, 1.0)
        c = rng.uniform(0.2, 0.8, 3) * (np.array(dims, np.float64) - 1)
        X, Y, Z = (i - c[0]) * spacing, (j - c[1]) * spacing, (k - c[2]) * spacing
        ss = (s * spacing) ** 2
        g = a * np.exp(-(X * X + Y * Y + Z * Z) / (2 * ss))
        p += g
        gx -= g * X / ss
        gy -= g * Y / ss
        gz -= g * Z / ss
    mask = None
    if sphere_radius is not None:
        cc = (np.array(dims, np.float64) - 1) / 2.0
        r = np.sqrt((i - cc[0]) ** 2 + (j - cc[1]) ** 2 + (k - cc[2]) ** 2)
        mask = (r > sphere_radius).astype(np.float32)
    return _finish(p, gx, gy, gz, rho, noise, seed, dims, (spacing,) * 3, mask=mask, name="blobs%d" % nx)


def vortex_ring(dims, ring_radius, centre, core=4.0, amplitude=1.0, noise=0.05, seed=0, rho=1.0, spacing=1e-3):
    """Low-pressure Gaussian core around a ring of radius `ring_radius` (cells) in the
    plane z = centre[2]: p = -A exp(-d^2 / (2 core^2)), d = distance to the ring."""
    i, j, k = _grid(dims)
    X, Y, Z = i - centre[0], j - centre[1], k - centre[2]
    rho_xy = np.sqrt(X * X + Y * Y) + 1e-12
    dr = rho_xy - ring_radius
    d2 = dr * dr + Z * Z
    p = -amplitude * np.exp(-d2 / (2 * core * core))
    # dp/dx_phys = dp/dd2 * dd2/dx / spacing
    f = p * (-1.0 / (2 * core * core))
    gx = f * 2 * dr * (X / rho_xy) / spacing
    gy = f * 2 * dr * (Y / rho_xy) / spacing
    gz = f * 2 * Z / spacing
    return _finish(p, gx, gy, gz, rho, noise, seed, dims, (spacing,) * 3, name="vortex_ring")


def batch_snapshots(count=64, lo=32, hi=160, seed=0, noise=0.05):
    """Snapshots of uneven seeded sizes (each dimension ~ U[lo, hi]) with a vortex ring whose
    radius and position vary per snapshot."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        dims = tuple(int(d) for d in rng.integers(lo, hi + 1, 3))
        m = min(dims[0], dims[1])
        R = rng.uniform(0.15, 0.3) * m
        c = np.array(dims, np.float64) / 2.0 + rng.uniform(-0.1, 0.1, 3) * np.array(dims)
        out.append(vortex_ring(dims, R, c, core=max(2.0, 0.06 * m), noise=noise, seed=seed * 1000 + s))
    return out


def relative_l2(p, q, gauge="mean", ref=None, weights=None) -> float:
    """Relative L2 difference of p against q after removing the constant (mean or the value
    at voxel index `ref`)."""
    p = np.asarray(p, np.float64).reshape(-1)
    q = np.asarray(q, np.float64).reshape(-1)
    sel = np.ones(p.shape, bool) if weights is None else np.asarray(weights).reshape(-1) > 0
    if gauge == "point":
        p = p - p[ref]
        q = q - q[ref]
    elif gauge == "mean":
        p = p - p[sel].mean()
        q = q - q[sel].mean()
    d = p[sel] - q[sel]
    n = np.linalg.norm(q[sel])
    return float(np.linalg.norm(d) / (n if n > 0 else 1.0))
