"""Seeded synthetic inputs shaped like the reference's workloads.

The reference publishes no datasets for this path (its copper-foam / bubble /
smoke scans are not distributed), so seeded phantoms stand in for them:
ellipsoid phantoms with smooth RBF deformations (the 64^3 CPU-runnable
workload) and a band-limited foam (the 256^3 workload).  Pure numpy.
"""
import numpy as np


def golden_angles(nproj):
    """Golden-ratio angle sequence in degrees, one per projection."""
    return (np.arange(nproj, dtype=np.float64) * 360.0 * 0.6180339887) % 360.0


def ellipsoids(n, count=20, seed=0):
    """n^3 float32 volume of `count` random ellipsoids (additive densities)."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pts = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float64)
    vol = np.zeros(n ** 3, np.float64)
    for _ in range(count):
        c = rng.uniform(0.15 * n, 0.85 * n, 3)
        ax = rng.uniform(3.0, 16.0, 3) * (n / 64.0)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, a, b, cc = q
        R = np.array([[1 - 2 * (b * b + cc * cc), 2 * (a * b - cc * w), 2 * (a * cc + b * w)],
                      [2 * (a * b + cc * w), 1 - 2 * (a * a + cc * cc), 2 * (b * cc - a * w)],
                      [2 * (a * cc - b * w), 2 * (b * cc + a * w), 1 - 2 * (a * a + b * b)]])
        d = (pts - c) @ R
        inside = ((d / ax) ** 2).sum(1) <= 1.0
        vol[inside] += rng.uniform(0.1, 1.0)
    return vol.reshape(n, n, n).astype(np.float32)


def rbf_flow(n, amp=3.0, sigma=12.0, count=8, seed=1):
    """Smooth 3-component displacement field (planar channels, shape (3,n,n,n))."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    f = np.zeros((3, n, n, n), np.float64)
    s = sigma * (n / 64.0)
    for _ in range(count):
        c = rng.uniform(0.2 * n, 0.8 * n, 3)
        v = rng.normal(size=3)
        g = np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
        for k in range(3):
            f[k] += v[k] * g
    m = np.abs(f).max()
    if m > 0:
        f *= amp / m
    return f.astype(np.float32)


def foam(n, seed=0, cutoff=1.0 / 16, pct=70.0):
    """Band-limited Gaussian noise thresholded at a percentile: 1 in struts, 0 in voids."""
    rng = np.random.default_rng(seed)
    w = rng.normal(size=(n, n, n))
    k = np.fft.fftfreq(n)
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    mask = (kx ** 2 + ky ** 2 + kz ** 2) <= cutoff ** 2
    b = np.real(np.fft.ifftn(np.fft.fftn(w) * mask))
    thr = np.percentile(b, pct)
    return (b > thr).astype(np.float32)
