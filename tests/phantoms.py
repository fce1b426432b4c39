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


# ---------------------------------------------------------------------------
# The 64^3 CPU-runnable workload, generated with arithmetic that gives the same
# bits on every machine: seeded integer-derived uniforms, and only IEEE-exact
# elementwise operations (+, -, *, /, sqrt, floor, ldexp; no BLAS, FFT or libm
# transcendental), so fixtures made on one host pin runs on another.
# ---------------------------------------------------------------------------
_LN2_HI = 6.93147180369123816490e-01
_LN2_LO = 1.90821492927058770002e-10


def det_exp(x):
    """exp(x) for float64 arrays x <= 0 from exact operations only: x = k ln2
    + r with |r| <= ln2 / 2, a degree-14 Taylor polynomial of r in Horner form,
    times 2^k (ldexp).  Relative error below 1e-15."""
    x = np.maximum(np.asarray(x, np.float64), -700.0)
    k = np.floor(x * (1.0 / 0.6931471805599453) + 0.5)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, 1.0)
    for n in range(14, 0, -1):
        p = p * r
        p = p / n
        p = p + 1.0
    return np.ldexp(p, k.astype(np.int64))


def _rotation(rng):
    """A uniform random rotation: a uniform point of the 4-ball (rejection
    sampling), normalised to a unit quaternion."""
    while True:
        q = rng.uniform(-1.0, 1.0, 4)
        s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]
        if 1e-6 < s <= 1.0:
            break
    w, a, b, c = q / np.sqrt(s)
    return np.array([[1 - 2 * (b * b + c * c), 2 * (a * b - c * w), 2 * (a * c + b * w)],
                     [2 * (a * b + c * w), 1 - 2 * (a * a + c * c), 2 * (b * c - a * w)],
                     [2 * (a * c - b * w), 2 * (b * c + a * w), 1 - 2 * (a * a + b * b)]])


def ellipsoid_params(n, count=20, seed=0):
    """Ellipsoids of the 64^3 workload: centres uniform in the central 70 % of
    the grid, semi-axes uniform in [3, 16] voxels (scaled by n / 64), uniform
    random rotations, densities uniform in [0.1, 1.0]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        c = rng.uniform(0.15 * n, 0.85 * n, 3)
        ax = rng.uniform(3.0, 16.0, 3) * (n / 64.0)
        R = _rotation(rng)
        out.append((c, ax, R, rng.uniform(0.1, 1.0)))
    return out


def rbf_params(n, count=8, sigma=12.0, amp=3.0, seed=1):
    """Gaussian RBF displacement of the 64^3 workload: `count` centres uniform
    in the central 60 %, directions uniform in [-1, 1]^3, width sigma (scaled
    by n / 64), normalised so the largest component on the grid is amp."""
    rng = np.random.default_rng(seed)
    cs = [rng.uniform(0.2 * n, 0.8 * n, 3) for _ in range(count)]
    vs = [rng.uniform(-1.0, 1.0, 3) for _ in range(count)]
    s = sigma * (n / 64.0)
    u = rbf_eval(n, cs, vs, s, 1.0)
    m = np.abs(u).max()
    return cs, vs, s, (amp / m if m > 0 else 0.0)


def rbf_eval(n, cs, vs, s, scale):
    """(3, n, n, n) float64 displacement of the RBF set at the voxel centres."""
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    u = np.zeros((3, n, n, n), np.float64)
    for c, v in zip(cs, vs):
        dx, dy, dz = x - c[0], y - c[1], z - c[2]
        g = det_exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * s * s))
        for k in range(3):
            u[k] = u[k] + g * v[k]
    return u * scale


def ellipsoids_at(n, ells, disp=None):
    """Float64 volume of the ellipsoids evaluated at x - disp(x) (the
    backward-mapped, analytically deformed phantom); disp (3, n, n, n) or None."""
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    if disp is not None:
        x, y, z = x - disp[0], y - disp[1], z - disp[2]
    vol = np.zeros((n, n, n), np.float64)
    for c, ax, R, dens in ells:
        px, py, pz = x - c[0], y - c[1], z - c[2]
        q = 0.0
        for j in range(3):
            dj = (px * R[0, j] + py * R[1, j]) + pz * R[2, j]
            dj = dj / ax[j]
            q = q + dj * dj
        vol = vol + np.where(q <= 1.0, dens, 0.0)
    return vol


def normal_irwin_hall(rng, shape):
    """Approximately standard normal samples as the sum of 12 uniforms minus 6
    (exact arithmetic, no libm)."""
    acc = np.zeros(shape, np.float64)
    for _ in range(12):
        acc = acc + rng.random(shape)
    return acc - 6.0


def deforming_scan_64(orc64, scan, n=64, nproj=64, seed=0):
    """Measured projections of the 64^3 workload: projection k sees the
    ellipsoid phantom deformed by t_k * u with t_k = k / nproj (the RBF field
    u, largest component 3 voxels), projected by the FP64 oracle projector,
    plus Gaussian noise of standard deviation 1 % of the largest value.
    orc64 is the FP64 oracle (test infrastructure).  Returns (projs float32
    (nproj, H, W), angles, undeformed phantom float32)."""
    ells = ellipsoid_params(n, seed=seed)
    cs, vs, s, scale = rbf_params(n, seed=seed + 1)
    ang = golden_angles(nproj)
    W, H = scan.det
    projs = np.zeros((nproj, H, W), np.float64)
    u1 = rbf_eval(n, cs, vs, s, 1.0)
    for k in range(nproj):
        t = k / float(nproj)
        vol_k = ellipsoids_at(n, ells, u1 * (scale * t))
        projs[k] = orc64.forward(scan, ang[k], vol_k)[0]
    rng = np.random.default_rng(seed + 2)
    projs = projs + normal_irwin_hall(rng, projs.shape) * (0.01 * projs.max())
    return projs.astype(np.float32), ang, ellipsoids_at(n, ells).astype(np.float32)
