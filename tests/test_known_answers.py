"""Analytic known answers of the path, checked on the oracle (which the GPU
path equals bit for bit, tests/test_gpu_parity.py): the ray length through a
ball is its chord; a ray's sample count is ceil(length / sample distance) + 1;
a constant volume projects to c * sd * count; a zero flow warps the interior
onto itself; CG recovers a known solution of the screened-Laplacian system."""
import numpy as np
import pytest

import oracle as O
import phantoms as P

N, W = 48, 72


@pytest.fixture(scope="module")
def scan():
    return O.make_scan((N, N, N), (W, W), 8)


@pytest.mark.parametrize("angle", [0.0, 33.3, 101.0, 245.7])
def test_sample_count_and_constant_volume(orc, scan, angle):
    sd = orc.lib.orc_sample_distance(1.0)
    img, ln, wt = orc.forward(scan, angle, np.full((N, N, N), 0.7, np.float32))
    hit = wt > 0
    assert hit.sum() > 1000
    count = np.ceil(ln[hit] / sd) + 1
    # the march re-derives t in float, so a ray whose length sits within an
    # ulp of a multiple of sd can take one sample more or less
    assert np.mean(wt[hit] == count) > 0.999 and np.max(np.abs(wt[hit] - count)) <= 1
    pred = 0.7 * sd * wt[hit]
    assert np.max(np.abs(img[hit] - pred) / pred) < 1e-5


def test_ball_chord(orc, scan):
    z, y, x = np.mgrid[0:N, 0:N, 0:N].astype(np.float32)
    c, r = (N - 1) / 2.0, 15.0
    ball = (((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) <= r * r).astype(np.float32)
    for angle in (0.0, 71.0):
        img, _, _ = orc.forward(scan, angle, ball)
        centre = img[W // 2 - 1:W // 2 + 1, W // 2 - 1:W // 2 + 1]
        assert np.all(np.abs(centre - 2 * r) < 0.5), centre


def test_zero_flow_warp_is_the_identity_inside(orc):
    src = P.ellipsoids(N, seed=1)
    aabb = np.array([0, N, 0, N, 0, N], np.float32)
    out = orc.advect([N] * 3, aabb, np.zeros((3, N, N, N), np.float32), src, 1.0)
    inner = (slice(2, N - 2),) * 3
    assert np.array_equal(out[inner], src[inner])


def test_cg_recovers_a_known_solution(orc):
    n = 24
    rng = np.random.default_rng(7)
    x_true = rng.standard_normal((n, n, n)).astype(np.float32)
    a, b = 1.0, 0.3
    xp = np.pad(x_true, 1, mode="edge")  # Neumann neighbours: the edge value
    sn = (xp[1:-1, 1:-1, :-2] + xp[1:-1, 1:-1, 2:] + xp[1:-1, :-2, 1:-1] + xp[1:-1, 2:, 1:-1] +
          xp[:-2, 1:-1, 1:-1] + xp[2:, 1:-1, 1:-1])
    rhs = (a * x_true - b * (sn - 6.0 * x_true)).astype(np.float32)
    x = np.zeros_like(rhs)
    its = orc.cg_screened_laplacian([n] * 3, a, b, rhs, x, rel_tol=1e-6, max_iters=500, abs_tol=1e-12, mode=0)
    assert 0 < its < 500
    assert np.linalg.norm(x - x_true) / np.linalg.norm(x_true) < 1e-4
