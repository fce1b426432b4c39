"""Errors against the FP64 oracle (oracle/_build/libwaporacle64.so: the same
restatement with every float quantity in double).  The GPU path equals the
FP32 oracle bit for bit (tests/test_gpu_parity.py) and the FP32 oracle equals
the reference's own code (tests/test_oracle_golden.py), so the FP32-vs-FP64
distances measured here are the product's and the reference's distances from
exact-in-double arithmetic.  Bounds: projections 1e-5 relative L2 with the same
sample counts, volumes 1e-4 and flows 1e-3 after two fixed-count outer
iterations (measured: 3.5e-6, 3.3e-5, 1.3e-4)."""
import numpy as np
import pytest

import oracle as O
import phantoms as P

N, W, H, NP = 32, 48, 48, 16


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def o64():
    return O.Oracle(fp64=True)


@pytest.fixture(scope="module")
def data(orc):
    vol = P.ellipsoids(N, seed=0)
    flow = P.rbf_flow(N, amp=2.0, seed=1)
    ang = P.golden_angles(NP)
    scan = O.make_scan((N, N, N), (W, H), NP, nframes_cli=2)
    return vol, flow, ang, scan


def test_fp64_oracle_is_double(o64, orc, data):
    vol, _, ang, scan = data
    img, _, _ = o64.forward(scan, ang[0], vol)
    assert img.dtype == np.float64 and orc.forward(scan, ang[0], vol)[0].dtype == np.float32


def test_projections_against_fp64(o64, orc, data):
    vol, _, ang, scan = data
    for a in ang[:6]:
        i32, l32, w32 = orc.forward(scan, a, vol)
        i64, l64, w64 = o64.forward(scan, a, vol)
        assert np.array_equal(w32, w64.astype(np.float32))  # sample counts
        assert rel(i32, i64) < 1e-5
        assert rel(l32, l64) < 1e-6


def test_warp_and_flow_level_against_fp64(o64, orc, data):
    vol, flow, _, _ = data
    aabb = np.array([0, N, 0, N, 0, N], np.float32)
    assert rel(orc.advect([N] * 3, aabb, flow, vol, 1.0), o64.advect([N] * 3, aabb, o64.arr(flow), o64.arr(vol), 1.0)) < 1e-5
    I1 = P.ellipsoids(N, seed=3)
    I2 = orc.advect([N] * 3, aabb, flow, I1, 1.0)
    out = []
    for o in (orc, o64):
        V = o.arr(flow * 0.3)
        Y = [o.arr(np.zeros((3, N, N, N))) for _ in range(3)] + [o.arr(np.zeros((N, N, N)))]
        o.flow_level([N] * 3, o.arr(I1), o.arr(I2), V, *Y, 0.0, 0.05, 120, 2, aabb, [4] * 6)
        out.append(V)
    assert rel(out[0], out[1]) < 1e-4


def test_outer_iterations_against_fp64(o64, orc, data):
    vol, _, ang, scan = data
    projs = np.stack([orc.forward(scan, a, vol)[0] for a in ang]).astype(np.float32)
    projs += np.random.default_rng(2).normal(scale=0.01 * projs.max(), size=projs.shape).astype(np.float32)
    scan.gmax = float(projs[0].max())
    sched = O.Schedule(n_cp=2, nb_sart=2, nb_projwarp=1, wp_frames=2, flow_tol=0.0, flow_lambda=0.05, flow_iters=60,
                       flow_warps=2, flow_eta=0.5, flow_sigma=0.8, flow_scales=2, cut=8, deterministic=1)
    states = []
    for o in (orc, o64):
        F = o.level_frames(2, NP, 0)[0]
        st = {k: o.arr(np.zeros((F,) + s)) for k, s in
              (("vols", (N, N, N)), ("flows", (3, N, N, N)), ("ytv", (3, N, N, N)), ("ytp", (N, N, N)),
               ("xbar", (N, N, N)), ("xprev", (N, N, N)))}
        for _ in range(2):
            o.outer_iteration(scan, sched, ang, o.arr(projs), 0, st)
        states.append(st)
    s32, s64 = states
    for f in range(len(s32["vols"])):
        assert rel(s32["vols"][f], s64["vols"][f]) < 1e-4, f
        if np.linalg.norm(s64["flows"][f]) > 0:
            assert rel(s32["flows"][f], s64["flows"][f]) < 1e-3, f
