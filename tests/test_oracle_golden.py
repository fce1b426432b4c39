"""The CPU oracle against golden fixtures produced by the reference's own code.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs
the reference's sources (compiled headless into oracle/_ref) on seeded
inputs.  Every comparison is bit-exact: the oracle restates the reference's
float arithmetic operation for operation.
"""
import os

import numpy as np
import pytest

import oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(G, name + ".npz")))


@pytest.fixture(scope="module")
def ps():
    return load("projector_solver")


@pytest.fixture(scope="module")
def fc():
    return load("flow_components")


def _scan(d, nframes=2, gmax=1.0):
    N, _, W, H, NP = [int(v) for v in d["dims"]]
    return O.make_scan((N, N, N), (W, H), NP, nframes_cli=nframes, gmax=float(gmax))


def test_forward_projection(orc, ps):
    scan = _scan(ps)
    for p, a in enumerate(ps["angles"]):
        img, ln, wt = orc.forward(scan, a, ps["vol"])
        assert np.array_equal(wt, ps["weight"][p]), p
        assert np.array_equal(ln, ps["len"][p]), p
        assert np.array_equal(img, ps["img"][p]), p


def test_ray_backprojection_dead_path(orc, ps):
    c, w = orc.ray_backproject(_scan(ps), ps["angles"][3], ps["corr"])
    assert np.array_equal(c, ps["raybp_contrib"])
    assert np.array_equal(w, ps["raybp_weight"])


def test_sart_proximal_operator(orc, ps):
    scan = _scan(ps, gmax=ps["gmax"])
    N = scan.vol[0]
    st, en = [int(v) for v in ps["sart_window"]]
    out, _ = orc.sart_prox(scan, ps["angles"], ps["projs"], st, en, 2, [8, N - 8] * 3, ps["sart_in"].copy())
    assert np.array_equal(out, ps["sart_out"])


def test_warp_and_project(orc, ps):
    scan = _scan(ps, gmax=ps["gmax"])
    v = ps["sart_out"].copy()
    fl0 = ps["wap_flow0"]
    for ik, rt in ps["wap_steps"]:
        fwd = fl0 if rt < 0 else np.zeros_like(fl0)
        v = orc.warp_and_project(scan, ps["angles"], ps["projs"], int(ik), float(rt), fwd, fl0, v.copy())
    assert np.array_equal(v, ps["wap_out"])


def test_advect_blur_resize_gradient(orc, fc):
    N = fc["I1"].shape[0]
    aabb = [0, N, 0, N, 0, N]
    assert np.array_equal(orc.advect([N] * 3, aabb, fc["flow"], fc["I1"], 1.0), fc["I2"])
    assert np.array_equal(orc.advect([N] * 3, [0, 2 * N] * 3, fc["flow"], fc["I1"], -0.7), fc["advect_box2"])
    assert np.array_equal(orc.blur([N] * 3, fc["I1"], 0.8), fc["blur"])
    assert np.array_equal(orc.resize([N] * 3, fc["flow"], (10, 10, 10)), fc["resize_down"])
    assert np.array_equal(orc.resize([N] * 3, fc["flow"], (40, 27, 30)), fc["resize_up"])
    for g, k in zip(orc.gradient([N] * 3, fc["I1"]), ("gx", "gy", "gz")):
        assert np.array_equal(g, fc[k])


def test_flow_level_and_multiscale(orc, fc):
    N = fc["I1"].shape[0]
    aabb = [0, N, 0, N, 0, N]
    V = (fc["flow"] * 0.3).astype(np.float32)
    Y = [np.zeros((3, N, N, N), np.float32) for _ in range(3)] + [np.zeros((N, N, N), np.float32)]
    orc.flow_level([N] * 3, fc["I1"], fc["I2"], V, *Y, 0.0, 0.05, 40, 2, aabb, [3] * 6, deterministic=1)
    assert np.array_equal(V, fc["level_V"])
    for y, k in zip(Y, ("level_Y1", "level_Y2", "level_Y3", "level_Y4")):
        assert np.array_equal(y, fc[k])
    out, _ = orc.flow_multiscale([N] * 3, fc["I1"], fc["I2"], (fc["flow"] * 0.5).astype(np.float32), 0.0, 0.05, 25,
                                 2, 0.5, 0.8, 2, [4] * 6)
    assert np.array_equal(out, fc["multiscale_V"])


def test_cg_reference_update_rule(orc, fc):
    N = fc["cg_rhs"].shape[0]
    x = np.zeros_like(fc["cg_rhs"])
    orc.cg_screened_laplacian([N] * 3, 1.0, 0.5, fc["cg_rhs"], x, 1e-5, 60, 1e-9, mode=1)
    assert np.array_equal(x, fc["cg_x"])


def test_full_render_two_levels(orc):
    """PSART::Render end to end: CP prior, SART, 5-level flow with the 0.008
    tolerance, warp-and-project, over two time levels."""
    d = load("render")
    N, _, W, H, NP = [int(v) for v in d["dims"]]
    scan = O.make_scan((N, N, N), (W, H), NP, nframes_cli=1, gmax=float(d["gmax"]))

    def fresh(F):
        return dict(vols=np.zeros((F, N, N, N), np.float32), flows=np.zeros((F, 3, N, N, N), np.float32),
                    ytv=np.zeros((F, 3, N, N, N), np.float32), ytp=np.zeros((F, N, N, N), np.float32),
                    xbar=np.zeros((F, N, N, N), np.float32), xprev=np.zeros((F, N, N, N), np.float32))

    sched = O.Schedule(n_cp=2, nb_sart=2, nb_projwarp=1, wp_frames=1, flow_tol=0.008, flow_lambda=0.05,
                       flow_iters=3000, flow_warps=3, flow_eta=0.5, flow_sigma=0.8, flow_scales=5, cut=8,
                       deterministic=1)
    s0 = fresh(1)
    orc.outer_iteration(scan, sched, d["angles"], d["projs"], 0, s0)
    s1 = fresh(2)
    s1["vols"][0] = s0["vols"][0]
    s1["vols"][1] = s0["vols"][0]
    sched.n_cp = 10
    orc.outer_iteration(scan, sched, d["angles"], d["projs"], 1, s1)
    assert np.array_equal(s1["vols"][0], d["level1_vol0"])
    assert np.array_equal(s1["vols"][1], d["level1_vol1"])
    assert np.array_equal(s1["flows"][0], d["level1_flow0"])
