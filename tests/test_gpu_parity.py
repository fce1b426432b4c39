"""GPU parity: every kernel of the C ABI against the CPU oracle on seeded inputs.

Integer/index results (sample counts, traversal) and every path whose
arithmetic is the reference's are compared bit for bit; the FP32-FMA variants
and the atomic splat are compared within the stated tolerances.
"""
import numpy as np
import pytest

import phantoms as P
from conftest import rel_l2

pytestmark = pytest.mark.gpu

N, W, H, NP = 32, 48, 48, 16


@pytest.fixture(scope="module")
def setup(wapmod, orc, torch_cuda):
    import oracle as O
    torch = torch_cuda
    vol = P.ellipsoids(N, seed=0)
    flow = P.rbf_flow(N, amp=2.0, seed=1)
    ang = P.golden_angles(NP)
    oscan = O.make_scan((N, N, N), (W, H), NP, nframes_cli=2)
    projs = np.stack([orc.forward(oscan, a, vol)[0] for a in ang]).astype(np.float32)
    projs += np.random.default_rng(2).normal(scale=0.01 * projs.max(), size=projs.shape).astype(np.float32)
    wscan = wapmod.make_scan((N, N, N), (W, H), NP, nframes_cli=2)
    ctx = wapmod.Context(wscan, ang)
    ctx.upload_projections(projs)
    oscan.gmax = ctx.gmax
    yield dict(torch=torch, ctx=ctx, vol=vol, flow=flow, ang=ang, oscan=oscan, projs=projs, O=O)
    ctx.close()


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def test_gmax_is_max_of_first_projection(setup):
    assert setup["ctx"].gmax == np.float32(setup["projs"][0].max())


def test_forward_projection_bitexact(setup, orc):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    dvol = dev(torch, s["vol"])
    for p in range(NP):
        img = torch.zeros((H, W), device="cuda")
        ln = torch.zeros_like(img)
        wt = torch.zeros_like(img)
        ctx.forward(p, dvol, img, ln, wt)
        ctx.synchronize()
        oi, ol, ow = orc.forward(s["oscan"], s["ang"][p], s["vol"])
        assert np.array_equal(host(wt), ow), "sample counts differ at projection %d" % p
        assert np.array_equal(host(ln), ol)
        assert np.array_equal(host(img), oi)


@pytest.mark.parametrize("n,bricks", [(32, 1), (37, 1), (37, 0)])
def test_forward_projection_brick_layout_bitexact(wapmod, orc, torch_cuda, n, bricks):
    """fp_bricks = 1 (the default): the projector reads a 4x4x4 brick-layout
    copy of the volume (a ragged size pads the last bricks); fp_bricks = 0:
    the linear volume.  Both give the oracle's bits."""
    import oracle as O
    torch = torch_cuda
    d = 48
    vol = P.ellipsoids(n, seed=6)
    ang = P.golden_angles(6)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (d, d), 6), ang)
    ctx.set_tuning("fp_bricks", bricks)
    oscan = O.make_scan((n, n, n), (d, d), 6)
    dvol = dev(torch, vol)
    try:
        for p in range(6):
            img = torch.zeros((d, d), device="cuda")
            ln, wt = torch.zeros_like(img), torch.zeros_like(img)
            ctx.forward(p, dvol, img, ln, wt)
            ctx.synchronize()
            oi, ol, ow = orc.forward(oscan, ang[p], vol)
            assert np.array_equal(host(wt), ow) and np.array_equal(host(ln), ol) and np.array_equal(host(img), oi), p
    finally:
        ctx.close()


def test_forward_projection_config0_size(wapmod, orc, torch_cuda):
    import oracle as O
    torch = torch_cuda
    n, d = 64, 96
    vol = P.ellipsoids(n, seed=4)
    ang = P.golden_angles(8)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (d, d), 8), ang)
    oscan = O.make_scan((n, n, n), (d, d), 8)
    dvol = dev(torch, vol)
    for p in (0, 3, 7):
        img = torch.zeros((d, d), device="cuda")
        wt = torch.zeros_like(img)
        ctx.forward(p, dvol, img, None, wt)
        ctx.synchronize()
        oi, _, ow = orc.forward(oscan, ang[p], vol)
        assert np.array_equal(host(wt), ow)
        assert np.array_equal(host(img), oi)
    ctx.close()


def test_correction_and_voxel_backprojection(setup, orc):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    rng = np.random.default_rng(7)
    p = 5
    meas = s["projs"][p]
    img, ln, _ = orc.forward(s["oscan"], s["ang"][p], s["vol"])
    dual = rng.normal(scale=0.1, size=(H, W)).astype(np.float32)
    odual = dual.copy()
    oc = orc.correction(meas, img, ln, odual, s["oscan"].alpha)
    dd = dev(torch, dual)
    dc = torch.zeros((H, W), device="cuda")
    ctx.correction(W * H, dev(torch, meas), dev(torch, img), dev(torch, ln), dd, dc)
    ctx.synchronize()
    assert np.array_equal(host(dc), oc)
    assert np.array_equal(host(dd), odual)
    box = [8, N - 8, 8, N - 8, 8, N - 8]
    for mode in (0, 1):
        base = (s["vol"] * 0.5).astype(np.float32) if mode == 0 else np.zeros_like(s["vol"])
        ov = orc.bp_voxel(s["oscan"], s["ang"][p], oc, box if mode == 0 else [0, N, 0, N, 0, N], mode, base.copy())
        for exact in (1, 0):
            dv = dev(torch, base)
            ctx.backproject_voxel(p, dc, box if mode == 0 else [0, N, 0, N, 0, N], mode, exact, dv)
            ctx.synchronize()
            if exact:
                assert np.array_equal(host(dv), ov), "exact BP mode %d" % mode
            else:
                assert rel_l2(host(dv), ov) < 1e-5, "fast BP mode %d" % mode


def test_ray_backprojection_matches_dead_path(setup, orc):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    corr = np.random.default_rng(5).normal(size=(H, W)).astype(np.float32)
    oc, ow = orc.ray_backproject(s["oscan"], s["ang"][4], corr)
    dcon = torch.zeros((N, N, N), device="cuda")
    dw = torch.zeros_like(dcon)
    ctx.backproject_ray(4, dev(torch, corr), dcon, dw)
    ctx.synchronize()
    # FP32 atomics reorder the sums (the reference's own += races under OpenMP).
    assert rel_l2(host(dcon), oc) < 1e-5
    assert rel_l2(host(dw), ow) < 1e-5


@pytest.mark.parametrize("n,det,nproj", [(48, 64, 12), (61, 80, 12)])
def test_ray_backprojection_every_angle_and_odd_grids(wapmod, orc, torch_cuda, n, det, nproj):
    """The shared-memory slab accumulation against the oracle's sequential
    splat on every projection of a scan (rays of all directions, grazing
    entries at the silhouette), on a grid whose width is a multiple of 4 (the
    float4 flush) and one that is not (the scalar flush)."""
    import oracle as O
    torch = torch_cuda
    ang = P.golden_angles(nproj)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (det, det), nproj), ang)
    try:
        oscan = O.make_scan((n, n, n), (det, det), nproj)
        rng = np.random.default_rng(n)
        for p in range(nproj):
            corr = rng.normal(size=(det, det)).astype(np.float32)
            oc, ow = orc.ray_backproject(oscan, ang[p], corr)
            dcon = torch.zeros((n, n, n), device="cuda")
            dw = torch.zeros_like(dcon)
            torch.cuda.synchronize()
            ctx.backproject_ray(p, dev(torch, corr), dcon, dw)
            ctx.synchronize()
            assert rel_l2(host(dw), ow) < 1e-5, "weights, projection %d" % p
            assert rel_l2(host(dcon), oc) < 1e-5, "contributions, projection %d" % p
    finally:
        ctx.close()


def test_ray_driven_sart_matches_oracle(setup, orc):
    """--bp Raybased: the SART proximal operator with the ray-driven matched
    backprojection and column-sum normalisation, against the oracle's
    restatement of the same update (within the reordering of the FP32 atomic
    sums)."""
    s = setup
    ctx = s["ctx"]
    ctx.level_setup(0)
    _, st, en, _, _ = orc.level_frames(2, NP, 0)
    v1 = (s["vol"] * 0.5).astype(np.float32)
    ctx.upload_volume(1, v1)
    ctx.set_tuning("bp_ray", 1)
    try:
        ctx.sart_prox(1, nb_sart=2, cut=8, exact=1)
    finally:
        ctx.set_tuning("bp_ray", 0)
    got = ctx.download_volume(1)
    ov, _ = orc.sart_prox_ray(s["oscan"], s["ang"], s["projs"], int(st[1]), int(en[1]), 2, [8, N - 8] * 3, v1.copy())
    assert rel_l2(got, ov) < 1e-5
    assert not np.array_equal(got, v1)


@pytest.mark.parametrize("dt,box", [(0.7, 1), (-1.0, 1), (-1.0, 2)])
def test_advect_bitexact(setup, orc, dt, box):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb = np.array([0, box * N, 0, box * N, 0, box * N], np.float32)
    src = np.stack([s["vol"], P.ellipsoids(N, seed=9)])
    out = torch.zeros((2, N, N, N), device="cuda")
    ctx.advect([N, N, N], aabb, dev(torch, s["flow"]), dev(torch, src), 2, dt, out)
    ctx.synchronize()
    ref = orc.advect([N, N, N], aabb, s["flow"], src.astype(np.float32), dt)
    assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("extreme", ["huge", "nan"])
def test_advect_bitexact_with_extreme_velocity(setup, orc, extreme):
    """A velocity field the cell-centre shortcut must not take (a component at
    or above 2^124, or a NaN): the warp falls back to the full clamped
    tricubic everywhere and still gives the oracle's result."""
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb = np.array([0, N, 0, N, 0, N], np.float32)
    flow = s["flow"].copy()
    flow[1, 3, 4, 5] = 3.0e37 if extreme == "huge" else np.nan
    out = torch.zeros((1, N, N, N), device="cuda")
    ctx.advect([N, N, N], aabb, dev(torch, flow), dev(torch, s["vol"]), 1, 0.7, out)
    ctx.synchronize()
    ref = orc.advect([N, N, N], aabb, flow, s["vol"], 0.7)
    assert np.array_equal(host(out), ref.reshape(1, N, N, N), equal_nan=True)


def test_packed_cubic_equals_scalar_cubic(setup):
    """The warp evaluates CImg's cubic two lanes at a time in packed FP32
    instructions; on 2^24 pseudo-random input pairs (any float bits,
    subnormals, signed zeros) it gives the scalar evaluation's bits, in the
    reference and the precision form's arithmetic."""
    assert setup["ctx"].check_packed_cubic(1 << 24, seed=12345) == 0


def test_blur_and_resize_bitexact(setup, orc):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    src = s["vol"]
    out = torch.zeros((N, N, N), device="cuda")
    ctx.blur([N, N, N], 1, 0.8, dev(torch, src), out)
    ctx.synchronize()
    assert np.array_equal(host(out), orc.blur([N, N, N], src, 0.8))
    for od in [(16, 16, 16), (64, 64, 64), (20, 40, 33), (32, 32, 16)]:
        o = torch.zeros((3, od[2], od[1], od[0]), device="cuda")
        ctx.resize([N, N, N], 3, dev(torch, s["flow"]), od, o)
        ctx.synchronize()
        assert np.array_equal(host(o), orc.resize([N, N, N], s["flow"], od)), od


def _flow_inputs(s, orc):
    aabb = np.array([0, N, 0, N, 0, N], np.float32)
    I1 = P.ellipsoids(N, seed=3)
    I2 = orc.advect([N] * 3, aabb, s["flow"], I1, 1.0)
    return aabb, I1, I2


@pytest.mark.parametrize("tol,iters,nwarps", [(0.0, 120, 2), (0.008, 3000, 1)])
def test_flow_level_bitexact(setup, orc, tol, iters, nwarps):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb, I1, I2 = _flow_inputs(s, orc)
    roi = [4] * 6
    V0 = (s["flow"] * 0.3).astype(np.float32)
    Y = [np.zeros((3, N, N, N), np.float32) for _ in range(3)] + [np.zeros((N, N, N), np.float32)]
    oV, oY = V0.copy(), [y.copy() for y in Y]
    tot, oits = orc.flow_level([N] * 3, I1, I2, oV, *oY, tol, 0.05, iters, nwarps, aabb, roi, deterministic=1)
    dV = dev(torch, V0)
    dY = [dev(torch, y) for y in Y]
    its = ctx.flow_level([N] * 3, dev(torch, I1), dev(torch, I2), dV, *dY, tol, 0.05, iters, nwarps, aabb, roi)
    assert list(its) == list(oits)
    assert np.array_equal(host(dV), oV)
    for a, b in zip(dY, oY):
        assert np.array_equal(host(a), b)


def _smooth_random(rng, shape, passes=3):
    a = rng.random(shape).astype(np.float32)
    for _ in range(passes):
        for ax in range(3):
            a = (a + np.roll(a, 1, ax) + np.roll(a, -1, ax)) / np.float32(3)
    return a.astype(np.float32)


@pytest.mark.parametrize("form,zchunk", [(1, 0), (1, 5), (2, 0), (2, 3), (3, 0), (3, 5)])
@pytest.mark.parametrize("dims", [(32, 32, 32), (37, 29, 23), (40, 27, 21)])
def test_flow_level_kernel_forms_bitexact(setup, orc, form, zchunk, dims):
    """Fused and primal+dual forms, default and odd z-chunks, on a grid whose
    sides are not multiples of the tile: every form matches the oracle bit for
    bit through residual (50, 100) and Kty-store (49, 99) iterations."""
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    nx, ny, nz = dims
    rng = np.random.default_rng(11)
    I1 = _smooth_random(rng, (nz, ny, nx))
    I2 = _smooth_random(rng, (nz, ny, nx))
    V0 = (rng.normal(size=(3, nz, ny, nx)) * 0.7).astype(np.float32)
    Y = [np.zeros((3, nz, ny, nx), np.float32) for _ in range(3)] + [np.zeros((nz, ny, nx), np.float32)]
    aabb = np.array([0, nx, 0, ny, 0, nz], np.float32)
    roi = [3, 4, 2, 5, 1, 3]
    oV, oY = V0.copy(), [y.copy() for y in Y]
    _, oits = orc.flow_level(list(dims), I1, I2, oV, *oY, 0.0, 0.05, 120, 2, aabb, roi, deterministic=1)
    dV = dev(torch, V0)
    dY = [dev(torch, y) for y in Y]
    ctx.set_tuning("pd_form", form)
    ctx.set_tuning("pd_zchunk", zchunk)
    try:
        its = ctx.flow_level(list(dims), dev(torch, I1), dev(torch, I2), dV, *dY, 0.0, 0.05, 120, 2, aabb, roi)
        assert ctx.get_tuning(list(dims)) == (form, zchunk)  # form 3 falls back to 2 when nx % 4 != 0
    finally:
        ctx.set_tuning("pd_form", 0)
        ctx.set_tuning("pd_zchunk", 0)
    assert list(its) == list(oits)
    assert np.array_equal(host(dV), oV)
    for a, b in zip(dY, oY):
        assert np.array_equal(host(a), b)


def test_flow_level_autotuned_plan(setup):
    """The autotuner records a valid plan for a grid after its first level."""
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    dims = (40, 24, 20)
    rng = np.random.default_rng(12)
    I1 = _smooth_random(rng, dims[::-1])
    I2 = _smooth_random(rng, dims[::-1])
    V = torch.zeros((3,) + dims[::-1], device="cuda")
    Y = [torch.zeros((3,) + dims[::-1], device="cuda") for _ in range(3)] + [torch.zeros(dims[::-1], device="cuda")]
    aabb = np.array([0, dims[0], 0, dims[1], 0, dims[2]], np.float32)
    ctx.flow_level(list(dims), dev(torch, I1), dev(torch, I2), V, *Y, 0.0, 0.05, 10, 1, aabb, [2] * 6)
    form, zchunk = ctx.get_tuning(list(dims))
    assert form in (1, 2, 3) and 1 <= zchunk <= dims[2]


def test_flow_multiscale_bitexact(setup, orc):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb, I1, I2 = _flow_inputs(s, orc)
    V0 = (s["flow"] * 0.5).astype(np.float32)
    ov, otot = orc.flow_multiscale([N] * 3, I1, I2, V0, 0.0, 0.05, 60, 2, 0.5, 0.8, 3, [8] * 6)
    out = torch.zeros((3, N, N, N), device="cuda")
    tot = ctx.flow_multiscale([N] * 3, dev(torch, I1), dev(torch, I2), dev(torch, V0), 0.0, 0.05, 60, 2, 0.5, 0.8,
                              3, [8] * 6, out)
    assert tot == otot
    assert np.array_equal(host(out), ov)


@pytest.mark.parametrize("exact", [1, 0])
def test_sart_prox(setup, orc, exact):
    s = setup
    ctx, O = s["ctx"], s["O"]
    nf = ctx.level_setup(0)
    onf, st, en, ft, tu = orc.level_frames(2, NP, 0)
    assert nf == onf
    v1 = (s["vol"] * 0.5).astype(np.float32)
    ctx.upload_volume(1, v1)
    ctx.sart_prox(1, nb_sart=2, cut=8, exact=exact)
    got = ctx.download_volume(1)
    ov, _ = orc.sart_prox(s["oscan"], s["ang"], s["projs"], int(st[1]), int(en[1]), 2, [8, N - 8] * 3, v1.copy())
    if exact:
        assert np.array_equal(got, ov)
    else:
        assert rel_l2(got, ov) < 1e-4


def test_warp_and_project_bitexact(setup, orc):
    s = setup
    ctx = s["ctx"]
    ctx.level_setup(0)
    _, st, en, ft, tu = orc.level_frames(2, NP, 0)
    v1 = (s["vol"] * 0.5).astype(np.float32)
    fl0 = (s["flow"] * 0.7).astype(np.float32)
    ctx.upload_volume(1, v1)
    ctx.upload_flow(0, fl0)
    cur = v1.copy()
    for ik, rt in [(int(st[1]), -0.6), (int(en[1]), 0.9)]:
        ctx.warp_and_project(1, ik, rt, exact=1)
        fwd = fl0 if rt < 0 else np.zeros_like(fl0)
        cur = orc.warp_and_project(s["oscan"], s["ang"], s["projs"], ik, rt, fwd, fl0, cur.copy())
        assert np.array_equal(ctx.download_volume(1), cur)


def test_adaptive_warp_bitexact(setup, orc):
    """AdaptiveWarp (the reference's commented-out per-frame warp sweep,
    WaP_Tomo.cpp:878-1204) on frame 2 with two sweeps, against the oracle."""
    s = setup
    ctx = s["ctx"]
    F = ctx.level_setup(1)  # the second time level: 4 frames
    assert F >= 3
    _, st, en, ft, tu = orc.level_frames(2, NP, 1)
    f = 2
    v = (s["vol"] * 0.6).astype(np.float32)
    fl1 = (s["flow"] * 0.5).astype(np.float32)
    fl0 = (s["flow"] * -0.4).astype(np.float32)
    ctx.upload_volume(f, v)
    ctx.upload_flow(f - 1, fl1)
    ctx.upload_flow(f - 2, fl0)
    ctx.adaptive_warp(f, nb_warp=2, cut=8, exact=1)
    want = orc.adaptive_warp(s["oscan"], s["ang"], s["projs"], int(st[f]), int(en[f]), float(ft[f]), float(tu), 2,
                             [8, N - 8] * 3, fl1, fl0, v.copy())
    got = ctx.download_volume(f)
    assert np.array_equal(got, want)
    assert not np.array_equal(got, v)


def test_outer_iteration_bitexact(setup, orc, wapmod):
    s = setup
    ctx, O = s["ctx"], s["O"]
    F = ctx.level_setup(0)
    sched_o = O.Schedule(n_cp=2, nb_sart=2, nb_projwarp=1, wp_frames=2, flow_tol=0.0, flow_lambda=0.05,
                         flow_iters=60, flow_warps=2, flow_eta=0.5, flow_sigma=0.8, flow_scales=2, cut=8,
                         deterministic=1)
    sched_w = wapmod.reference_schedule(n_cp=2, nb_sart=2, wp_frames=2, flow_iters=60, flow_scales=2, flow_tol=0.0,
                                        flow_warps=2)
    state = dict(vols=np.zeros((F, N, N, N), np.float32), flows=np.zeros((F, 3, N, N, N), np.float32),
                 ytv=np.zeros((F, 3, N, N, N), np.float32), ytp=np.zeros((F, N, N, N), np.float32),
                 xbar=np.zeros((F, N, N, N), np.float32), xprev=np.zeros((F, N, N, N), np.float32))
    for it in range(2):
        st = ctx.outer_iteration(sched_w)
        orc.outer_iteration(s["oscan"], sched_o, s["ang"], s["projs"], 0, state)
        for f in range(F):
            assert np.array_equal(ctx.download_volume(f), state["vols"][f]), (it, f)
            assert np.array_equal(ctx.download_flow(f), state["flows"][f]), (it, f)
        assert st.kernel_launches > 0


def test_outer_iteration_steps_equal_the_whole(setup, wapmod):
    """The step decomposition (CP iterations, flow pairs, WaP pass) run in
    order gives the outer iteration's bits, with and without an observer."""
    s = setup
    ctx = s["ctx"]
    sched = wapmod.reference_schedule(n_cp=2, nb_sart=2, wp_frames=2, flow_iters=40, flow_scales=2, flow_tol=0.0,
                                      flow_warps=2)
    F = ctx.level_setup(0)
    ctx.outer_iteration(sched)
    whole = [ctx.download_volume(f) for f in range(F)], [ctx.download_flow(f) for f in range(F)]
    events = []
    ctx.set_observer(lambda ev, lvl, a, b, d: events.append((ev, a, b)))
    try:
        F2 = ctx.level_setup(0)
        n = ctx.outer_iteration_nsteps(sched)
        assert F2 == F and n == 2 + (F - 1) + 1
        for k in range(n):
            ctx.outer_iteration_step(sched, k)
    finally:
        ctx.set_observer(None)
    for f in range(F):
        assert np.array_equal(ctx.download_volume(f), whole[0][f])
        assert np.array_equal(ctx.download_flow(f), whole[1][f])
    assert [e for e in events if e[0] == wapmod.WAP_EV_SART] == [(1, f, c) for c in (1, 2) for f in range(F)]
    assert [e[1] for e in events if e[0] == wapmod.WAP_EV_FLOW] == list(range(F - 1))
    assert len([e for e in events if e[0] == wapmod.WAP_EV_WARP]) > 0


def test_flow_lanes_give_the_same_outer_iteration(wapmod, orc, torch_cuda):
    """An outer iteration's flow pairs run concurrently on helper lanes
    (flow_lanes 2, 3, 4 and the automatic choice, 4 at this size) or one
    after another (1): the same volumes, flows and primal-dual iteration
    counts bit for bit, on a 6-frame scan (5 pairs), with the 0.008 tolerance
    so that levels stop early."""
    import oracle as O
    n, d, nproj = 32, 48, 24
    vol = P.ellipsoids(n, seed=21)
    ang = P.golden_angles(nproj)
    oscan = O.make_scan((n, n, n), (d, d), nproj, nframes_cli=6)
    projs = np.stack([orc.forward(oscan, a, vol)[0] for a in ang]).astype(np.float32)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (d, d), nproj, nframes_cli=6), ang)
    try:
        ctx.upload_projections(projs)
        sched = wapmod.reference_schedule(n_cp=2, nb_sart=2, wp_frames=6, flow_iters=120, flow_scales=2,
                                          flow_tol=0.008, flow_warps=2)
        got = {}
        for lanes in (1, 2, 3, 4, 0):
            ctx.set_tuning("flow_lanes", lanes)
            F = ctx.level_setup(0)
            assert F == 6
            st = ctx.outer_iteration(sched)
            got[lanes] = ([ctx.download_volume(f) for f in range(F)], [ctx.download_flow(f) for f in range(F)],
                          int(st.flow_pd_iterations))
        for lanes in (2, 3, 4, 0):
            assert got[lanes][2] == got[1][2]
            for f in range(6):
                assert np.array_equal(got[lanes][0][f], got[1][0][f]), (lanes, f)
                assert np.array_equal(got[lanes][1][f], got[1][1][f]), (lanes, f)
    finally:
        ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_cg_screened_laplacian(setup, orc, mode):
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    rhs = np.random.default_rng(3).normal(size=(N, N, N)).astype(np.float32)
    xo = np.zeros_like(rhs)
    oit = orc.cg_screened_laplacian([N] * 3, 1.0, 0.5, rhs, xo, 1e-5, 200, 1e-9, mode)
    dx = torch.zeros((N, N, N), device="cuda")
    it = ctx.cg_screened_laplacian([N] * 3, 1.0, 0.5, dev(torch, rhs), dx, 1e-5, 200, 1e-9, mode)
    assert abs(it - oit) <= 2
    assert rel_l2(host(dx), xo) < 1e-4


def test_precision_form_fp16_flow_state(setup, orc, wapmod):
    """The precision form (flow solver state as FP16 pairs; FP32 arithmetic
    with fused multiply-adds and hardware reciprocals in the primal-dual
    iteration, float pyramid growth, fused-multiply-add warps): same iteration
    counts at a fixed count, the flow within 2e-2 relative L2 of the exact FP32
    path, and an outer iteration's volumes within 1e-3 relative L2 of the FP32
    oracle and of the FP64 oracle."""
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb, I1, I2 = _flow_inputs(s, orc)
    V0 = (s["flow"] * 0.3).astype(np.float32)
    out = {}
    try:
        for bits in (32, 16):
            ctx.set_tuning("flow_bits", bits)
            dV = dev(torch, V0)
            dY = [torch.zeros((3, N, N, N), device="cuda") for _ in range(3)] + [torch.zeros((N, N, N), device="cuda")]
            its = ctx.flow_level([N] * 3, dev(torch, I1), dev(torch, I2), dV, *dY, 0.0, 0.05, 200, 2, aabb, [4] * 6)
            out[bits] = (host(dV), list(its))
        assert out[16][1] == out[32][1]
        assert rel_l2(out[16][0], out[32][0]) < 2e-2
        # an outer iteration with the precision form against the FP32 oracle
        import oracle as O
        F = ctx.level_setup(0)
        sched_w = wapmod.reference_schedule(n_cp=2, nb_sart=2, wp_frames=2, flow_iters=60, flow_scales=2,
                                            flow_tol=0.0, flow_warps=2)
        ctx.outer_iteration(sched_w)
        sched_o = O.Schedule(n_cp=2, nb_sart=2, nb_projwarp=1, wp_frames=2, flow_tol=0.0, flow_lambda=0.05,
                             flow_iters=60, flow_warps=2, flow_eta=0.5, flow_sigma=0.8, flow_scales=2, cut=8,
                             deterministic=1)
        state = dict(vols=np.zeros((F, N, N, N), np.float32), flows=np.zeros((F, 3, N, N, N), np.float32),
                     ytv=np.zeros((F, 3, N, N, N), np.float32), ytp=np.zeros((F, N, N, N), np.float32),
                     xbar=np.zeros((F, N, N, N), np.float32), xprev=np.zeros((F, N, N, N), np.float32))
        orc.outer_iteration(s["oscan"], sched_o, s["ang"], s["projs"], 0, state)
        # and against the FP64 oracle (the same algorithm in double)
        o64 = O.Oracle(fp64=True)
        state64 = {k: v.astype(np.float64) * 0 for k, v in state.items()}
        o64.outer_iteration(s["oscan"], sched_o, s["ang"], o64.arr(s["projs"]), 0, state64)
        for f in range(F):
            got = ctx.download_volume(f)
            assert rel_l2(got, state["vols"][f]) < 1e-3
            assert rel_l2(got, state64["vols"][f]) < 1e-3
    finally:
        ctx.set_tuning("flow_bits", 32)


def test_precision_form_stops_like_fp32(setup, orc, wapmod):
    """With the reference's tolerance (0.008) the precision form's flow level
    stops before its iteration cap as the exact FP32 path does, at a nearby
    iteration: its residual compares the stored FP16 states (the dual sees the
    new flow as stored), so FP16 rounding alone does not hold it above the
    tolerance."""
    s = setup
    torch, ctx = s["torch"], s["ctx"]
    aabb, I1, I2 = _flow_inputs(s, orc)
    V0 = (s["flow"] * 0.3).astype(np.float32)
    cap = 3000
    its = {}
    try:
        for bits in (32, 16):
            ctx.set_tuning("flow_bits", bits)
            dV = dev(torch, V0)
            dY = [torch.zeros((3, N, N, N), device="cuda") for _ in range(3)] + [torch.zeros((N, N, N), device="cuda")]
            its[bits] = list(ctx.flow_level([N] * 3, dev(torch, I1), dev(torch, I2), dV, *dY, 0.008, 0.05, cap, 2,
                                            aabb, [4] * 6))
    finally:
        ctx.set_tuning("flow_bits", 32)
    print("iterations per warp: FP32", its[32], "FP16", its[16])
    for w in range(2):
        assert its[32][w] < cap, its
        assert its[16][w] < cap, its
        assert abs(its[16][w] - its[32][w]) <= max(100, its[32][w] // 4), its


def test_precision_form_projector(setup, orc):
    """The precision form's SART step: the forward projector reads an FP16
    brick-layout copy of the volume and sums each ray with Kahan's
    compensation in FP32 (sample counts unchanged); the FP32 volumes take
    the updates.  Two sweeps stay within 1e-4 relative L2 of the reference
    arithmetic (the oracle)."""
    s = setup
    ctx = s["ctx"]
    ctx.level_setup(0)
    _, st, en, _, _ = orc.level_frames(2, NP, 0)
    v1 = (s["vol"] * 0.5).astype(np.float32)
    ctx.upload_volume(1, v1)
    ctx.set_tuning("flow_bits", 16)
    try:
        ctx.sart_prox(1, nb_sart=2, cut=8, exact=1)
    finally:
        ctx.set_tuning("flow_bits", 32)
    got = ctx.download_volume(1)
    ov, _ = orc.sart_prox(s["oscan"], s["ang"], s["projs"], int(st[1]), int(en[1]), 2, [8, N - 8] * 3, v1.copy())
    err = rel_l2(got, ov)
    assert 0 < err < 1e-4, err
