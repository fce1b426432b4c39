"""GPU parity at the benchmark's own configurations.

* The 64^3 CPU-runnable workload end to end: three outer iterations of
  PSART's schedule (5 CP x 2 SART, a 3-level flow at 3000 primal-dual
  iterations per warp and level, 3 warps, warp-and-project over every window)
  through wap_outer_iteration, compared bit for bit with SHA-256 digests that
  the oracle computed for every frame's volume and flow
  (tests/golden/make_config0.py); the inputs are regenerated here with
  bit-reproducible arithmetic and their digest checked first.
* The 256^3 x 384^2 workload's kernels at full size: forward projections,
  the reference's double-arithmetic backprojection, a warp, the primal-dual
  kernel in every form and z-chunk (the autotuned plan included), and one
  frame's share of an outer iteration on the benchmark's schedule (shortened
  flow) against the oracle bit for bit.
* The precision form at 256^3 against the FP64 oracle.
* The CP prior kernels alone against the oracle.
* The projector at the precision configuration's size (512^3 -> 768^2).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import phantoms as P
from conftest import rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


# ---------------------------------------------------------------------------
# 64^3 workload, three full outer iterations
# ---------------------------------------------------------------------------
def test_config0_outer_iterations_match_oracle_digests(wapmod, torch_cuda):
    import oracle as O
    path = os.path.join(HERE, "golden", "config0_digests.json")
    with open(path) as f:
        rec = json.load(f)
    n, det, nproj, F = rec["volume"], rec["detector"], rec["projections"], rec["frames"]
    oscan = O.make_scan((n, n, n), (det, det), nproj, nframes_cli=F)
    projs, ang, _ = P.deforming_scan_64(O.Oracle(fp64=True), oscan, n=n, nproj=nproj)
    assert sha(projs) == rec["inputs_sha256"], "the regenerated inputs differ from the ones the digests were made on"
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (det, det), nproj, nframes_cli=F), ang)
    try:
        ctx.upload_projections(projs)
        assert ctx.gmax == np.float32(rec["gmax"])
        assert ctx.level_setup(0) == F
        s = rec["schedule"]
        sched = wapmod.reference_schedule(n_cp=s["n_cp"], nb_sart=s["nb_sart"], wp_frames=s["wp_frames"],
                                          flow_iters=s["flow_iters"], flow_scales=s["flow_scales"],
                                          flow_tol=s["flow_tol"], cut=s["cut"], bp_exact=1,
                                          flow_warps=s["flow_warps"])
        for it, want in enumerate(rec["iterations"]):
            st = ctx.outer_iteration(sched)
            assert st.flow_pd_iterations == want["pd_iterations"]
            for f in range(F):
                v, fl = ctx.download_volume(f), ctx.download_flow(f)
                assert sha(v) == want["volumes"][f], "outer iteration %d frame %d volume: sum %.9g, oracle %.9g" % (
                    it + 1, f, v.astype(np.float64).sum(), want["volume_sums"][f])
                assert sha(fl) == want["flows"][f], "outer iteration %d frame %d flow: |sum| %.9g, oracle %.9g" % (
                    it + 1, f, np.abs(fl.astype(np.float64)).sum(), want["flow_abs_sums"][f])
    finally:
        ctx.close()


# ---------------------------------------------------------------------------
# 256^3 x 384^2 workload
# ---------------------------------------------------------------------------
N2, D2, NP2, F2 = 256, 384, 192, 3
FRAME = 1  # the frame whose share of the outer iteration is run


def _compress_flow(n, seed=1):
    """The benchmark's deformation per unit time: u_z = -0.25 (z - n/2) plus a
    smooth RBF perturbation (largest component 6 voxels)."""
    u = P.rbf_flow(n, amp=6.0, sigma=12.0, seed=seed)
    z = np.arange(n, dtype=np.float32).reshape(n, 1, 1)
    u[2] += -0.25 * (z - n / 2)
    return u


@pytest.fixture(scope="module")
def big(wapmod, torch_cuda):
    """Context, inputs and the FP32 oracle's frame-step result at 256^3."""
    import oracle as O
    torch = torch_cuda
    n = N2
    ang = P.golden_angles(NP2)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (D2, D2), NP2, nframes_cli=F2), ang)
    foam = P.foam(n, seed=0)
    flow = _compress_flow(n)
    aabb = np.array([0, n, 0, n, 0, n], np.float32)
    # frame volumes: the foam advanced by 0, 0.1, 0.2 units of the deformation
    dfoam, dflow = dev(torch, foam), dev(torch, flow)
    vols = []
    for f in range(F2):
        out = torch.empty_like(dfoam)
        torch.cuda.synchronize()
        ctx.advect([n] * 3, aabb, dflow, dfoam, 1, 0.1 * f, out)
        ctx.synchronize()
        vols.append(host(out))
    nf, st, en, ft, tu = wapmod.level_frames(ctx.scan, 0)
    need = [0] + list(range(int(st[FRAME]), int(en[FRAME]) + 1))
    projs = np.zeros((NP2, D2, D2), np.float32)
    img = torch.zeros((D2, D2), device="cuda")
    dv1 = dev(torch, vols[FRAME])
    for k in need:
        torch.cuda.synchronize()
        ctx.forward(k, dv1, img)
        ctx.synchronize()
        projs[k] = host(img)
    rng = np.random.default_rng(2)
    projs[need] += rng.normal(scale=0.01 * projs.max(), size=projs[need].shape).astype(np.float32)
    ctx.upload_projections(projs)
    oscan = O.make_scan((n, n, n), (D2, D2), NP2, nframes_cli=F2)
    oscan.gmax = ctx.gmax
    # the benchmark's schedule with a shortened flow: 52 primal-dual iterations
    # (one residual iteration at 50) on 2 levels, 1 warp
    kw = dict(n_cp=1, nb_sart=2, wp_frames=F2, flow_iters=52, flow_scales=2, flow_tol=0.0, cut=8, flow_warps=1)
    sched_o = O.Schedule(nb_projwarp=1, flow_lambda=0.05, flow_eta=0.5, flow_sigma=0.8, deterministic=0, **kw)

    def oracle_step(orc):
        cast = orc.arr
        state = dict(vols=cast(np.stack(vols)), flows=cast(np.zeros((F2, 3, n, n, n))),
                     ytv=cast(np.zeros((F2, 3, n, n, n))), ytp=cast(np.zeros((F2, n, n, n))),
                     xbar=cast(np.zeros((F2, n, n, n))), xprev=cast(np.zeros((F2, n, n, n))))
        orc.outer_iteration_frames(oscan, sched_o, ang, cast(projs), 0, FRAME, FRAME + 1, state)
        return state["vols"][FRAME].copy(), state["flows"][FRAME].copy()

    want32 = oracle_step(O.Oracle())
    yield dict(torch=torch, ctx=ctx, vols=vols, flow=flow, foam=foam, projs=projs, ang=ang, oscan=oscan, aabb=aabb,
               kw=kw, oracle_step=oracle_step, want32=want32, O=O)
    ctx.close()


def _frame_step(wapmod, b, bits, bp_exact):
    ctx = b["ctx"]
    ctx.set_tuning("flow_bits", bits)
    try:
        ctx.level_setup(0)
        for f in range(F2):
            ctx.upload_volume(f, b["vols"][f])
        ctx.outer_iteration_frames(wapmod.reference_schedule(bp_exact=bp_exact, **b["kw"]), FRAME, FRAME + 1)
        return ctx.download_volume(FRAME), ctx.download_flow(FRAME)
    finally:
        ctx.set_tuning("flow_bits", 32)


def test_256_kernels_bitexact(big, orc):
    """One 256^3 -> 384^2 forward projection (image, ray length, sample
    count), the reference's double-arithmetic backprojection and the FP32 one,
    and one warp, each against the oracle at full size."""
    b = big
    torch, ctx, n = b["torch"], b["ctx"], N2
    vol = b["vols"][FRAME]
    dvol = dev(torch, vol)
    for k in (0, 61, 150):
        img, ln, wt = (torch.zeros((D2, D2), device="cuda") for _ in range(3))
        torch.cuda.synchronize()
        ctx.forward(k, dvol, img, ln, wt)
        ctx.synchronize()
        oi, ol, ow = orc.forward(b["oscan"], b["ang"][k], vol)
        assert np.array_equal(host(wt), ow), "sample counts differ at projection %d" % k
        assert np.array_equal(host(ln), ol), "ray lengths differ at projection %d" % k
        assert np.array_equal(host(img), oi), "projection %d differs" % k
    corr = np.ascontiguousarray((b["projs"][61] - oi) * 1e-2, np.float32)
    box = [8, n - 8] * 3
    want = orc.bp_voxel(b["oscan"], b["ang"][61], corr, box, 0, vol.copy())
    for exact in (1, 0):
        dv = dev(torch, vol)
        torch.cuda.synchronize()
        ctx.backproject_voxel(61, dev(torch, corr), box, 0, exact, dv)
        ctx.synchronize()
        if exact:
            assert np.array_equal(host(dv), want)
        else:
            assert rel_l2(host(dv), want) < 1e-5
    out = torch.empty_like(dvol)
    torch.cuda.synchronize()
    ctx.advect([n] * 3, b["aabb"], dev(torch, b["flow"]), dvol, 1, -0.35, out)
    ctx.synchronize()
    assert np.array_equal(host(out), orc.advect([n] * 3, b["aabb"], b["flow"], vol, -0.35))


def test_256_pd_forms_and_zchunks_agree(big):
    """The primal-dual kernel at 256^3 in every form and several z-chunks,
    autotuned included, 52 iterations (a residual iteration at 50): all give
    the same bits (the autotuned plan is the one the frame-step test below
    compares with the oracle)."""
    b = big
    torch, ctx, n = b["torch"], b["ctx"], N2
    I1, I2 = b["vols"][0], b["vols"][1]
    V0 = (b["flow"] * 0.05).astype(np.float32)
    res = {}
    plans = [(0, 0), (3, 0), (3, 26), (3, 8), (3, 64), (2, 0), (1, 0)]
    for form, zc in plans:
        ctx.set_tuning("pd_form", form)
        ctx.set_tuning("pd_zchunk", zc)
        dV = dev(torch, V0)
        dY = [torch.zeros((3, n, n, n), device="cuda") for _ in range(3)] + [torch.zeros((n, n, n), device="cuda")]
        torch.cuda.synchronize()
        its = ctx.flow_level([n] * 3, dev(torch, I1), dev(torch, I2), dV, *dY, 0.0, 0.05, 52, 1, b["aabb"], [8] * 6)
        assert list(its) == [53]
        res[(form, zc)] = (host(dV), host(dY[3]))
        if (form, zc) == (0, 0):  # the autotuner's pick (forcing a form clears the tuned plans)
            picked = ctx.get_tuning([n] * 3)
            assert picked[0] in (1, 2, 3) and picked[1] >= 1, picked
        del dY
    ctx.set_tuning("pd_form", 0)
    ctx.set_tuning("pd_zchunk", 0)
    ref = res[(0, 0)]
    for k, v in res.items():
        assert np.array_equal(v[0], ref[0]) and np.array_equal(v[1], ref[1]), "plan %s differs" % (k,)


def test_256_frame_step_bitexact(big, wapmod):
    """One frame's share of an outer iteration at 256^3 x 384^2 (its CP
    iteration with 2 SART sweeps over its 7-projection window in the
    reference's double-arithmetic backprojection, the 2-level flow of its pair
    with the autotuned primal-dual plan, its warp-and-project window) is the
    oracle's bit for bit."""
    got_v, got_f = _frame_step(wapmod, big, 32, 1)
    want_v, want_f = big["want32"]
    assert np.array_equal(got_v, want_v), "volume rel L2 %.3g" % rel_l2(got_v, want_v)
    assert np.array_equal(got_f, want_f), "flow rel L2 %.3g" % rel_l2(got_f, want_f)


def test_256_flow_lanes_same_bits(big, wapmod):
    """The benchmark's two-frame step at 256^3 x 384^2 (frames 0 and 1: their
    CP and SART work, the two flow pairs they start, their warp-and-project
    windows; the bounded flow of this module) with the two pairs on two flow
    lanes at once and one after another: the same volumes and flows of every
    frame, bit for bit."""
    ctx = big["ctx"]
    sched = wapmod.reference_schedule(bp_exact=1, **big["kw"])

    def step(lanes):
        ctx.set_tuning("flow_lanes", lanes)
        ctx.level_setup(0)
        for f in range(F2):
            ctx.upload_volume(f, big["vols"][f])
        ctx.outer_iteration_frames(sched, 0, 2)
        return [ctx.download_volume(f) for f in range(F2)], [ctx.download_flow(f) for f in range(F2)]

    try:
        step(2)  # a flow shape's first pair runs alone (its plans are tuned undisturbed)
        one, two = step(1), step(2)
    finally:
        ctx.set_tuning("flow_lanes", 0)
    for f in range(F2):
        assert np.array_equal(two[0][f], one[0][f]), "volume %d rel L2 %.3g" % (f, rel_l2(two[0][f], one[0][f]))
        assert np.array_equal(two[1][f], one[1][f]), "flow %d rel L2 %.3g" % (f, rel_l2(two[1][f], one[1][f]))


def test_256_precision_form_against_fp64_oracle(big, wapmod):
    """The precision form (flow solver state in FP16 with its fast FP32
    arithmetic, FP32 backprojection) on the same 256^3 frame step: the
    reconstructed volume within 1e-3 relative L2 of the FP64 oracle (the
    reference's algorithm in double) and of the FP32 oracle; the flow, an
    ill-conditioned estimate, within 5e-3 of the FP64 oracle (the FP32 oracle
    itself is about 6e-4 from it on this step)."""
    O = big["O"]
    got_v, got_f = _frame_step(wapmod, big, 16, 0)
    want64_v, want64_f = big["oracle_step"](O.Oracle(fp64=True))
    want32_v, want32_f = big["want32"]
    ev64, ef64 = rel_l2(got_v, want64_v), rel_l2(got_f, want64_f)
    ev32 = rel_l2(got_v, want32_v)
    print("precision form at 256^3: volume %.3g (FP64 oracle), %.3g (FP32 oracle); flow %.3g (FP64 oracle); "
          "FP32 oracle vs FP64 oracle: volume %.3g, flow %.3g"
          % (ev64, ev32, ef64, rel_l2(want32_v, want64_v), rel_l2(want32_f, want64_f)))
    assert ev64 < 1e-3 and ev32 < 1e-3
    assert ef64 < 5e-3


# ---------------------------------------------------------------------------
# CP prior alone
# ---------------------------------------------------------------------------
def test_cp_prior_bitexact(wapmod, orc, torch_cuda):
    """Two Chambolle-Pock iterations with no SART sweep (TV and temporal dual,
    primal with its clamp, over-relaxation) over 4 frames against the oracle's
    CP functions (WaP_Tomo.cpp:586-689), so a CP error points here."""
    import oracle as O
    n, det, nproj, F = 24, 32, 16, 4
    ang = P.golden_angles(nproj)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (det, det), nproj, nframes_cli=F), ang)
    try:
        projs = np.random.default_rng(5).uniform(0, 2, (nproj, det, det)).astype(np.float32)
        ctx.upload_projections(projs)
        assert ctx.level_setup(0) == F
        vols = np.stack([P.ellipsoids(n, count=6, seed=10 + f) * (1.0 + 0.1 * f) for f in range(F)]).astype(np.float32)
        for f in range(F):
            ctx.upload_volume(f, vols[f])
        sched = wapmod.reference_schedule(n_cp=2, nb_sart=0, wp_frames=0, flow_iters=0, flow_scales=1, cut=4)
        ctx.outer_iteration_step(sched, 0)
        ctx.outer_iteration_step(sched, 1)
        oscan = O.make_scan((n, n, n), (det, det), nproj, nframes_cli=F)
        oscan.gmax = ctx.gmax
        box = np.array([4, n - 4] * 3, np.int32)
        x = vols.copy()
        ytv = np.zeros((F, 3, n, n, n), np.float32)
        ytp, xbar, xprev = (np.zeros((F, n, n, n), np.float32) for _ in range(3))
        zero = np.zeros((n, n, n), np.float32)
        _, st, en, _, _ = orc.level_frames(F, nproj, 0)
        import ctypes
        for _ in range(2):
            for f in range(F):
                nxt = xbar[f + 1] if f + 1 < F else zero
                orc.lib.orc_cp_dual(ctypes.byref(oscan), box, xbar[f], np.ascontiguousarray(nxt), ytv[f], ytp[f])
                prev = ytp[f - 1].ctypes.data if f > 0 else None
                orc.lib.orc_cp_primal(ctypes.byref(oscan), box, f, prev, ytp[f], ytv[f], x[f], xprev[f])
                # no SART sweep, but the proximal operator's final floor max(x * imROI, 0)
                orc.sart_prox(oscan, ang, projs, int(st[f]), int(en[f]), 0, box, x[f])
                orc.lib.orc_cp_overrelax(np.array([n] * 3, np.int32), box, x[f], xprev[f], xbar[f])
        for f in range(F):
            assert np.array_equal(ctx.download_volume(f), x[f]), "frame %d" % f
    finally:
        ctx.close()


# ---------------------------------------------------------------------------
# 512^3 x 768^2 (the precision configuration's size): the projector
# ---------------------------------------------------------------------------
def test_512_projection_bitexact_and_near_fp64(wapmod, orc, torch_cuda):
    """Forward projections of the 512^3 foam-and-smoke phantom onto a 768^2
    detector: bit-exact with the oracle (image, ray length, sample count).
    Against the FP64 oracle the reference's float arithmetic is about 4e-4
    relative L2 at this size (its sample positions are a float recurrence
    over some 900 steps per ray, whose drift grows with the grid; 3.5e-6 at
    32^3): held to 1e-3."""
    import oracle as O
    import precision_compare as P512
    torch = torch_cuda
    n, d, nproj = 512, 768, 360
    vol = P512.phantom(torch, n)
    torch.cuda.synchronize()
    h = vol.cpu().numpy()
    ang = P.golden_angles(nproj)
    ctx = wapmod.Context(wapmod.make_scan((n, n, n), (d, d), nproj, nframes_cli=3), ang)
    oscan = O.make_scan((n, n, n), (d, d), nproj, nframes_cli=3)
    o64 = O.Oracle(fp64=True)
    try:
        for k in (0, 121):
            img, ln, wt = (torch.zeros((d, d), device="cuda") for _ in range(3))
            torch.cuda.synchronize()
            ctx.forward(k, vol, img, ln, wt)
            ctx.synchronize()
            oi, ol, ow = orc.forward(oscan, ang[k], h)
            assert np.array_equal(host(wt), ow), "sample counts, projection %d" % k
            assert np.array_equal(host(ln), ol) and np.array_equal(host(img), oi), "projection %d" % k
            ref = o64.forward(oscan, ang[k], o64.arr(h))[0]
            err = rel_l2(host(img), ref)
            print("512^3 projection %d: %.3g relative L2 from the FP64 oracle" % (k, err))
            assert err < 1e-3
    finally:
        ctx.close()
