"""The batched form (include/wap/wap_batch.h): scans of uneven sizes
reconstructed together (SART steps of every scan in work-queue launches, the
CP iteration replayed as a CUDA graph, flows and warp-and-project on the
scans' streams) give, scan by scan, the bits of the same scan run alone
through wap_outer_iteration, over two outer iterations, with the autotuned
and with forced tile shapes."""
import numpy as np
import pytest

import phantoms as P

pytestmark = pytest.mark.gpu

# (side, detector, projections): uneven volumes, detectors and frame counts
SCANS = [(24, 36, 12), (32, 48, 16), (20, 28, 8), (36, 52, 20)]


@pytest.fixture(scope="module")
def scans(wapmod, orc, torch_cuda):
    import oracle as O
    out = []
    for k, (n, det, nproj) in enumerate(SCANS):
        vol = P.ellipsoids(n, count=8, seed=30 + k)
        ang = P.golden_angles(nproj) + 7.0 * k
        oscan = O.make_scan((n, n, n), (det, det), nproj, nframes_cli=nproj // 4)
        projs = np.stack([orc.forward(oscan, a, vol)[0] for a in ang]).astype(np.float32)
        projs += np.random.default_rng(k).normal(scale=0.01 * projs.max(), size=projs.shape).astype(np.float32)
        out.append(dict(scan=wapmod.make_scan((n, n, n), (det, det), nproj, nframes_cli=nproj // 4), ang=ang,
                        projs=projs, n=n))
    return out


def schedule(wapmod, F):
    return wapmod.reference_schedule(n_cp=2, nb_sart=2, wp_frames=F, flow_iters=30, flow_scales=2, flow_tol=0.0,
                                     flow_warps=1, cut=4)


def contexts(wapmod, scans):
    ctxs = []
    for s in scans:
        c = wapmod.Context(s["scan"], s["ang"])
        c.upload_projections(s["projs"])
        c.level_setup(0)
        ctxs.append(c)
    return ctxs


def frames(ctx):
    return ctx.L.wap_level_nframes(ctx.h)


def state(ctx):
    ctx.synchronize()
    F = frames(ctx)
    return [ctx.download_volume(f) for f in range(F)], [ctx.download_flow(f) for f in range(F)]


@pytest.fixture(scope="module")
def alone(wapmod, scans):
    """Each scan alone, two outer iterations, the state after each."""
    res = []
    for c in contexts(wapmod, scans):
        try:
            per = []
            for _ in range(2):
                c.outer_iteration(schedule(wapmod, frames(c)))
                per.append(state(c))
            res.append(per)
        finally:
            c.close()
    return res


@pytest.mark.parametrize("shapes", [None, (1, 2), (2, 1)])
def test_batch_equals_each_scan_alone(wapmod, scans, alone, shapes):
    ctxs = contexts(wapmod, scans)
    try:
        b = wapmod.Batch(ctxs)
        try:
            if shapes:
                b.set_tuning(*shapes)
            scheds = [schedule(wapmod, frames(c)) for c in ctxs]
            for it in range(2):
                st = b.outer_iteration(scheds)
                assert st.projections > 0 and st.flow_pd_iterations > 0
                for k, c in enumerate(ctxs):
                    vols, flows = state(c)
                    want_v, want_f = alone[k][it]
                    for f in range(len(vols)):
                        assert np.array_equal(vols[f], want_v[f]), (shapes, it, k, f)
                        assert np.array_equal(flows[f], want_f[f]), (shapes, it, k, f)
            fp, bp = b.get_tuning()
            assert 0 <= fp < 3 and 0 <= bp < 3
            if shapes:
                assert (fp, bp) == shapes
        finally:
            b.close()
    finally:
        for c in ctxs:
            c.close()


def test_batch_rejects_mixed_sweeps(wapmod, scans):
    ctxs = contexts(wapmod, scans[:2])
    try:
        b = wapmod.Batch(ctxs)
        try:
            s0, s1 = schedule(wapmod, frames(ctxs[0])), schedule(wapmod, frames(ctxs[1]))
            s1.nb_sart = 3
            with pytest.raises(wapmod.WapError):
                b.outer_iteration([s0, s1])
        finally:
            b.close()
    finally:
        for c in ctxs:
            c.close()
