"""The request loop on the GPU: jobs of uneven sizes admitted under an HBM
budget, stepped concurrently by several workers, give the same bits as each
job run alone; the reserved footprint covers what a context really holds."""
import numpy as np
import pytest

import phantoms as P

pytestmark = pytest.mark.gpu


def _job(wap, orc, O, n, nproj, seed):
    det = int(n * 1.5)
    vol = P.ellipsoids(n, count=6, seed=seed)
    ang = P.golden_angles(nproj)
    oscan = O.make_scan((n, n, n), (det, det), nproj, nframes_cli=nproj // 8)
    projs = np.stack([orc.forward(oscan, a, vol)[0] for a in ang]).astype(np.float32)
    scan = wap.make_scan((n, n, n), (det, det), nproj, nframes_cli=nproj // 8)
    sched = wap.reference_schedule(n_cp=2, nb_sart=2, wp_frames=nproj // 8, flow_iters=30, flow_scales=2,
                                   flow_tol=0.0, flow_warps=1)
    return scan, sched, ang, projs


def _alone(wap, scan, sched, ang, projs, outer, flow_bits=32):
    ctx = wap.Context(scan, ang)
    try:
        ctx.set_tuning("flow_bits", flow_bits)
        ctx.upload_projections(projs)
        F = ctx.level_setup(0)
        for _ in range(outer):
            ctx.outer_iteration(sched)
        return [ctx.download_volume(f) for f in range(F)], wap.load().wap_ctx_device_bytes(ctx.h)
    finally:
        ctx.close()


def test_served_jobs_match_the_same_jobs_alone(wapmod, orc, torch_cuda):
    import oracle as O
    wap = wapmod
    specs = [(24, 16, 1), (32, 24, 2), (20, 16, 3), (28, 16, 4)]
    jobs = [_job(wap, orc, O, n, p, seed) for n, p, seed in specs]
    outer = 2
    alone = [_alone(wap, *j, outer) for j in jobs]
    # the admission footprint covers the memory a context reaches
    for j, (_, used) in zip(jobs, alone):
        est = wap.job_device_bytes(j[0], j[1])
        assert used <= est < 3 * used + (8 << 20), (used, est)
    # a budget that fits about two jobs at a time forces queueing
    budget = int(2.2 * max(wap.job_device_bytes(j[0], j[1]) for j in jobs))
    srv = wap.Server(budget, workers=3)
    try:
        ids = [srv.submit(j[0], j[1], j[2], j[3], outer_iterations=outer) for j in jobs]
        for jid in ids:
            assert srv.wait(jid, 600.0) == wap.WAP_OK
        for jid, j, (vols, _) in zip(ids, jobs, alone):
            n = j[0].vol[0]
            info = srv.info(jid)
            assert info.state == wap.WAP_JOB_DONE
            assert info.t_submit <= info.t_admit <= info.t_done
            for f, v in enumerate(vols):
                assert np.array_equal(srv.result(jid, f, (n, n, n)), v), (jid, f)
            assert srv.release(jid) == wap.WAP_OK
        in_use, peak = srv.memory()
        assert in_use == 0 and 0 < peak <= budget
    finally:
        srv.close()


def test_server_rejects_a_job_larger_than_the_budget(wapmod, orc, torch_cuda):
    import oracle as O
    wap = wapmod
    scan, sched, ang, projs = _job(wap, orc, O, 24, 16, 5)
    srv = wap.Server(1 << 20, workers=1)
    try:
        with pytest.raises(wap.WapError):
            srv.submit(scan, sched, ang, projs)
    finally:
        srv.close()


def test_served_precision_form_matches_the_same_jobs_alone(wapmod, orc, torch_cuda):
    """Jobs submitted with flow_bits = 16 run the precision form in the mix
    and give the same bits as the same jobs run alone in that form; the
    footprint reserved for them includes the FP16 pair state."""
    import oracle as O
    wap = wapmod
    specs = [(32, 16, 6), (24, 24, 7), (40, 16, 8)]
    jobs = [_job(wap, orc, O, n, p, seed) for n, p, seed in specs]
    alone = [_alone(wap, *j, 1, flow_bits=16) for j in jobs]
    srv = wap.Server(int(2.5 * max(wap.job_device_bytes(j[0], j[1]) for j in jobs)), workers=2)
    try:
        ids = [srv.submit(j[0], j[1], j[2], j[3], outer_iterations=1, flow_bits=16) for j in jobs]
        for jid in ids:
            assert srv.wait(jid, 600.0) == wap.WAP_OK
        for jid, j, (vols, used) in zip(ids, jobs, alone):
            n = j[0].vol[0]
            info = srv.info(jid)
            assert info.device_bytes >= used, (info.device_bytes, used)
            for f, v in enumerate(vols):
                assert np.array_equal(srv.result(jid, f, (n, n, n)), v), (jid, f)
            assert srv.release(jid) == wap.WAP_OK
    finally:
        srv.close()
