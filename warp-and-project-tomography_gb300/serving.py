"""Served form: a seeded Poisson stream of reconstruction jobs of uneven sizes
through the request loop (wap.Server, include/wap/wap_serve.h).

Jobs run the reference's arithmetic (flow_bits 32) or the precision form
(flow_bits 16: the flow solver's state as FP16 pairs with its fast arithmetic).

Job mix (the served workload): volume sides drawn from {64, 96, 128, 192,
256} with weights 0.3/0.25/0.2/0.15/0.1, projection counts from {64, 128,
192}, detector side 1.5x the volume side, ellipsoid phantoms generated on the
device, arrivals at a mean rate per second (seed 3).  Each job is one outer
iteration of the reconstruction at time level 0 with frames = projections /
8, 2 CP iterations x 2 SART sweeps, a 2-level flow of 20 primal-dual
iterations and 1 warp per level, and the FP32 backprojection.  All inputs are
generated before the arrival clock starts; latency is submit -> results on the
host, on the server's clock.
"""
import time

import numpy as np

# The served configuration's accuracy target: a job served in another
# arithmetic must stay within this relative RMSE of the same job in the
# reference's arithmetic (the reconstruction-error bound of the precision form).
RMSE_TARGET = 1e-3
SIZES = (64, 96, 128, 192, 256)
WEIGHTS = (0.3, 0.25, 0.2, 0.15, 0.1)
NPROJS = (64, 128, 192)


def job_stream(n_jobs, rate, seed=3, max_side=256):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n_jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    sides = rng.choice(SIZES, size=n_jobs, p=WEIGHTS)
    sides = np.minimum(sides, max_side)
    nprojs = rng.choice(NPROJS, size=n_jobs)
    return [dict(t=float(t), n=int(n), nproj=int(p), seed=1000 + i)
            for i, (t, n, p) in enumerate(zip(arrivals, sides, nprojs))]


def served_schedule(wap, frames):
    s = wap.reference_schedule(n_cp=2, nb_sart=2, wp_frames=frames, flow_iters=20, flow_scales=2, flow_tol=0.0,
                               flow_warps=1, bp_exact=0)
    return s


def _phantom(torch, n, seed, count=12):
    g = torch.Generator(device="cuda").manual_seed(seed)
    ax = torch.arange(n, device="cuda", dtype=torch.float32)
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    vol = torch.zeros((n, n, n), device="cuda")
    for _ in range(count):
        c = (0.15 + 0.7 * torch.rand(3, device="cuda", generator=g)) * n
        r = (3.0 + 13.0 * torch.rand(3, device="cuda", generator=g)) * (n / 64.0)
        d = ((x - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((z - c[2]) / r[2]) ** 2
        vol += (d <= 1.0).float() * (0.1 + 0.9 * torch.rand(1, device="cuda", generator=g))
    return vol


def make_job(wap, torch, spec):
    """Scan, schedule, angles and host projections of one job."""
    n, nproj = spec["n"], spec["nproj"]
    det = int(round(1.5 * n))
    frames = max(1, nproj // 8)
    scan = wap.make_scan((n, n, n), (det, det), nproj, nframes_cli=frames)
    ang = (np.arange(nproj, dtype=np.float64) * 360.0 * 0.6180339887) % 360.0
    vol = _phantom(torch, n, spec["seed"])
    torch.cuda.synchronize()  # the context's stream does not wait on torch's
    ctx = wap.Context(scan, ang)
    try:
        projs = torch.empty((nproj, det, det), device="cuda")
        for k in range(nproj):
            ctx.forward(k, vol, projs[k])
        ctx.synchronize()
        host = projs.cpu().numpy()
    finally:
        ctx.close()
    return dict(scan=scan, sched=served_schedule(wap, frames), angles=ang, projs=host, n=n)


def run(wap, torch, n_jobs=40, rate=20.0, budget_gb=150.0, workers=3, seed=3, max_side=256, flow_bits=(32,)):
    """The job stream through the request loop once per entry of flow_bits
    (the same jobs and arrival times each time); one result dict per entry."""
    specs = job_stream(n_jobs, rate, seed, max_side)
    jobs = [make_job(wap, torch, s) for s in specs]
    torch.cuda.synchronize()
    runs = [_serve(wap, specs, jobs, rate, budget_gb, workers, fb) for fb in flow_bits]
    # Accuracy of every form against the first (the reference's arithmetic):
    # relative RMSE of each job's first-frame volume.
    base = runs[0].pop("_frame0")
    for r in runs[1:]:
        got = r.pop("_frame0")
        err = np.array([float(np.linalg.norm(g.astype(np.float64) - b) / max(np.linalg.norm(b.astype(np.float64)),
                                                                             1e-30)) for g, b in zip(got, base)])
        r["rmse_vs_reference_arithmetic"] = {
            "measure": "relative RMSE of each job's first-frame volume against the same job served in the "
                       "reference's arithmetic", "target": RMSE_TARGET,
            "jobs_within_target": int((err <= RMSE_TARGET).sum()), "max": float(err.max()),
            "p50": float(np.percentile(err, 50)), "p99": float(np.percentile(err, 99))}
    return runs


def _serve(wap, specs, jobs, rate, budget_gb, workers, flow_bits):
    n_jobs = len(specs)
    budget = int(budget_gb * (1 << 30))
    srv = wap.Server(budget, workers=workers)
    try:
        start = time.perf_counter()
        ids = []
        for s, j in zip(specs, jobs):
            delay = s["t"] - (time.perf_counter() - start)
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(j["scan"], j["sched"], j["angles"], j["projs"], outer_iterations=1,
                                  flow_bits=flow_bits))
        for jid in ids:
            if srv.wait(jid, 3600.0) != wap.WAP_OK:
                raise wap.WapError("served job %d failed" % jid)
        infos = [srv.info(jid) for jid in ids]
        _, peak = srv.memory()
        frame0 = []
        for jid, j in zip(ids, jobs):
            frame0.append(srv.result(jid, 0, (j["n"],) * 3))
            srv.release(jid)
    finally:
        srv.close()
    lat = np.array([i.t_done - i.t_submit for i in infos])
    wait = np.array([i.t_admit - i.t_submit for i in infos])
    span = max(i.t_done for i in infos) - min(i.t_submit for i in infos)
    return {
        "jobs": n_jobs, "arrival_rate_per_s": rate, "workers": workers, "budget_gb": budget_gb,
        "throughput_jobs_per_s": n_jobs / span,
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                      "p99": float(np.percentile(lat, 99)), "mean": float(lat.mean())},
        "admission_wait_s_mean": float(wait.mean()),
        "peak_reserved_gb": peak / float(1 << 30),
        "sides": {str(k): int(sum(1 for s in specs if s["n"] == k)) for k in SIZES},
        "job": "1 outer iteration, frames = projections/8, 2 CP x 2 SART, 2-level flow x 20 PD its, FP32 BP",
        "flow_bits": flow_bits, "_frame0": frame0,
    }


def batched_schedule(wap, frames, flow_iters):
    """The batched configuration's schedule: 4 CP iterations x 2 SART sweeps
    (8 sweeps), a 3-level flow (flow_iters primal-dual iterations, 1 warp per
    level), warp-and-project over every window, the reference's double
    backprojection."""
    return wap.reference_schedule(n_cp=4, nb_sart=2, wp_frames=frames, flow_iters=flow_iters, flow_scales=3,
                                  flow_tol=0.0, flow_warps=1, bp_exact=1)


def run_batched(wap, torch, n_jobs=48, seed=5, outer=1, flow_iters=40):
    """Batched form: n_jobs independent scans of uneven sizes (sides from {48,
    64, 96, 128, 160}, projections uniform in [48, 256], detector 1.5x the
    side, frames = projections / 4) reconstructed (a) one after another
    through the plain path, one context at a time, and (b) together through
    wap_batch (include/wap/wap_batch.h): the SART steps of every scan in
    work-queue launches, each CP iteration a replayed CUDA graph, the flows
    and warp-and-project passes on the scans' own streams.  Returns both wall
    times (outer iterations of every scan) and checks that every scan's
    volumes and flows are identical."""
    rng = np.random.default_rng(seed)
    specs = [dict(t=0.0, n=int(rng.choice((48, 64, 96, 128, 160))), nproj=int(rng.integers(48, 257)),
                  seed=2000 + i) for i in range(n_jobs)]
    jobs = []
    for sp in specs:
        j = make_job(wap, torch, sp)
        j["scan"] = wap.make_scan((j["n"],) * 3, tuple(j["scan"].det), sp["nproj"], nframes_cli=max(1, sp["nproj"] // 4))
        jobs.append(j)
    torch.cuda.synchronize()

    def ctx_of(j):
        c = wap.Context(j["scan"], j["angles"])
        c.upload_projections(j["projs"])
        c.level_setup(0)
        return c

    t0 = time.perf_counter()
    plain = []
    for j in jobs:
        ctx = ctx_of(j)
        try:
            F = ctx.L.wap_level_nframes(ctx.h)
            for _ in range(outer):
                ctx.outer_iteration(batched_schedule(wap, F, flow_iters))
            plain.append(([ctx.download_volume(f) for f in range(F)], [ctx.download_flow(f) for f in range(F)]))
        finally:
            ctx.close()
    t_loop = time.perf_counter() - t0
    ctxs = [ctx_of(j) for j in jobs]
    try:
        b = wap.Batch(ctxs)
        try:
            scheds = [batched_schedule(wap, c.L.wap_level_nframes(c.h), flow_iters) for c in ctxs]
            for c in ctxs:
                c.synchronize()
            t0 = time.perf_counter()
            for _ in range(outer):
                st = b.outer_iteration(scheds)
            t_batch = time.perf_counter() - t0
            shapes = b.get_tuning()
        finally:
            b.close()
        same = True
        for c, (vols, flows) in zip(ctxs, plain):
            c.synchronize()
            for f in range(len(vols)):
                same = same and np.array_equal(c.download_volume(f), vols[f]) and np.array_equal(
                    c.download_flow(f), flows[f])
    finally:
        for c in ctxs:
            c.close()
    return {"scans": n_jobs, "outer_iterations": outer, "loop_s": t_loop, "batched_s": t_batch,
            "speedup": t_loop / t_batch, "identical": bool(same), "tile_shapes": {"fp": shapes[0], "bp": shapes[1]},
            "launches_per_batch_outer_iteration": int(st.kernel_launches),
            "sides": {str(k): int(sum(1 for s in specs if s["n"] == k)) for k in (48, 64, 96, 128, 160)},
            "projections_total": int(sum(s["nproj"] for s in specs)),
            "job": "4 CP x 2 SART, 3-level flow x %d PD its x 1 warp, WaP over all windows, exact BP; frames = "
                   "projections / 4" % flow_iters}


def run_sequential(wap, torch, n_jobs=3, seed=3, max_side=256, flow_bits=32):
    """The first n_jobs of the stream run one after another on their own
    contexts (no request loop): per job its phase times from the library's
    stats.  Used to attribute a served job's GPU time (e.g. under an ncu
    launch list)."""
    out = []
    for spec in job_stream(n_jobs, 20.0, seed, max_side):
        j = make_job(wap, torch, spec)
        ctx = wap.Context(j["scan"], j["angles"])
        try:
            ctx.set_tuning("flow_bits", flow_bits)
            ctx.upload_projections(j["projs"])
            F = ctx.level_setup(0)
            t0 = time.perf_counter()
            st = ctx.outer_iteration(j["sched"])
            ctx.synchronize()
            out.append({"side": spec["n"], "projections": spec["nproj"], "frames": F,
                        "seconds": time.perf_counter() - t0, "cp_sart_s": st.ms_cp / 1e3, "flow_s": st.ms_flow / 1e3,
                        "wap_s": st.ms_wap / 1e3, "kernel_launches": int(st.kernel_launches)})
        finally:
            ctx.close()
    return out


if __name__ == "__main__":
    import argparse
    import json
    import os
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch as _torch

    import build as _build
    import wap as _wap

    ap = argparse.ArgumentParser(description="served jobs one after another, with per-phase times; or, with "
                                             "--served N, the served stream of N jobs through the request loop in "
                                             "both arithmetics")
    ap.add_argument("--jobs", type=int, default=3)
    ap.add_argument("--flow-bits", type=int, default=32)
    ap.add_argument("--served", type=int, default=0)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--workers", type=int, default=3)
    a = ap.parse_args()
    _build.build()
    if a.served:
        plain, fast = run(_wap, _torch, n_jobs=a.served, rate=a.rate, workers=a.workers, flow_bits=(32, 16))
        print(json.dumps({"serving": plain, "serving_precision": fast}))
    else:
        for rec in run_sequential(_wap, _torch, n_jobs=a.jobs, flow_bits=a.flow_bits):
            print(json.dumps(rec))
