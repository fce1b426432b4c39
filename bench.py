"""Throughput benchmark: WaP outer iterations per second at 256^3 x 192 projections.

Workload (the 256^3 GPU-vs-CPU configuration): a 256^3 FP32 foam phantom
(band-limited noise thresholded at the 70th percentile), compressed over time
(u_z = -0.25 t (z - z0) plus a smooth RBF perturbation of <= 6 voxels), 192
cone-beam projections at 384x384 on golden-ratio angles, one deformation state
each, Poisson noise at I0 = 1e4.  Seeded synthetic data stands in for the
reference's (unpublished) scans.  48 frames (4 projections each, windows +-3),
schedule of PSART::Render: 5 CP iterations x 2 SART sweeps, a 4-level L1-TV
flow (tol 0.008, lambda 0.05, <= 3000 iterations, 3 warps) for every
adjacent pair, then warp-and-project over every frame's window.

A "step" is the complete share of an outer iteration of --frames-per-step
consecutive frames (2 by default: their CP + SART steps, the flow pairs they
start, which run concurrently on the library's flow lanes, their
warp-and-project windows): an outer iteration is exactly F / 2 such steps, so
value = outer-iter/s = 2 / (F * mean step time).  A whole outer iteration at this size is minutes of
GPU time, which is why the unit streamed here is the frame share.

value times the steps on the device with inputs resident; e2e times the same
steps with each step's inputs (its projection window) copied host->device
from pinned memory and its results (volume and flow) copied back.

--impl reference times the reference algorithm on the host CPU (the oracle
port of the reference's OpenMP code) on a bounded sample: one forward and
back projection, one warp, one CP frame pass at full size and 50 primal-dual
iterations at each pyramid level per step (ms_per_step is that sample's wall
time), composed into
outer-iter/s from the op counts of one whole outer iteration measured on the
GPU (outer_iteration_counts_256.json in the package; the GPU path performs the
reference's operations bit for bit, so the counts are the reference's too).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "warp-and-project-tomography_gb300")
for _p in (PKG, os.path.join(REPO, "tests"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "WaP outer-iter/s at 256^3 x 192 proj"
PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")
# Algorithmic bytes of one primal-dual iteration per voxel, the figure the
# roofline is quoted against: the two-kernel minimum of the iteration (30
# y-words, 15 v-words, 7 u-words; optical_flow.h:478-813).
PD_BYTES_PER_VOXEL = 4 * (30 + 15 + 7)
# The single-pass minimum (read and write y and v once, read u once), which
# only the fused kernel form reaches.
PD_BYTES_MIN_PER_VOXEL = 4 * (10 + 10 + 3 + 3 + 4)
# DRAM bytes (read + write) of one primal-dual iteration at 256^3 per kernel
# form (1 fused, 2 primal + dual, 3 TMA-fed fused), from ncu captures
# (dram__bytes_read.sum + dram__bytes_write.sum) of
# warp-and-project-tomography_gb300/kernel_bench.py --kernel pd --n 256.
PD_TRAFFIC_256 = {1: 1.98e9, 2: 3.29e9, 3: 1.95e9}
PD_TRAFFIC_SOURCE = {1: "profiles/pd_fused_kernel_256cube_traffic.md", 2: "profiles/pd_fused_kernel_256cube_traffic.md",
                     3: "profiles/pd_tma_kernel_256cube_full.md"}
PD_FORMS = {1: "pd_fused_kernel", 2: "pd_primal_kernel + pd_dual_kernel", 3: "pd_tma_kernel (TMA-fed fused)",
            4: "pd_tma_kernel<__half> (precision form)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--det", type=int, default=384)
    ap.add_argument("--nproj", type=int, default=192)
    ap.add_argument("--scales", type=int, default=4)
    ap.add_argument("--flow-iters", type=int, default=3000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-jobs", type=int, default=40,
                    help="jobs of the served-form measurement added to the line (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-workers", type=int, default=3)
    ap.add_argument("--flow-bits", type=int, default=32, choices=[32, 16],
                    help="32: the reference's arithmetic; 16: the precision form (FP16 flow state)")
    ap.add_argument("--precision-steps", type=int, default=10,
                    help="frame-steps re-timed in the precision form for the line's precision_form object (0: skip)")
    ap.add_argument("--batch-jobs", type=int, default=48,
                    help="scans of the batched-form comparison added to the line (0: skip)")
    ap.add_argument("--batch-flow-iters", type=int, default=40,
                    help="primal-dual iterations per level and warp of the batched scans' flows")
    ap.add_argument("--kernel-reps", type=int, default=5,
                    help="timed launches per kernel of the line's per-kernel roofline table (0: skip)")
    ap.add_argument("--frames-per-step", type=int, default=2,
                    help="consecutive frames a step covers: their CP and SART work, their flow pairs (which run "
                         "concurrently on the library's flow lanes) and their warp-and-project windows")
    ap.add_argument("--flow-lanes", type=int, default=0,
                    help="flow pairs the library runs concurrently (its flow_lanes tuning key; 0: the library's "
                         "automatic choice, 2 lanes at 256^3)")
    ap.add_argument("--full-outer", action="store_true",
                    help="also time one whole outer iteration (all frames in pass order; minutes at 256^3)")
    ap.add_argument("--save-outer-counts", default="",
                    help="with --full-outer: write that outer iteration's op counts to this JSON file (the counts "
                         "the CPU legs compose their outer-iter/s from)")
    return ap.parse_args()


# Op counts of one whole outer iteration of the default workload, measured by
# `python bench.py --full-outer --save-outer-counts <this file>` on a GB300.
# The GPU path is bit-exact with the reference, so the reference performs the
# same operations (in particular the same primal-dual iterations per level,
# which the tolerance stops early on the coarse levels).
OUTER_COUNTS = os.path.join(PKG, "outer_iteration_counts_256.json")
COUNT_KEYS = ("projections", "backprojections", "advect_voxels", "cp_frame_passes", "pd_voxel_iters")


def outer_counts(args):
    """The measured counts when the workload is the default one, else None."""
    if (args.n, args.det, args.nproj, args.scales, args.flow_iters) != (256, 384, 192, 4, 3000):
        return None
    try:
        with open(OUTER_COUNTS) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    c = {k: float(d["op_counts"][k]) for k in COUNT_KEYS}
    c["pd_iterations_per_level"] = [float(x) for x in d["pd_iterations_per_level_finest_first"]]
    return c


def bench_config(args, F):
    """The workload's config object, shared by both arms."""
    fs = getattr(args, "frames_per_step", 2)
    return {"workload": "256^3 volume, 192 proj at 384^2, 48 frames, 5 CP x 2 SART, 4-level L1-TV flow "
                        "(tol 0.008, <=3000 its, 3 warps), WaP over all windows" if (args.n, args.det, args.nproj) ==
                        (256, 384, 192) else
                        "%d^3 volume, %d proj at %d^2, %d frames, 5 CP x 2 SART, %d-level L1-TV flow (tol 0.008, "
                        "<=%d its, 3 warps), WaP over all windows"
                        % (args.n, args.nproj, args.det, F, args.scales, args.flow_iters),
            "step": "%d consecutive frames' share of an outer iteration (their CP and SART work, their flow pairs, "
                    "their warp-and-project windows); %d steps make one outer iteration" % (fs, F // fs),
            "volume": [args.n] * 3, "detector": [args.det] * 2, "projections": args.nproj, "frames": F,
            "parallelism": "single", "l2": "working set > L2 (GBs per step)",
            "bp_arithmetic": "reference double (exact)"}


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def workload(args, torch, ctx_factory):
    """Phantom, deformation, projections; returns (ctx, projs_device, angles, meta)."""
    import phantoms as P
    n, d, nproj = args.n, args.det, args.nproj
    nframes = nproj // 4
    torch.manual_seed(2)
    base = torch.from_numpy(P.foam(n, seed=0)).cuda()
    rbf = torch.from_numpy(P.rbf_flow(n, amp=6.0, sigma=12.0, seed=1)).cuda()
    ang = P.golden_angles(nproj)
    ctx = ctx_factory(n, d, nproj, nframes, ang)
    z = torch.arange(n, device="cuda", dtype=torch.float32).view(n, 1, 1).expand(n, n, n)
    projs = torch.empty((nproj, d, d), device="cuda")
    img = torch.empty((d, d), device="cuda")
    # backward-mapped deformation, trilinear (grid_sample) -- data generation only
    zz, yy, xx = torch.meshgrid(*(torch.arange(n, device="cuda", dtype=torch.float32),) * 3, indexing="ij")
    for k in range(nproj):
        t = k / float(nproj - 1)
        ux = t * rbf[0]
        uy = t * rbf[1]
        uz = -0.25 * t * (z - n / 2) + t * rbf[2]
        g = torch.stack([(xx - ux) / (n - 1) * 2 - 1, (yy - uy) / (n - 1) * 2 - 1, (zz - uz) / (n - 1) * 2 - 1], -1)
        vol_t = torch.nn.functional.grid_sample(base.view(1, 1, n, n, n), g.view(1, n, n, n, 3), align_corners=True,
                                                mode="bilinear", padding_mode="zeros").view(n, n, n).contiguous()
        ctx.forward(k, vol_t, img)
        ctx.synchronize()
        projs[k].copy_(img)
    kappa = 3.0 / float(projs.max())
    I0 = 1e4
    counts = torch.poisson(I0 * torch.exp(-kappa * projs), generator=None)
    projs = (-torch.log(torch.clamp(counts, min=1.0) / I0) / kappa).contiguous()
    del base, rbf, z, zz, yy, xx
    torch.cuda.empty_cache()
    return ctx, projs, ang, dict(nframes=nframes)


class ClockSampler:
    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU legs' reports."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(args, counts, threads):
    """Time the oracle port of the reference's CPU path on a bounded sample and
    compose seconds per outer iteration from the op counts of one outer
    iteration: one forward projection, one bicubic backprojection, one warp
    (on 4 threads, the reference's hard-coded worker count, advection.h:134-141),
    one CP frame pass, and 50 primal-dual iterations (one of them a residual
    iteration) at every pyramid level, weighted by that level's iterations."""
    import oracle as O
    import phantoms as P
    orc = O.Oracle()
    n, d = args.n, args.det
    scan = O.make_scan((n, n, n), (d, d), args.nproj, nframes_cli=args.nproj // 4, threads=threads)
    scan.gmax = 1.0
    vol = P.foam(n, seed=0)
    ang = P.golden_angles(args.nproj)
    t = {}
    t0 = time.time()
    img, ln, wt = orc.forward(scan, ang[5], vol)
    t["fp"] = time.time() - t0
    corr = np.ascontiguousarray(img * 1e-3, np.float32)
    v2 = vol.copy()
    t0 = time.time()
    orc.bp_voxel(scan, ang[5], corr, [8, n - 8, 8, n - 8, 8, n - 8], 0, v2)
    t["bp"] = time.time() - t0
    flow = P.rbf_flow(n, amp=3.0, seed=1)
    aabb = [0, n, 0, n, 0, n]
    t0 = time.time()
    warped = orc.advect([n] * 3, aabb, flow, vol, 0.5, 4)
    t["advect"] = time.time() - t0
    nv = n ** 3
    ytv = np.zeros((3, n, n, n), np.float32)
    ytp = np.zeros((n, n, n), np.float32)
    xp = np.zeros((n, n, n), np.float32)
    box = np.array([8, n - 8] * 3, np.int32)
    t0 = time.time()
    orc.lib.orc_cp_dual(O.ctypes.byref(scan), box, vol, vol, ytv, ytp)
    orc.lib.orc_cp_primal(O.ctypes.byref(scan), box, 1, ytp.ctypes.data, ytp, ytv, v2, xp)
    orc.lib.orc_cp_overrelax(np.array([n] * 3, np.int32), box, v2, xp, ytp)
    t["cp"] = time.time() - t0
    del ytv, ytp, xp
    pd_its = 50
    t["pd_iteration_per_level"] = []
    for lev in range(len(counts["pd_iterations_per_level"])):
        step = 1 << lev
        m = n // step
        # a deforming pair (the volume and its warp by the smooth flow), as the
        # reference's frame pairs are
        I1 = np.ascontiguousarray(vol[::step, ::step, ::step])
        I2 = np.ascontiguousarray(warped.reshape(vol.shape)[::step, ::step, ::step])
        V = np.zeros((3, m, m, m), np.float32)
        Y = [np.zeros((3, m, m, m), np.float32) for _ in range(3)] + [np.zeros((m, m, m), np.float32)]
        orc.flow_level([m] * 3, I1, I2, V, *Y, 0.0, 0.05, pd_its - 1, 1, [0, m, 0, m, 0, m],
                       [max(1, 8 >> lev)] * 6, deterministic=0)
        t["pd_iteration_per_level"].append(orc.lib.orc_last_pd_seconds() / pd_its)
    sec = (counts["projections"] * t["fp"] + counts["backprojections"] * t["bp"] +
           counts["advect_voxels"] / nv * t["advect"] + counts["cp_frame_passes"] * t["cp"] +
           sum(i * s for i, s in zip(counts["pd_iterations_per_level"], t["pd_iteration_per_level"])))
    sample = ("composed from one %d^3->%d^2 forward projection, one bicubic backprojection, one warp (4 threads, "
              "as the reference), one CP frame pass and %d primal-dual iterations at each of %d pyramid levels "
              "(OpenMP, %d threads; CPU: %s), weighted by the op counts of one outer iteration"
              % (n, d, pd_its, len(counts["pd_iterations_per_level"]), threads, cpu_model()))
    return sec, t, sample


def kernel_table(ctx, torch, stream, args, frame, peak):
    """Per-kernel rooflines of the hot path, timed on the library's stream with
    CUDA events (median of args.kernel_reps launches after one warm-up) on the
    run's own frame volume and flow.  Algorithmic bytes per launch (FP32
    storage, V voxels, D detector pixels, V_roi the backprojection box):
      fp          forward projection with its outputs: V*4 + 16*D
      bp          voxel-driven backprojection over the ROI: 2*V_roi*4 + 4*D
      sart_step   one SART step (projection with the fused correction and dual
                  update, then backprojection): 3*V*4 + 20*D
      advect      one warp of a volume by a 3-channel flow: V*(2*4 + 3*4)
    The frame's state is restored afterwards."""
    import wap
    n, d = args.n, args.det
    nv, D = n ** 3, d * d
    nf, st, en, ft, tu = wap.level_frames(ctx.scan, 0)
    proj = int(st[frame])
    saved_vol = ctx.download_volume(frame)
    saved_flow = ctx.download_flow(frame)
    with torch.cuda.stream(stream):
        vol = torch.from_numpy(saved_vol).cuda()
        flow = torch.from_numpy(saved_flow).cuda()
        img, ln, wt = (torch.zeros((d, d), device="cuda") for _ in range(3))
        out = torch.empty_like(vol)
        work = vol.clone()
    stream.synchronize()

    def timed(fn):
        fn()
        stream.synchronize()
        ts = []
        for _ in range(args.kernel_reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            stream.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    rows = []

    def row(name, ms, nbytes, **extra):
        gbs = nbytes / (ms / 1e3) / 1e9
        r = {"kernel": name, "ms_per_launch": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
             "frac": gbs / peak}
        r.update(extra)
        rows.append(r)

    ms = timed(lambda: ctx.forward(proj, vol, img, ln, wt))
    samples = float(wt.sum())
    row("fp (forward projection, brick-layout copy included)", ms, nv * 4 + 16 * D,
        samples=samples, gsamples_per_s=samples / ms / 1e6)
    cut = 8
    box = [cut, n - cut] * 3
    nroi = (n - 2 * cut) ** 3
    with torch.cuda.stream(stream):
        corr = ((img - img.mean()) * 1e-3).contiguous()
    for exact in (1, 0):
        ms = timed(lambda: ctx.backproject_voxel(proj, corr, box, 0, exact, work))
        row("bp_voxel exact (the reference's double arithmetic)" if exact else "bp_voxel FP32", ms,
            2 * nroi * 4 + 4 * D)
    ms = timed(lambda: ctx.advect([n] * 3, [0, n, 0, n, 0, n], flow, vol, 1, 0.5, out))
    row("advect", ms, nv * (2 * 4 + 3 * 4))
    win = int(en[frame]) - int(st[frame]) + 1
    ms = timed(lambda: ctx.sart_prox(frame, nb_sart=1, cut=cut, exact=1)) / win
    row("sart_step (exact BP; one SART sweep over the %d-projection window / %d)" % (win, win), ms,
        3 * nv * 4 + 20 * D)
    # One flow primal-dual iteration at this size with the GPU to itself: a
    # compute context on the bench's stream runs 60 iterations of a flow level
    # on the frame's volume pair, every tenth launch timed (in the timed region
    # the flow lanes run two pairs at once, so there a launch shares the GPU).
    pc = wap.Context(None, None)
    try:
        pc.set_stream(stream.cuda_stream)
        pc.set_profiling(True)
        with torch.cuda.stream(stream):
            I2 = torch.from_numpy(ctx.download_volume(frame + 1)).cuda()
            V = torch.zeros((3, n, n, n), device="cuda")
            Y = [torch.zeros((3, n, n, n), device="cuda") for _ in range(3)] + [torch.zeros((n, n, n), device="cuda")]
        stream.synchronize()
        pc.flow_level([n] * 3, vol, I2, V, *Y, 0.0, 0.05, 59, 1, [0, n, 0, n, 0, n], [8] * 6)
        pc.synchronize()
        st_pd = pc.stats()
        ms = st_pd.ms_pd / max(st_pd.pd_timed, 1)
        row("pd_iteration (one flow primal-dual iteration, the GPU to itself)", ms, PD_BYTES_MIN_PER_VOXEL * nv,
            launches_timed=int(st_pd.pd_timed))
        del V, Y, I2
    finally:
        pc.close()
    ctx.upload_volume(frame, saved_vol)
    return rows


def run_gb300(args):
    import torch
    import wap
    import build
    import replicas
    rank, world, local, dist = dist_init(args)
    torch.cuda.set_device(local)
    build.build()
    stream = torch.cuda.Stream()

    def factory(n, d, nproj, nframes, ang):
        c = wap.Context(wap.make_scan((n, n, n), (d, d), nproj, nframes_cli=nframes), ang, device=local)
        c.set_stream(stream.cuda_stream)
        return c

    with torch.cuda.stream(stream):
        ctx, projs, ang, meta = workload(args, torch, factory)
    F = meta["nframes"]
    ctx.set_projections_device(projs)
    ctx.set_tuning("flow_bits", args.flow_bits)
    ctx.set_tuning("flow_lanes", args.flow_lanes)
    ctx.level_setup(0)
    sched = wap.reference_schedule(n_cp=5, nb_sart=2, wp_frames=F, flow_iters=args.flow_iters,
                                   flow_scales=args.scales, flow_tol=0.008, cut=8, bp_exact=1)
    # Initial reconstruction (untimed): one CP + SART pass over all frames so the
    # flow solver sees structured volumes, as it does after the first pass.
    init = wap.reference_schedule(n_cp=1, nb_sart=1, wp_frames=0, flow_iters=0, flow_scales=1, cut=8, bp_exact=0)
    init.flow_warps = 0
    ctx.outer_iteration(init)
    ctx.set_profiling(True)
    n, d = args.n, args.det
    nv = n ** 3
    np_ = d * d
    # pinned host mirrors for the end-to-end leg
    h_projs = torch.empty((args.nproj, d, d), pin_memory=True)
    h_projs.copy_(projs)
    h_vol = torch.empty((n, n, n), pin_memory=True)
    h_flow = torch.empty((3, n, n, n), pin_memory=True)
    nf, st, en, ft, tu = wap.level_frames(ctx.scan, 0)

    # results of a step go back to pinned host memory (end-to-end leg)
    def d2h(f):
        ctx.call("wap_frame_volume_download", f, h_vol.data_ptr())
        ctx.call("wap_frame_flow_download", f, h_flow.data_ptr())

    FS = args.frames_per_step
    order = replicas.frame_order(rank, args.warmup + args.steps, F, span=FS)
    for i in range(args.warmup):
        f = order[i]
        with torch.cuda.stream(stream):
            projs[int(st[f]):int(en[f + FS - 1]) + 1].copy_(h_projs[int(st[f]):int(en[f + FS - 1]) + 1],
                                                           non_blocking=True)
        ctx.outer_iteration_frames(sched, f, f + FS)
        for g in range(f, f + FS):
            d2h(g)
    stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t_dev, t_e2e = 0.0, 0.0
    agg = dict(pd_voxel_iters=0.0, advect_voxels=0.0, projections=0, backprojections=0, cp_frame_passes=0,
               kernel_launches=0, flow_pd_iterations=0, ms_pd=0.0, pd_timed=0, ms_cp=0.0, ms_flow=0.0, ms_wap=0.0)
    h2d_bytes = 0
    pd_vox = 0
    lev_ms = [0.0] * args.scales
    lev_its = [0] * args.scales
    for i in range(args.warmup, args.warmup + args.steps):
        f = order[i]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        s0, s1 = int(st[f]), int(en[f + FS - 1]) + 1
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            projs[s0:s1].copy_(h_projs[s0:s1], non_blocking=True)
            ev[1].record(stream)
        s = ctx.outer_iteration_frames(sched, f, f + FS)
        with torch.cuda.stream(stream):
            ev[2].record(stream)
            for g in range(f, f + FS):
                d2h(g)
            ev[3].record(stream)
        stream.synchronize()
        t_dev += ev[1].elapsed_time(ev[2]) / 1e3
        t_e2e += ev[0].elapsed_time(ev[3]) / 1e3
        h2d_bytes += (s1 - s0) * np_ * 4
        for k in agg:
            agg[k] += getattr(s, k)
        for l in range(args.scales):
            lev_ms[l] += s.ms_flow_level[l]
            lev_its[l] += s.pd_iters_level[l]
        pd_vox = max(pd_vox, s.pd_timed_voxels)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        import torch.distributed as tdist
        t_dev, t_e2e = replicas.max_over_ranks([t_dev, t_e2e], tdist, device="cuda")
        tdist.barrier()
    K = args.steps
    value = replicas.aggregate_rate(world, K * FS / F, t_dev)
    pd_side = round(pd_vox ** (1.0 / 3.0))
    form, zchunk = ctx.get_tuning([pd_side] * 3)
    level_plans = [list(ctx.get_tuning([int(n * 0.5 ** l)] * 3)) for l in range(args.scales)]
    precision = None
    if world == 1 and args.precision_steps > 0 and args.flow_bits == 32:
        # The same frame-steps again in the precision form: the flow solver's
        # state in FP16 with its fast arithmetic, and the FP32 backprojection.
        ctx.set_tuning("flow_bits", 16)
        sched16 = wap.reference_schedule(n_cp=5, nb_sart=2, wp_frames=F, flow_iters=args.flow_iters,
                                         flow_scales=args.scales, flow_tol=0.008, cut=8, bp_exact=0)
        t16 = 0.0
        porder = replicas.frame_order(rank, args.warmup + args.steps + args.precision_steps, F, span=FS)
        for i in range(args.warmup, args.warmup + args.precision_steps):
            f = porder[args.steps + i]  # frames after the timed ones
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
            ctx.outer_iteration_frames(sched16, f, f + FS)
            with torch.cuda.stream(stream):
                e1.record(stream)
            stream.synchronize()
            t16 += e0.elapsed_time(e1) / 1e3
        ctx.set_tuning("flow_bits", 32)
        v16 = replicas.aggregate_rate(1, args.precision_steps * FS / F, t16)
        # Accuracy from identical state: one frame-step of a 3-frame scan of the
        # same size in both arithmetics (precision_compare.py).
        import precision_compare
        acc = precision_compare.compare(torch, wap, n, d, args.nproj, args.flow_iters, args.scales)
        precision = {"flow_bits": 16, "value": v16, "unit": "outer-iter/s", "ms_per_step": t16 / args.precision_steps * 1e3,
                     "speedup_vs_fp32": v16 / value,
                     "accuracy_from_identical_state": {
                         "workload": "one frame-step of a 3-frame %d^3 foam-and-smoke scan (%d proj at %d^2), both "
                                     "arithmetics from the same state (precision_compare.py)" % (n, args.nproj, d),
                         "speedup": acc["precision_form"]["speedup"],
                         "pd_iterations": {"reference_arithmetic": acc["reference_arithmetic"]["pd_iterations"],
                                           "precision_form": acc["precision_form"]["pd_iterations"]},
                         "volume_rel_l2_vs_reference_arithmetic":
                             acc["precision_form"]["volume_rel_l2_vs_reference_arithmetic"],
                         "flow_rel_l2_vs_reference_arithmetic":
                             acc["precision_form"]["flow_rel_l2_vs_reference_arithmetic"]},
                     "note": "frame-steps of the frames after the timed ones, with the flow solver's dual, flow and "
                             "linearisation stored in FP16 (FP32 fused multiply-adds and hardware reciprocals in the "
                             "primal-dual iteration; its residual compares the stored states, so a level stops once "
                             "the FP16 state no longer moves by the tolerance), the projector reading FP16 brick "
                             "copies with Kahan-compensated ray sums, and the FP32 backprojection in place of the "
                             "reference's double bicubic; at fixed iteration counts the volume is 1.5e-4 and the "
                             "flow 1.1e-3 from the FP64 oracle at 256^3 "
                             "(tests/test_baseline_configs.py::test_256_precision_form_against_fp64_oracle)"}
    e2e = replicas.aggregate_rate(world, K * FS / F, t_e2e)
    pd_ms = agg["ms_pd"] / max(agg["pd_timed"], 1)
    achieved = PD_BYTES_MIN_PER_VOXEL * pd_vox / (pd_ms / 1e3) / 1e9
    contract = PD_BYTES_PER_VOXEL * pd_vox / (pd_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    kernels = None
    if rank == 0 and args.kernel_reps > 0:
        kernels = kernel_table(ctx, torch, stream, args, order[args.warmup], peak)
    pd_alone = next((r for r in (kernels or []) if r["kernel"].startswith("pd_iteration")), None)
    full = None
    if args.full_outer:
        # One whole outer iteration, all frames in pass order (CP passes over all
        # frames, every flow pair, the warp-and-project pass), timed directly.
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.time()
        with torch.cuda.stream(stream):
            e0.record(stream)
        so = ctx.outer_iteration(sched)
        with torch.cuda.stream(stream):
            e1.record(stream)
        stream.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        full = {"seconds": sec, "value": 1.0 / sec, "unit": "outer-iter/s", "wall_seconds": time.time() - w0,
                "pd_iterations": int(so.flow_pd_iterations), "phase_ms": {"cp_sart": so.ms_cp, "flow": so.ms_flow,
                                                                         "wap": so.ms_wap},
                "pd_iterations_per_level": [int(so.pd_iters_level[l]) for l in range(args.scales)],
                "op_counts": {k: float(getattr(so, k)) for k in COUNT_KEYS},
                "note": "one wap_outer_iteration over all %d frames, CUDA events on the library's stream" % F}
        if rank == 0 and args.save_outer_counts:
            with open(args.save_outer_counts, "w") as f:
                json.dump({"workload": bench_config(args, F)["workload"],
                           "made_by": "python bench.py --full-outer --save-outer-counts <file> (one GB300)",
                           "outer_iteration_seconds": sec, "pd_iterations": full["pd_iterations"],
                           "pd_iterations_per_level_finest_first": full["pd_iterations_per_level"],
                           "op_counts": full["op_counts"]}, f, indent=1)
                f.write("\n")
    result = {
        "metric": METRIC, "value": value, "unit": "outer-iter/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": t_dev / K * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded foam phantom, RBF+compression, Poisson I0=1e4)",
        "config": dict(bench_config(args, F), parallelism="replicas" if world > 1 else "single"),
        "e2e": {"value": e2e, "unit": "outer-iter/s", "h2d_bytes_per_step": h2d_bytes // K,
                "d2h_bytes_per_step": FS * 4 * nv * 4},
        "gpu_launches": int(agg["kernel_launches"]),
        "roofline": {"kernel": "one flow primal-dual iteration at %d^3: %s (z-chunk %d, autotuned)"
                               % (pd_side, PD_FORMS.get(form, "?"), zchunk), "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": PD_TRAFFIC_256.get(form) if pd_side == 256 else None,
                     "traffic_source": ("ncu capture, %s" % PD_TRAFFIC_SOURCE[form])
                     if pd_side == 256 and form in PD_TRAFFIC_SOURCE else None,
                     "algorithmic_bytes": PD_BYTES_MIN_PER_VOXEL * pd_vox, "bytes_per_voxel": PD_BYTES_MIN_PER_VOXEL,
                     "contract_bytes_per_voxel": PD_BYTES_PER_VOXEL, "contract_achieved": contract,
                     "contract_frac": contract / peak,
                     "note": "achieved counts the 120 B/voxel a single-pass iteration must move (read and write the "
                             "dual y (10 words) and the flow v (3) once, read the linearisation u (4)); the "
                             "two-kernel contract figure, 208 B/voxel, is kept as contract_*",
                     "ms_per_launch": pd_ms, "launches_timed": int(agg["pd_timed"]),
                     "alone": ({"ms_per_launch": pd_alone["ms_per_launch"], "achieved": pd_alone["achieved_gbs"],
                                "frac": pd_alone["frac"],
                                "note": "the same kernel with the GPU to itself (60 iterations of a flow level on the "
                                        "run's frame pair, every tenth launch timed); in the timed region the flow "
                                        "lanes run two pairs at once, so a launch there shares the GPU with the other "
                                        "pair's work and takes longer while the step as a whole finishes sooner"}
                               if pd_alone else None)},
        "phase_ms_per_step": {"cp_sart": agg["ms_cp"] / K, "flow": agg["ms_flow"] / K, "wap": agg["ms_wap"] / K},
        "pd_iterations_per_step": agg["flow_pd_iterations"] / K,
        "flow_levels_finest_first": {"sides": [int(n * 0.5 ** l) for l in range(args.scales)],
                                     "ms_per_step": [v / K for v in lev_ms],
                                     "pd_iterations_per_step": [v / K for v in lev_its],
                                     "pd_form_and_zchunk": level_plans},
        "op_counts_per_outer_iteration": {k: agg[k] * F / (K * FS) for k in ("projections", "backprojections",
                                                                       "advect_voxels", "cp_frame_passes",
                                                                       "pd_voxel_iters")},
        "clocks": clk,
    }
    if kernels:
        result["kernels"] = kernels
    if full:
        result["full_outer_iteration"] = full
    if precision:
        result["precision_form"] = precision
    if args.flow_bits == 16:
        result["dtype"] = "f32 arithmetic, f16 flow state"
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        counts = outer_counts(args)
        source = "measured counts of one whole outer iteration (%s)" % os.path.relpath(OUTER_COUNTS, REPO)
        if counts is None:
            counts = {k: agg[k] * F / (K * FS) for k in COUNT_KEYS}
            counts["pd_iterations_per_level"] = [x * F / (K * FS) for x in lev_its]
            source = "counts of the timed frame-steps, times frames / steps"
        threads = os.cpu_count() or 1
        w0 = time.time()
        sec, parts, sample = cpu_sample(args, counts, threads)
        result["cpu_baseline"] = {"value": 1.0 / sec, "unit": "outer-iter/s", "cores": threads, "kind": "port",
                                  "sample": sample + "; " + source, "sample_seconds": time.time() - w0,
                                  "composed_seconds_per_outer_iteration": sec, "component_seconds": parts}
    if rank == 0 and world == 1 and (args.serve_jobs > 0 or args.batch_jobs > 0):
        del projs
        ctx.close()
        torch.cuda.empty_cache()
    if rank == 0 and world == 1 and args.serve_jobs > 0:
        # Served form: p50/p95/p99 latency of a Poisson job stream through the
        # request loop (see serving.py for the job mix).
        # The same stream twice: the reference's arithmetic, then the precision
        # form (flow_bits 16 per job).
        import serving
        result["serving"], result["serving_precision"] = serving.run(
            wap, torch, n_jobs=args.serve_jobs, rate=args.serve_rate, workers=args.serve_workers, flow_bits=(32, 16))
    if rank == 0 and world == 1 and args.batch_jobs > 0:
        # Batched form: uneven scans looped through the plain path vs reconstructed
        # together through wap_batch (same results, checked).
        import serving
        result["batched"] = serving.run_batched(wap, torch, n_jobs=args.batch_jobs, flow_iters=args.batch_flow_iters)
    if rank == 0:
        print(json.dumps(result))
    if dist:
        import torch.distributed as tdist
        tdist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle as O
    orc = O.Oracle()
    F = args.nproj // 4
    counts = outer_counts(args)
    source = "measured counts of one whole outer iteration (%s)" % os.path.relpath(OUTER_COUNTS, REPO)
    if counts is None:
        # Op counts of one outer iteration of the same schedule from its
        # structure (windows of <= 7, 5 CP x 2 SART, 3 warps, every flow level
        # at its iteration cap: an upper bound on the primal-dual work).
        nf, st, en, ft, tu = orc.level_frames(F, args.nproj, 0)
        win = (en - st + 1).astype(np.int64)
        nv = args.n ** 3
        lvl = sum((1.0 / 8 ** l) for l in range(args.scales))
        counts = {"projections": float(5 * 2 * win.sum() + win.sum()),
                  "backprojections": float(5 * 2 * win.sum() + win.sum()),
                  "advect_voxels": float(2 * win.sum() * nv + (F - 1) * 3 * lvl * nv),
                  "cp_frame_passes": float(5 * F),
                  "pd_voxel_iters": float((F - 1) * 3 * (args.flow_iters + 1) * lvl * nv),
                  "pd_iterations_per_level": [float((F - 1) * 3 * (args.flow_iters + 1))] * args.scales}
        source = "op counts from the schedule's structure, every flow level at its iteration cap"
    threads = os.cpu_count() or 1
    composed, walls, parts = [], [], None
    for i in range(args.warmup + args.steps):
        w0 = time.time()
        sec, parts, sample = cpu_sample(args, counts, threads)
        if i >= args.warmup:
            composed.append(sec)
            walls.append(time.time() - w0)
    sec = float(np.mean(composed))
    v = 1.0 / sec
    # A step is one bounded CPU sample of the workload (its wall time is
    # ms_per_step); value is outer-iter/s composed from the sample's component
    # times and the op counts of one outer iteration.
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "outer-iter/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(walls)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, F),
        "cpu_baseline": {"value": v, "unit": "outer-iter/s", "cores": threads, "kind": "port",
                         "sample": sample + "; " + source, "composed_seconds_per_outer_iteration": sec,
                         "component_seconds": parts},
        "e2e": {"value": v, "unit": "outer-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gb300(a)
