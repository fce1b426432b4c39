"""Per-kernel micro-benchmark of the GB300 library (device-resident inputs,
CUDA-event timing on the library's stream).

    python kernel_bench.py --kernel pd --n 256 --iters 100 [--pd-form 0|1|2|3]
    python kernel_bench.py --kernel fp|bp|bp_exact|bp_ray|advect|all --n 256 --det 384

Prints one JSON line per kernel: milliseconds per launch and the achieved
bandwidth against the kernel's algorithmic bytes:
  pd      one fused primal-dual iteration, 120 B per voxel (y 10+10, v 3+3, u 4);
          62 B per voxel in the precision form (--flow-bits 16, FP16 pairs)
  fp      forward projection, V*4 + 16*D bytes (volume once, 4 outputs per pixel)
  bp      voxel-driven backprojection over the ROI, 2*V*4 + 4*D bytes
  advect  one warp of a 1-channel volume by a smooth 3-channel flow, V*(2+3)*4 bytes
  bp_ray  ray-driven matched backprojection (contribution and weight sums,
          read and written once each: 16*V + 4*D bytes), --splat-form 1 for the
          one-global-atomic-per-tap form
Used to make the per-kernel ncu captures summarised under profiles/.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def main():
    import torch

    import build
    import wap
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", default="all", choices=["pd", "fp", "bp", "bp_exact", "bp_ray", "advect", "all"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--det", type=int, default=384)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--pd-form", type=int, default=0, help="0 autotuned, 1 fused, 2 primal+dual, 3 TMA-fed fused")
    ap.add_argument("--pd-zchunk", type=int, default=0)
    ap.add_argument("--flow-bits", type=int, default=32, help="16: the precision form (FP16 flow state)")
    ap.add_argument("--splat-form", type=int, default=0, help="1: one global atomic per tap in the ray-driven splat")
    ap.add_argument("--fp-bricks", type=int, default=1, help="0: the projector reads the linear volume (1: brick-layout copy)")
    a = ap.parse_args()
    build.build()
    n, d = a.n, a.det
    ang = (np.arange(16) * 360.0 * 0.6180339887) % 360.0
    ctx = wap.Context(wap.make_scan((n, n, n), (d, d), 16), ang)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)
    peak = None
    try:
        with open(os.path.join(HERE, "..", "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        pass
    nv = n ** 3

    def timed(fn, reps):
        fn()
        stream.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            stream.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    def report(name, ms, nbytes, extra=None):
        gbs = nbytes / (ms / 1e3) / 1e9
        out = {"kernel": name, "n": n, "ms": ms, "algorithmic_bytes": nbytes, "gbs": gbs,
               "frac_of_measured_hbm": (gbs / peak) if peak else None}
        out.update(extra or {})
        print(json.dumps(out))

    with torch.cuda.stream(stream):
        vol = torch.rand((n, n, n), device="cuda", generator=g)
        projs = torch.rand((16, d, d), device="cuda", generator=g)
    ctx.set_projections_device(projs)
    ctx.set_tuning("fp_bricks", a.fp_bricks)
    if a.kernel in ("fp", "all"):
        img = torch.zeros((d, d), device="cuda")
        wt = torch.zeros_like(img)
        ln = torch.zeros_like(img)
        ms = timed(lambda: ctx.forward(3, vol, img, ln, wt), a.reps)
        stream.synchronize()
        report("fp", ms, nv * 4 + 16 * d * d, {"samples": float(wt.sum()), "gsamples_per_s": float(wt.sum()) / ms / 1e6})
    if a.kernel in ("bp", "bp_exact", "all"):
        corr = torch.rand((d, d), device="cuda", generator=g) * 1e-3
        v2 = vol.clone()
        box = [8, n - 8, 8, n - 8, 8, n - 8]
        nb = (n - 16) ** 3
        for exact in ([1] if a.kernel == "bp_exact" else [0] if a.kernel == "bp" else [0, 1]):
            ms = timed(lambda: ctx.backproject_voxel(3, corr, box, 0, exact, v2), a.reps)
            report("bp_exact" if exact else "bp", ms, 2 * nb * 4 + 4 * d * d)
    if a.kernel in ("bp_ray", "all"):
        ctx.set_tuning("splat_form", a.splat_form)
        corr = torch.rand((d, d), device="cuda", generator=g) - 0.5
        con = torch.zeros((n, n, n), device="cuda")
        wsum = torch.zeros_like(con)
        ms = timed(lambda: ctx.backproject_ray(3, corr, con, wsum), a.reps)
        report("bp_ray", ms, 16 * nv + 4 * d * d, {"splat_form": a.splat_form})
    if a.kernel in ("advect", "all"):
        # a smooth flow of up to 4 voxels (a random 8^3 lattice interpolated
        # trilinearly), like the displacement fields the solver warps by
        lat = torch.rand((3, 1, 8, 8, 8), device="cuda", generator=g) * 8 - 4
        flow = torch.nn.functional.interpolate(lat, size=(n, n, n), mode="trilinear",
                                               align_corners=True)[:, 0].contiguous()
        out = torch.zeros((1, n, n, n), device="cuda")
        ms = timed(lambda: ctx.advect([n, n, n], [0, n, 0, n, 0, n], flow, vol, 1, 0.7, out), a.reps)
        report("advect", ms, nv * 5 * 4)
    if a.kernel in ("pd", "all"):
        I1 = torch.rand((n, n, n), device="cuda", generator=g)
        I2 = torch.rand((n, n, n), device="cuda", generator=g)
        V = torch.randn((3, n, n, n), device="cuda", generator=g)
        Y = [torch.zeros((3, n, n, n), device="cuda") for _ in range(3)] + [torch.zeros((n, n, n), device="cuda")]
        ctx.set_profiling(True)
        ctx.set_tuning("pd_form", a.pd_form)
        ctx.set_tuning("pd_zchunk", a.pd_zchunk)
        ctx.set_tuning("flow_bits", a.flow_bits)
        its = ctx.flow_level([n, n, n], I1, I2, V, *Y, 0.0, 0.05, a.iters - 1, 1, [0, n, 0, n, 0, n], [8] * 6)
        st = ctx.stats()
        ms = st.ms_pd / max(st.pd_timed, 1)
        form, zc = ctx.get_tuning([n, n, n])
        # bytes moved once per iteration: FP32 state 120 B/voxel; the precision
        # form's FP16 pairs 62 B/voxel (v's third component padded)
        report("pd", ms, (62 if a.flow_bits == 16 else 120) * nv, {"iterations": int(its[0]), "form": form,
                                                                    "zchunk": zc})
    ctx.close()


if __name__ == "__main__":
    main()
