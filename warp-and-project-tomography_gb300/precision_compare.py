"""The precision form against the reference arithmetic on one frame's share
of an outer iteration, from identical state: seconds in both arithmetics and
the precision form's distance from the reference arithmetic.  The default is
the precision configuration, 512^3 x 768^2; bench.py runs it at the
benchmark's 256^3 x 384^2 for its precision line's accuracy.

Workload (seeded, generated on the GPU): an n^3 foam (band-limited noise
thresholded at the 70th percentile: struts of density 1.0) overlaid with a
smoke-like density from 3 octaves of value noise in [0, 0.6] (the larger of
the two per voxel), moved by a divergence-free curl-noise velocity field of
at most 8 voxels per frame; cone-beam projections on golden-ratio angles; 3
frames (each frame's volume is the phantom advanced by its frame index), 1 %
Gaussian noise on the projections of the run frame's window.  Schedule:
PSART's 5 CP x 2 SART, a 4-level flow (tolerance 0.008, at most --flow-iters
iterations, 3 warps), warp-and-project over the window.

Reports JSON: seconds per frame-step in both arithmetics (each after an
untimed short run that tunes the primal-dual plans of every pyramid level),
their primal-dual iteration counts, and the precision form's relative L2
distance from the reference arithmetic for the frame's volume and flow.  The
projector at 512^3 is compared with the FP64 oracle in
tests/test_baseline_configs.py.

    python precision_compare.py [--n 512] [--det 768] [--nproj 360] [--flow-iters 3000]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
for _p in (HERE,):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def value_noise(torch, n, cells, gen):
    """Smooth noise in [0, 1]: a random lattice of cells^3 values, upsampled
    trilinearly to n^3."""
    lat = torch.rand((1, 1, cells, cells, cells), device="cuda", generator=gen)
    return torch.nn.functional.interpolate(lat, size=(n, n, n), mode="trilinear", align_corners=True)[0, 0]


def phantom(torch, n, seed=0):
    gen = torch.Generator(device="cuda").manual_seed(seed)
    w = torch.randn((n, n, n), device="cuda", generator=gen)
    k = torch.fft.fftfreq(n, device="cuda")
    kz, ky, kx = torch.meshgrid(k, k, k, indexing="ij")
    b = torch.fft.ifftn(torch.fft.fftn(w) * ((kx ** 2 + ky ** 2 + kz ** 2) <= (1.0 / 16) ** 2)).real
    del w, kz, ky, kx
    thr = torch.quantile(b.flatten()[::97].float(), 0.7)
    foam = (b > thr).float()
    del b
    smoke = torch.zeros((n, n, n), device="cuda")
    for o, cells in enumerate((8, 16, 32)):
        smoke += value_noise(torch, n, cells, gen) * 0.5 ** o
    smoke = 0.6 * (smoke - smoke.min()) / (smoke.max() - smoke.min())
    return torch.maximum(foam, smoke).contiguous()


def curl_velocity(torch, n, vmax=8.0, seed=1):
    """Divergence-free velocity: the curl (central differences) of a smooth
    random vector potential, scaled to a largest component of vmax."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    A = [value_noise(torch, n, 6, gen) for _ in range(3)]

    def d(f, axis):  # central difference along x (2), y (1) or z (0) of a [z, y, x] volume
        return (torch.roll(f, -1, axis) - torch.roll(f, 1, axis)) * 0.5

    vx = d(A[2], 1) - d(A[1], 0)
    vy = d(A[0], 0) - d(A[2], 2)
    vz = d(A[1], 2) - d(A[0], 1)
    v = torch.stack([vx, vy, vz])
    return (v * (vmax / v.abs().max())).contiguous()


def compare(torch, wap, n=512, d=768, P=360, flow_iters=3000, scales=4):
    """One frame-step in the reference arithmetic and in the precision form,
    from the same state; returns the report dict."""
    F, frame = 3, 1
    ang = (np.arange(P, dtype=np.float64) * 360.0 * 0.6180339887) % 360.0
    ctx = wap.Context(wap.make_scan((n, n, n), (d, d), P, nframes_cli=F), ang)
    out = {"volume": n, "detector": d, "projections": P, "frames": F, "flow_iters": flow_iters, "scales": scales}
    try:
        t0 = time.time()
        base = phantom(torch, n)
        vel = curl_velocity(torch, n)
        aabb = [0, n, 0, n, 0, n]
        vols = []
        for f in range(F):
            o = torch.empty_like(base)
            torch.cuda.synchronize()
            ctx.advect([n] * 3, aabb, vel, base, 1, float(f), o)
            ctx.synchronize()
            vols.append(o)
        del vel
        nf, st, en, ft, tu = wap.level_frames(ctx.scan, 0)
        need = [0] + list(range(int(st[frame]), int(en[frame]) + 1))
        projs = torch.zeros((P, d, d), device="cuda")
        torch.cuda.synchronize()  # the context's stream does not wait on torch's
        for k in need:
            ctx.forward(k, vols[frame], projs[k])
        ctx.synchronize()
        gen = torch.Generator(device="cuda").manual_seed(2)
        scale = 0.01 * float(projs.max())
        for k in need:
            projs[k] += torch.randn((d, d), device="cuda", generator=gen) * scale
        torch.cuda.synchronize()
        ctx.set_projections_device(projs)
        out["generation_s"] = time.time() - t0
        host_vols = [v.cpu().numpy() for v in vols]

        def frame_step(bits, exact, iters):
            ctx.set_tuning("flow_bits", bits)
            ctx.level_setup(0)
            for f in range(F):
                ctx.upload_volume(f, host_vols[f])
            sched = wap.reference_schedule(n_cp=5, nb_sart=2, wp_frames=F, flow_iters=iters,
                                           flow_scales=scales, flow_tol=0.008, cut=8, bp_exact=exact)
            ctx.synchronize()
            w0 = time.time()
            s = ctx.outer_iteration_frames(sched, frame, frame + 1)
            ctx.synchronize()
            sec = time.time() - w0
            res = (ctx.download_volume(frame), ctx.download_flow(frame))
            ctx.set_tuning("flow_bits", 32)
            return sec, s, res

        frame_step(32, 1, 2)  # untimed: tunes each level's primal-dual plan in both arithmetics
        frame_step(16, 0, 2)
        sec32, s32, r32 = frame_step(32, 1, flow_iters)
        sec16, s16, r16 = frame_step(16, 0, flow_iters)

        def rel(x, y):
            x, y = x.astype(np.float64), y.astype(np.float64)
            return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30))

        out["reference_arithmetic"] = {"seconds": sec32, "pd_iterations": int(s32.flow_pd_iterations),
                                       "ms_cp": s32.ms_cp, "ms_flow": s32.ms_flow, "ms_wap": s32.ms_wap}
        out["precision_form"] = {"seconds": sec16, "pd_iterations": int(s16.flow_pd_iterations),
                                 "ms_cp": s16.ms_cp, "ms_flow": s16.ms_flow, "ms_wap": s16.ms_wap,
                                 "speedup": sec32 / sec16,
                                 "volume_rel_l2_vs_reference_arithmetic": rel(r16[0], r32[0]),
                                 "flow_rel_l2_vs_reference_arithmetic": rel(r16[1], r32[1])}
    finally:
        ctx.close()
    return out


def main():
    import torch

    import build
    import wap
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--det", type=int, default=768)
    ap.add_argument("--nproj", type=int, default=360)
    ap.add_argument("--flow-iters", type=int, default=3000)
    ap.add_argument("--scales", type=int, default=4)
    a = ap.parse_args()
    build.build()
    print(json.dumps(compare(torch, wap, a.n, a.det, a.nproj, a.flow_iters, a.scales)))


if __name__ == "__main__":
    main()
