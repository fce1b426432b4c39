"""Speed of the oracle port against the reference's own compiled code, on the
same host and thread count: how representative the port is as the CPU
baseline.  Test infrastructure: it needs the reference build in oracle/_ref
(built from the reference's sources by `make ref`), so it runs where those
sources are, not on the GPU machine.

Times, at one size (default 256^3 volume, 384^2 detector, 192 projections,
4 frames so that the reference's session stays a few GB):
  forward   one cone-beam projection of a frame's volume (all threads)
  sart      one SART sweep over a frame's projection window (projection,
            correction, voxel-driven bicubic backprojection per projection),
            reported per projection, on one thread: the reference's SART
            corrupts its heap when its OpenMP loops run on several threads
            (built with gcc here), so both sides run it single-threaded
  advect    one warp of a volume by a smooth flow (4 threads: the reference's
            advect hard-codes 4 worker threads, advection.h:134-141)
  flow      --flow-iters primal-dual iterations of one flow level (1 warp,
            all threads), the second of two calls (warm allocator)

    python oracle/reference_speed.py [--n 256] [--det 384] [--nproj 192] [--flow-iters 20] [--threads 0]

Prints one JSON object: seconds per component for the port and the reference
and their ratio (reference / port).
"""
import argparse
import ctypes
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402


def smooth_volume(n, seed):
    """Seeded smooth random volume in [0, 1] (block-averaged noise)."""
    rng = np.random.default_rng(seed)
    c = max(n // 8, 2)
    lat = rng.random((c + 1, c + 1, c + 1)).astype(np.float32)
    idx = np.minimum(np.arange(n) * c // n, c)
    v = lat[np.ix_(idx, idx, idx)]
    return np.ascontiguousarray(v, np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--det", type=int, default=384)
    ap.add_argument("--nproj", type=int, default=192)
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--flow-iters", type=int, default=20)
    ap.add_argument("--threads", type=int, default=0, help="OpenMP threads (0: all)")
    a = ap.parse_args()
    T = a.threads if a.threads > 0 else os.cpu_count()
    n, d, P, F = a.n, a.det, a.nproj, a.frames
    orc = O.Oracle()
    ref = O.Reference()
    gomp = ctypes.CDLL("libgomp.so.1")  # the OpenMP runtime both libraries use
    scan = O.make_scan((n, n, n), (d, d), P, nframes_cli=F, threads=T)
    scan1 = O.make_scan((n, n, n), (d, d), P, nframes_cli=F, threads=1)
    ang = (np.arange(P, dtype=np.float64) * 360.0 * 0.6180339887) % 360.0
    vol = smooth_volume(n, 0)
    nf, st, en, ft, tu = orc.level_frames(F, P, 0)
    frame = 1
    p0, p1 = int(st[frame]), int(en[frame])
    projs = np.zeros((P, d, d), np.float32)
    for k in range(p0, p1 + 1):
        projs[k] = orc.forward(scan, ang[k], vol)[0]
    out = {"volume": n, "detector": d, "projections": P, "frames": F, "window": [p0, p1],
           "threads": T, "port": {}, "reference": {}}
    with tempfile.TemporaryDirectory() as wd:
        gomp.omp_set_num_threads(T)
        gmax = ref.create(scan, projs, ang, wd)
        scan.gmax = scan1.gmax = gmax
        ref.lib.wref_set_volume(0, frame, vol)
        img = np.zeros((d, d), np.float32)
        ln = np.zeros_like(img)
        wt = np.zeros_like(img)
        # forward projection
        t0 = time.time()
        orc.forward(scan, ang[p0], vol)
        out["port"]["forward"] = time.time() - t0
        t0 = time.time()
        ref.lib.wref_forward(0, frame, p0, 0, 0.0, img, ln, wt)
        out["reference"]["forward"] = time.time() - t0
        # one SART sweep over the window
        box = np.array([8, n - 8] * 3, np.int32)
        v = vol.copy()
        t0 = time.time()
        orc.sart_prox(scan1, ang, projs, p0, p1, 1, box, v)
        out["port"]["sart_per_projection_1_thread"] = (time.time() - t0) / (p1 - p0 + 1)
        gomp.omp_set_num_threads(1)
        t0 = time.time()
        ref.lib.wref_sart_prox(0, frame, 1, 1)
        out["reference"]["sart_per_projection_1_thread"] = (time.time() - t0) / (p1 - p0 + 1)
        gomp.omp_set_num_threads(T)
        # warp by a smooth flow
        flow = (np.stack([smooth_volume(n, s) for s in (3, 4, 5)]) * 6.0 - 3.0).astype(np.float32)
        aabb = np.array([0, n, 0, n, 0, n], np.float32)
        dims = np.array([n, n, n], np.int32)
        t0 = time.time()
        warped = orc.advect([n] * 3, aabb, flow, vol, 0.5, 4)
        out["port"]["advect"] = time.time() - t0
        wout = np.zeros_like(vol)
        t0 = time.time()
        ref.lib.wref_advect(dims, aabb, flow, vol, 1, 0.5, wout)
        out["reference"]["advect"] = time.time() - t0
        out["advect_same_bits"] = bool(np.array_equal(wout, warped.reshape(wout.shape)))
        gomp.omp_set_num_threads(T)
        # one flow level on a deforming pair
        I2 = np.ascontiguousarray(warped.reshape(vol.shape))
        roi = np.array([8] * 6, np.int32)
        its = a.flow_iters

        def state():
            return (np.zeros((3, n, n, n), np.float32),
                    [np.zeros((3, n, n, n), np.float32) for _ in range(3)] + [np.zeros((n, n, n), np.float32)])

        # each flow level twice, timing the second call: the first one's
        # allocations of about 40 volume-sized work arrays page in fresh memory,
        # which costs more than the iterations on some hosts
        for rep in range(2):
            V, Y = state()
            t0 = time.time()
            orc.flow_level([n] * 3, vol, I2, V, *Y, 0.0, 0.05, its - 1, 1, aabb, list(roi), deterministic=0)
            out["port"]["flow_level"] = time.time() - t0
            out["port_flow_pd_loop_seconds"] = orc.lib.orc_last_pd_seconds()
            Vr, Yr = state()
            t0 = time.time()
            ref.lib.wref_flow_level(dims, vol, I2, Vr, *Yr, 0.0, 0.05, its - 1, 1, aabb, roi)
            out["reference"]["flow_level"] = time.time() - t0
        out["flow_same_bits"] = bool(np.array_equal(V, Vr))
        ref.lib.wref_destroy()
    out["flow_iterations"] = its
    out["ratio_reference_over_port"] = {k: out["reference"][k] / out["port"][k] for k in out["port"]}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
