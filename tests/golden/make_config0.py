"""Digests of the 64^3 CPU-runnable workload, computed by the oracle.

The workload: a 64^3 phantom of 20 ellipsoids deforming by a smooth RBF field
(largest component 3 voxels, scaled by t_k = k / 64), 64 cone-beam projections
at 96x96 on golden-ratio angles (source-axis 4x and source-detector 6x the
volume width), 1 % Gaussian noise; 16 frames (projections / 4), three outer
iterations of PSART's schedule: 5 Chambolle-Pock iterations of 2 SART sweeps
each (10 SART sweeps), a 3-level L1-TV flow (lambda 0.05, 3 warps, eta 0.5,
sigma 0.8) at the reference's 3000 primal-dual iterations per warp and level
with the stopping tolerance at 0 (a fixed count, so the OpenMP order of the
reference's residual sum cannot change the result), and warp-and-project over
every frame's window.  The inputs are generated with bit-reproducible
arithmetic (tests/phantoms.py), so their digest is recorded too.

Writes tests/golden/config0_digests.json: SHA-256 of the float32 bytes of
every frame's volume and flow after each outer iteration, plus float64 sums
for diagnosis.  Minutes to tens of minutes of CPU time (all cores):

    python tests/golden/make_config0.py [--flow-iters N] [--out FILE]
"""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, ".."))
import oracle as O  # noqa: E402
import phantoms as P  # noqa: E402

N, DET, NPROJ, FRAMES, OUTER = 64, 96, 64, 16, 3


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def schedule(flow_iters):
    """PSART's per-level schedule for this workload (oracle mirror)."""
    return dict(n_cp=5, nb_sart=2, nb_projwarp=1, wp_frames=FRAMES, flow_tol=0.0, flow_lambda=0.05,
                flow_iters=flow_iters, flow_warps=3, flow_eta=0.5, flow_sigma=0.8, flow_scales=3, cut=8)


def inputs():
    """(scan, projections, angles) of the workload, from the FP64 oracle projector."""
    scan = O.make_scan((N, N, N), (DET, DET), NPROJ, nframes_cli=FRAMES)
    projs, ang, _ = P.deforming_scan_64(O.Oracle(fp64=True), scan, n=N, nproj=NPROJ)
    return scan, projs, ang


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--flow-iters", type=int, default=3000)
    ap.add_argument("--out", default=os.path.join(HERE, "config0_digests.json"))
    a = ap.parse_args()
    orc = O.Oracle()
    scan, projs, ang = inputs()
    scan.gmax = float(projs[0].max())  # G_Max = max of the first projection image (WaP_Tomo.cpp:347-348)
    sch = O.Schedule(deterministic=0, **schedule(a.flow_iters))
    F = FRAMES
    nv = N ** 3
    state = dict(vols=np.zeros((F, N, N, N), np.float32), flows=np.zeros((F, 3, N, N, N), np.float32),
                 ytv=np.zeros((F, 3, N, N, N), np.float32), ytp=np.zeros((F, N, N, N), np.float32),
                 xbar=np.zeros((F, N, N, N), np.float32), xprev=np.zeros((F, N, N, N), np.float32))
    rec = {"workload": __doc__.split("\n\n")[1].replace("\n", " "), "schedule": schedule(a.flow_iters),
           "volume": N, "detector": DET, "projections": NPROJ, "frames": F, "gmax": scan.gmax,
           "inputs_sha256": digest(projs), "angles_sha256": hashlib.sha256(ang.tobytes()).hexdigest(),
           "iterations": []}
    for it in range(OUTER):
        t0 = time.time()
        Fo, tot = orc.outer_iteration(scan, sch, ang, projs, 0, state)
        assert Fo == F
        rec["iterations"].append({
            "pd_iterations": tot,
            "volumes": [digest(state["vols"][f]) for f in range(F)],
            "flows": [digest(state["flows"][f]) for f in range(F)],
            "volume_sums": [float(state["vols"][f].astype(np.float64).sum()) for f in range(F)],
            "flow_abs_sums": [float(np.abs(state["flows"][f].astype(np.float64)).sum()) for f in range(F)],
        })
        print("outer iteration %d: %.1f s, %d PD iterations" % (it + 1, time.time() - t0, tot), flush=True)
    with open(a.out, "w") as f:
        json.dump(rec, f, indent=1)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
