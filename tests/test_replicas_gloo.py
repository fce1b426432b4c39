"""Multi-rank bookkeeping on CPU (gloo, world size 2): each rank runs an
independent replica job through the oracle, the job time is the max over
ranks, and every rank's result equals the same job run alone."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _job(seed):
    sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
    sys.path.insert(0, HERE)
    import oracle as O
    import phantoms as P
    orc = O.Oracle()
    N, W, NP = 20, 24, 6
    vol = P.ellipsoids(N, count=5, seed=seed)
    ang = P.golden_angles(NP)
    scan = O.make_scan((N, N, N), (W, W), NP, gmax=2.0, threads=1)
    projs = np.stack([orc.forward(scan, a, vol)[0] for a in ang]).astype(np.float32)
    out, _ = orc.sart_prox(scan, ang, projs, 0, NP - 1, 1, [4, N - 4] * 3, np.zeros_like(vol))
    return out


def _worker(rank, world, port, q):
    import time

    import torch.distributed as dist
    sys.path.insert(0, os.path.join(HERE, "..", "warp-and-project-tomography_gb300"))
    import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t0 = time.time()
    out = _job(replicas.job_seed(rank, 50))
    dt = time.time() - t0 + 0.01 * rank
    tmax = replicas.max_over_ranks([dt], dist)[0]
    order = replicas.frame_order(rank, 4, 48)
    q.put((rank, float(out.sum()), dt, tmax, order))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=300) for _ in range(2)])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, os.path.join(HERE, "..", "warp-and-project-tomography_gb300"))
    import replicas
    for rank, checksum, dt, tmax, order in res:
        alone = _job(replicas.job_seed(rank, 50))
        assert checksum == pytest.approx(float(alone.sum()), rel=0, abs=0)
        assert tmax == pytest.approx(max(r[2] for r in res))
        assert all(0 <= f < 47 for f in order)
    assert res[0][4] != res[1][4]
    assert replicas.aggregate_rate(2, 3, 1.5) == pytest.approx(4.0)
