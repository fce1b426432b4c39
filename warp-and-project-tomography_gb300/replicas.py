"""Replica bookkeeping for multi-GPU runs.

The warp-and-project hot path has no exchange step a single scan needs
across GPUs at this tier: each GPU runs an independent replica (its own scan,
or its own share of frames of a long scan) and the job-wide throughput is
the total work over the slowest rank's time.  This module holds that logic
so the benchmark and its CPU (gloo) tests use the same code.
"""
import os


def env_rank():
    """(rank, world, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def frame_order(rank, count, nframes, stride=7, span=1):
    """First frames of the steps a rank streams, a step covering `span`
    consecutive frames each of which starts a flow pair: a rank-specific
    rotation over the frames f with f + span < nframes, advancing by span, so
    that replicas work on different data."""
    starts = max(1, nframes - span)
    return [(rank * stride + i * span) % starts for i in range(count)]


def job_seed(rank, base=0):
    """Seed of the synthetic scan a replica reconstructs."""
    return base + 1000 * rank


def max_over_ranks(values, dist=None, device=None):
    """Element-wise max of a list of floats over all ranks (the slowest rank's
    time defines the job's time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return list(values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def aggregate_rate(world, units_per_rank, seconds_max):
    """Job-wide throughput: all ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds_max
