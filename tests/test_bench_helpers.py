"""bench.py's host-side helpers: the workload config both arms print, and the
op counts of one measured outer iteration that the CPU legs compose with."""
import argparse
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _defaults(**kw):
    a = argparse.Namespace(n=256, det=384, nproj=192, scales=4, flow_iters=3000)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_outer_counts_file_matches_the_default_workload():
    c = bench.outer_counts(_defaults())
    assert c is not None, "the committed counts of one outer iteration are missing"
    for k in bench.COUNT_KEYS:
        assert c[k] > 0, k
    per_level = c["pd_iterations_per_level"]
    assert len(per_level) == 4 and all(x > 0 for x in per_level)
    with open(bench.OUTER_COUNTS) as f:
        d = json.load(f)
    assert d["workload"] == bench.bench_config(_defaults(), 48)["workload"]
    assert sum(per_level) == d["pd_iterations"]
    # PD voxel-iterations = sum over levels of iterations x that level's voxels
    # (256^3, 128^3, 64^3, 32^3)
    assert c["pd_voxel_iters"] == pytest.approx(sum(i * (256 >> l) ** 3 for l, i in enumerate(per_level)), rel=1e-9)


def test_outer_counts_only_for_the_default_workload():
    assert bench.outer_counts(_defaults(n=128)) is None
    assert bench.outer_counts(_defaults(flow_iters=300)) is None


def test_both_arms_share_the_config_object():
    cfg = bench.bench_config(_defaults(), 48)
    assert cfg["volume"] == [256] * 3 and cfg["detector"] == [384] * 2 and cfg["projections"] == 192
    assert cfg["frames"] == 48 and "workload" in cfg
    small = bench.bench_config(_defaults(n=64, det=96, nproj=64), 16)
    assert small["workload"].startswith("64^3 volume, 64 proj at 96^2, 16 frames")
