"""Host-side pieces of the served form that need no GPU: the seeded Poisson
job stream (sizes, projection counts and arrival times of the served
configuration) and the request loop's argument checks."""
import numpy as np

import serving


def test_job_stream_is_seeded_and_follows_the_mix():
    a = serving.job_stream(400, 20.0, seed=3)
    b = serving.job_stream(400, 20.0, seed=3)
    assert a == b
    t = np.array([j["t"] for j in a])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(len(a) / t[-1] - 20.0) < 3.0  # mean rate 20 jobs/s
    sides = np.array([j["n"] for j in a])
    assert set(sides) <= set(serving.SIZES) and set(j["nproj"] for j in a) <= set(serving.NPROJS)
    freq = np.array([np.mean(sides == s) for s in serving.SIZES])
    assert np.all(np.abs(freq - np.array(serving.WEIGHTS)) < 0.08)
    assert len({j["seed"] for j in a}) == len(a)


def test_job_stream_caps_the_side():
    assert max(j["n"] for j in serving.job_stream(200, 20.0, seed=3, max_side=128)) <= 128


def test_served_schedule(wapmod):
    s = serving.served_schedule(wapmod, 16)
    assert (s.n_cp, s.nb_sart, s.wp_frames, s.flow_iters, s.flow_scales, s.flow_warps, s.bp_exact) == \
        (2, 2, 16, 20, 2, 1, 0)
    assert s.flow_tol == 0.0
