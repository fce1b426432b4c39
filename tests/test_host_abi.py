"""Host-side checks of the C ABI that need no GPU: the shared library loads and
exports every function include/wap/wap.h declares, the host geometry and
frame windows match the oracle, and calls fail with a status, not a crash,
when no GPU is present or arguments are invalid."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
import phantoms as P

INC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "wap")


def declared():
    txt = "".join(open(os.path.join(INC, f)).read() for f in sorted(os.listdir(INC)) if f.endswith(".h"))
    return sorted(set(re.findall(r"WAP_API\s+[^;(]*?\b(wap_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(wapmod):
    names = declared()
    assert len(names) >= 30
    L = wapmod.load()
    for n in names:
        assert hasattr(L, n), n
    # and the Python binding covers them all
    assert set(names) - set(wapmod.SIGNATURES) <= {"wap_cg_screened_laplacian_noalloc"}


@pytest.mark.parametrize("angle", [0.0, 37.5, 222.4922359499621, 359.9])
def test_host_geometry_matches_oracle(wapmod, orc, angle):
    ws = wapmod.make_scan((48, 40, 32), (64, 50), 10, vs=0.75, ds=1.25, sid=150.0, sdd=260.0, oxyz=(1.5, -2.0, 0.5))
    os_ = O.make_scan((48, 40, 32), (64, 50), 10, vs=0.75, ds=1.25, sid=150.0, sdd=260.0, oxyz=(1.5, -2.0, 0.5))
    p2m, m2v, mvv2m, eye = wapmod.projection_geometry(ws, angle)
    op2m, om2v, omv, ov2m, oeye = orc.geometry(os_, angle)
    assert np.array_equal(p2m, op2m)
    assert np.array_equal(m2v, om2v)
    assert np.array_equal(eye, oeye)
    # the BP's combined matrix MV * V2M, summed in the reference's order
    mv = omv.reshape(4, 4).T.astype(np.float32)
    v2m = ov2m.reshape(4, 4).T.astype(np.float32)
    ref = np.zeros((4, 4), np.float32)
    for r in range(4):
        for c in range(4):
            acc = np.float32(0)
            for k in range(4):
                acc = np.float32(acc + np.float32(mv[r, k] * v2m[k, c]))
            ref[r, c] = acc
    assert np.array_equal(mvv2m.reshape(4, 4).T, ref)


@pytest.mark.parametrize("nframes,nproj,level", [(1, 192, 0), (1, 192, 1), (48, 192, 0), (5, 64, 1), (100, 130, 1)])
def test_frame_windows(wapmod, orc, nframes, nproj, level):
    ws = wapmod.make_scan((16, 16, 16), (16, 16), nproj, nframes_cli=nframes)
    got = wapmod.level_frames(ws, level)
    ref = orc.level_frames(nframes, nproj, level)
    assert got[0] == ref[0]
    for a, b in zip(got[1:4], ref[1:4]):
        assert np.array_equal(a, b)
    assert got[4] == ref[4]


def test_create_without_gpu_or_with_bad_scan_fails_cleanly(wapmod):
    import torch
    L = wapmod.load()
    h = ctypes.c_void_p()
    bad = wapmod.make_scan((2, 16, 16), (16, 16), 4)
    assert L.wap_create(ctypes.byref(h), ctypes.byref(bad), np.zeros(4).ctypes.data, 0) == wapmod.WAP_EINVAL
    good = wapmod.make_scan((16, 16, 16), (16, 16), 4)
    r = L.wap_create(ctypes.byref(h), ctypes.byref(good), np.zeros(4).ctypes.data, 0)
    if not torch.cuda.is_available():
        assert r == wapmod.WAP_ENODEV
    else:
        assert r == wapmod.WAP_OK
        L.wap_destroy(h)
    assert L.wap_create(None, ctypes.byref(good), None, 0) == wapmod.WAP_EINVAL


def test_reference_tree_live_pin(orc):
    """Where the reference tree exists, re-pin a forward projection live."""
    if not O.reference_tree() or not os.path.exists(O.REF_SO):
        pytest.skip("reference tree not present")
    import tempfile
    ref = O.Reference()
    N, W, H, NP = 20, 24, 24, 4
    vol = P.ellipsoids(N, count=5, seed=40)
    ang = P.golden_angles(NP)
    scan = O.make_scan((N, N, N), (W, H), NP)
    projs = np.stack([orc.forward(scan, a, vol)[0] for a in ang]).astype(np.float32)
    ref.create(scan, projs, ang, tempfile.mkdtemp())
    ref.lib.wref_set_volume(0, 0, vol)
    i, l, w = (np.zeros((H, W), np.float32) for _ in range(3))
    ref.lib.wref_forward(0, 0, 2, 0, 0.0, i, l, w)
    oi, ol, ow = orc.forward(scan, ang[2], vol)
    ref.lib.wref_destroy()
    assert np.array_equal(ow, w) and np.array_equal(oi, i) and np.array_equal(ol, l)


def test_job_footprint_grows_with_the_job(wapmod):
    sched = wapmod.reference_schedule(n_cp=2, flow_scales=4)
    small = wapmod.job_device_bytes(wapmod.make_scan((64,) * 3, (96, 96), 64, nframes_cli=8), sched)
    big = wapmod.job_device_bytes(wapmod.make_scan((128,) * 3, (192, 192), 64, nframes_cli=8), sched)
    more = wapmod.job_device_bytes(wapmod.make_scan((128,) * 3, (192, 192), 128, nframes_cli=16), sched)
    assert 0 < small < big < more
    # 256^3 x 192 projections, 48 frames: dominated by 13 floats per voxel per frame
    full = wapmod.job_device_bytes(wapmod.make_scan((256,) * 3, (384, 384), 192, nframes_cli=48), sched)
    assert 48 * 13 * 4 * 256 ** 3 < full < 1.3 * 48 * 13 * 4 * 256 ** 3


def test_server_without_a_gpu_is_an_error(wapmod, torch_available=None):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(wapmod.WapError):
        wapmod.Server(1 << 30, workers=1)


def test_block_cache_is_empty_without_contexts(wapmod):
    L = wapmod.load()
    assert L.wap_trim_cache(-1) == 0
    assert L.wap_cached_bytes() == 0
