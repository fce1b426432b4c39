"""CoherentVolume (CoherentVolume.h:16-85, CoherentVolume.cpp:33-258): the
block-partitioned volume with constant-block compression, header-only in the
facade (include/wap/coherent_volume.hpp).  Checked against the reference's own
class where its pointer steps are defined (one block per axis) and against a
model of the block partition for many blocks, with constant blocks, ragged
edge blocks and NaN-free random data.  No GPU needed."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
INC = os.path.join(os.path.dirname(HERE), "include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("cv") / "cv_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + INC, os.path.join(HERE, "facade", "coherent_volume_check.cpp"),
                    "-o", exe], check=True)
    return exe


def run(checker, tmp_path, bs, vol):
    d, h, w = vol.shape
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(src, "wb") as f:
        f.write(np.array(list(bs) + [w, h, d], np.int32).tobytes())
        f.write(np.ascontiguousarray(vol, np.float32).tobytes())
    r = subprocess.run([checker, src, dst], capture_output=True, timeout=60)
    assert r.returncode == 0, r
    raw = open(dst, "rb").read()
    n = vol.size
    vals = np.frombuffer(raw[:4 * n], np.float32).reshape(vol.shape)
    mm = np.frombuffer(raw[4 * n:4 * n + 16], np.float64)
    stored = int(np.frombuffer(raw[4 * n + 16:], np.int32)[0])
    return vals, mm, stored


def volume(shape, bs, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=shape).astype(np.float32)
    # make some blocks constant
    d, h, w = shape
    for bz in range(0, d, bs[2]):
        for by in range(0, h, bs[1]):
            for bx in range(0, w, bs[0]):
                if rng.random() < 0.4:
                    v[bz:bz + bs[2], by:by + bs[1], bx:bx + bs[0]] = rng.choice([0.0, 1.5])
    return v


@pytest.mark.parametrize("shape,bs", [((20, 24, 28), (4, 4, 4)), ((17, 9, 30), (8, 4, 5)), ((7, 7, 7), (3, 2, 5))])
def test_block_partition(checker, tmp_path, shape, bs):
    v = volume(shape, bs, sum(shape))
    vals, mm, stored = run(checker, tmp_path, bs, v)
    assert np.array_equal(vals, v)
    assert mm[0] == v.min() and mm[1] == v.max()
    d, h, w = shape
    nonconst = 0
    for bz in range(0, d, bs[2]):
        for by in range(0, h, bs[1]):
            for bx in range(0, w, bs[0]):
                blk = v[bz:bz + bs[2], by:by + bs[1], bx:bx + bs[0]]
                nonconst += int(blk.min() != blk.max())
    assert stored == nonconst


def test_matches_the_reference_class_on_one_block(checker, tmp_path):
    if not os.path.exists(O.REF_SO) or not O.reference_tree():
        pytest.skip("the reference build is not present")
    ref = O.Reference()
    f = ref.lib.wref_coherent_volume
    f.restype = ctypes.c_int
    for shape, bs, seed in [((12, 10, 16), (16, 16, 16), 1), ((5, 6, 7), (7, 6, 5), 2), ((8, 8, 8), (8, 8, 8), 3)]:
        v = volume(shape, shape[::-1], seed)
        if seed == 3:
            v[:] = 2.25  # a constant volume: the block keeps no data
        d, h, w = shape
        want = np.zeros_like(v)
        mm = np.zeros(2, np.float64)
        rc = f(np.array(bs, np.int32).ctypes.data, np.array([w, h, d], np.int32).ctypes.data,
               np.ascontiguousarray(v).ctypes.data, want.ctypes.data, mm.ctypes.data)
        assert rc == 0
        got, gmm, stored = run(checker, tmp_path, bs, v)
        assert np.array_equal(got, want)
        assert np.array_equal(gmm, mm)
        assert stored == int(v.min() != v.max())
