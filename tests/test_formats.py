"""Host file formats and scan tables of the command line, against the
reference's own CImg code (golden fixtures made by tests/golden/make_golden.py
from CImg's load_analyze / save_analyze / get_split) and the oracle's
restatement of the angle generator.  No GPU needed."""
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "formats.npz")
CASES = ["f32_le", "i16_be", "u8_le", "i32_le", "f64_nii", "f32_be_nii"]


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("name", CASES)
def test_analyze_load_matches_cimg(wapmod, gold, tmp_path, name):
    hdr = gold[name + "_hdr"].tobytes()
    raw = gold[name + "_raw"].tobytes()
    if name.endswith("nii"):
        path = tmp_path / (name + ".nii")
        path.write_bytes(hdr + raw)
    else:
        path = tmp_path / (name + ".hdr")
        path.write_bytes(hdr)
        (tmp_path / (name + ".img")).write_bytes(raw)
    (w, h, d, c), _ = wapmod.analyze_info(str(path))
    assert (w, h, d, c) == (5, 4, 3, 2)
    got = wapmod.analyze_load(str(path))
    assert np.array_equal(got.ravel(), gold[name + "_loaded"])
    if not name.endswith("nii"):  # the .img name finds its header too
        assert np.array_equal(wapmod.analyze_load(str(tmp_path / (name + ".img"))).ravel(), gold[name + "_loaded"])


def test_analyze_save_is_byte_identical_to_cimg(wapmod, gold, tmp_path):
    wapmod.analyze_save(str(tmp_path / "out.hdr"), gold["save_data"])
    assert (tmp_path / "out.hdr").read_bytes() == gold["save_hdr"].tobytes()
    assert (tmp_path / "out.img").read_bytes() == gold["save_img"].tobytes()


@pytest.mark.parametrize("name", ["vol.hdr", "vol.img", "vol", "vol.nii"])
def test_analyze_round_trip(wapmod, tmp_path, name):
    a = np.random.default_rng(3).normal(size=(3, 7, 6, 5)).astype(np.float32)
    p = str(tmp_path / name)
    wapmod.analyze_save(p, a)
    back = wapmod.analyze_load(p if name != "vol" else p + ".hdr")
    assert np.array_equal(back, a)


def test_analyze_missing_file_is_an_error(wapmod, tmp_path):
    with pytest.raises(wapmod.WapError):
        wapmod.analyze_load(str(tmp_path / "nope.hdr"))


def test_split_z_matches_cimg(wapmod, gold):
    t = gold["split_table"]
    i = 0
    while i < len(t):
        depth, nb = int(t[i]), int(t[i + 1])
        first, count = t[i + 2:i + 2 + nb], t[i + 2 + nb:i + 2 + 2 * nb]
        f, c = wapmod.split_z(depth, nb)
        assert np.array_equal(f, first) and np.array_equal(c, count), (depth, nb)
        i += 2 + 2 * nb
    with pytest.raises(wapmod.WapError):
        wapmod.split_z(4, 5)


def test_read_angles_like_the_reference_stream(wapmod, tmp_path):
    p = tmp_path / "angles.txt"
    p.write_text("0 137.5\n275.0\t52.5e0   x 10\n")
    a, n = wapmod.read_angles(str(p), 6)
    assert n == 4
    assert list(a) == [0.0, 137.5, 275.0, 52.5, 0.0, 0.0]
    with pytest.raises(wapmod.WapError):
        wapmod.read_angles(str(tmp_path / "missing.txt"), 3)


@pytest.mark.parametrize("np_,ns,p,nz", [(100, 1, 2, 50), (192, 1, 2, 1000), (64, 3, 3, 7), (37, 5, 2, 4)])
def test_lds_angles_match_restatement(wapmod, np_, ns, p, nz):
    got = wapmod.lds_angles(np_, ns, p, nz)
    ref = O.lds_angles(np_, ns, p, nz)
    assert np.array_equal(got, ref)
    if (ns, p) == (1, 2):
        # van der Corput in base 2: 0, 1/2, 1/4, 3/4, 1/8, ... of the circle
        assert list(got[:5]) == [0.0, 180.0, 90.0, 270.0, 45.0]
