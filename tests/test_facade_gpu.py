"""The drop-in layer on the GPU: the headless command line reproduces the
reference's complete PSART::Render (golden fixture made by the reference
itself) bit for bit and writes the reference's dump files, and the C++ facade
(reference names and signatures) matches the oracle call by call."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
import phantoms as P

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(REPO, "tests", "golden")
CLI = os.path.join(REPO, "warp-and-project-tomography_gb300", "lib", "wap_tomo")


@pytest.fixture(scope="module")
def built(wapmod, torch_cuda):
    import build
    build.build()
    return wapmod


def test_cli_render_matches_the_reference_bit_for_bit(built, tmp_path):
    wap = built
    d = np.load(os.path.join(GOLD, "render.npz"))
    N, _, W, H, NP = [int(v) for v in d["dims"]]
    projs = d["projs"].astype(np.float32)  # (NP, H, W): x fastest, the stack along z
    wap.analyze_save(str(tmp_path / "projs.hdr"), projs)
    (tmp_path / "angles.txt").write_text(" ".join("%.17g" % a for a in d["angles"]))
    args = [CLI, "-f", str(N), "-f", str(N), "-f", str(N), "-u", str(W), "-u", str(H), "-i", "projs.hdr",
            "-g", str(4 * N), "-j", str(6 * N), "-c", "1", "-d", "1", "-a", "0.1", "-s", "0.3", "-t", "0.3",
            "-v", "1", "--oxyz", "0", "--oxyz", "0", "--oxyz", "0", "--sdg", "0", "--nproj", str(NP),
            "--angles", "angles.txt", "-o", "out/test", "--save-final", "final"]
    r = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    v0 = wap.analyze_load(str(tmp_path / "final.level01.f000.vol.hdr"))[0]
    v1 = wap.analyze_load(str(tmp_path / "final.level01.f001.vol.hdr"))[0]
    f0 = wap.analyze_load(str(tmp_path / "final.level01.f000.flow.hdr"))
    assert np.array_equal(v0, d["level1_vol0"])
    assert np.array_equal(v1, d["level1_vol1"])
    assert np.array_equal(f0, d["level1_flow0"])
    # the reference's own dump names, with the states it writes there
    st10 = wap.analyze_load(str(tmp_path / "out" / "test.f001.out00.st10.flevel01.hdr"))[0]
    assert np.array_equal(st10, d["level1_vol1"])
    assert (tmp_path / "out" / "test.f000.out00.st01.flevel00.hdr").exists()
    for c in "uvw":
        assert (tmp_path / "VelocityField" / ("Flow%03d.s0.050.h1.000.f000.outloop000.%s.hdr" % (N, c))).exists()
    assert any(p.name.startswith("warpedI000") for p in (tmp_path / "warpedVolume").iterdir())
    assert any(p.name.endswith("flevel01.hdr") for p in (tmp_path / "WarpStep").iterdir())


@pytest.fixture(scope="module")
def checker(built, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("facade") / "facade_check")
    lib = os.path.join(REPO, "warp-and-project-tomography_gb300", "lib")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(REPO, "include"),
                        os.path.join(REPO, "tests", "facade", "facade_check.cpp"), "-o", out, "-L" + lib,
                        "-lwap_gb300", "-Wl,-rpath," + lib], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run(checker, *args):
    r = subprocess.run([checker] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def test_facade_advect(built, orc, checker, tmp_path):
    wap = built
    n = 24
    src = P.ellipsoids(n, seed=21)
    vel = P.rbf_flow(n, amp=2.0, seed=22)
    wap.analyze_save(str(tmp_path / "vel.hdr"), vel)
    wap.analyze_save(str(tmp_path / "src.hdr"), src)
    _run(checker, "advect", tmp_path / "vel.hdr", tmp_path / "src.hdr", 0.6, tmp_path / "out.hdr")
    got = wap.analyze_load(str(tmp_path / "out.hdr"))[0]
    ref = orc.advect([n] * 3, np.array([0, n, 0, n, 0, n], np.float32), vel, src, 0.6)
    assert np.array_equal(got, ref)


def test_facade_flow_multiscale_and_level(built, orc, checker, tmp_path):
    wap = built
    n = 32
    I1 = P.ellipsoids(n, seed=23)
    aabb = np.array([0, n, 0, n, 0, n], np.float32)
    fl = P.rbf_flow(n, amp=1.5, seed=24)
    I2 = orc.advect([n] * 3, aabb, fl, I1, 1.0)
    V0 = (fl * 0.2).astype(np.float32)
    for nm, a in (("I1", I1), ("I2", I2), ("V0", V0)):
        wap.analyze_save(str(tmp_path / (nm + ".hdr")), a)
    _run(checker, "flow", tmp_path / "I1.hdr", tmp_path / "I2.hdr", tmp_path / "V0.hdr", 40, 3, 6, tmp_path / "o.hdr")
    ov, _ = orc.flow_multiscale([n] * 3, I1, I2, V0, 0.0, 0.05, 40, 2, 0.5, 0.8, 3, [6] * 6)
    assert np.array_equal(wap.analyze_load(str(tmp_path / "o.hdr")), ov)
    _run(checker, "level", tmp_path / "I1.hdr", tmp_path / "I2.hdr", tmp_path / "V0.hdr", 60, 4, tmp_path / "l.hdr")
    oV = V0.copy()
    Y = [np.zeros((3, n, n, n), np.float32) for _ in range(3)] + [np.zeros((n, n, n), np.float32)]
    orc.flow_level([n] * 3, I1, I2, oV, *Y, 0.0, 0.05, 60, 2, aabb, [4] * 6, deterministic=1)
    assert np.array_equal(wap.analyze_load(str(tmp_path / "l.hdr")), oV)


def test_facade_cg(built, orc, checker, tmp_path):
    wap = built
    n = 20
    rhs = np.random.default_rng(25).normal(size=(n, n, n)).astype(np.float32)
    wap.analyze_save(str(tmp_path / "b.hdr"), rhs)
    _run(checker, "cg", tmp_path / "b.hdr", 1.0, 0.5, 60, tmp_path / "x.hdr")
    x = np.zeros_like(rhs)
    orc.cg_screened_laplacian([n] * 3, 1.0, 0.5, rhs, x, 1e-5, 60, 1e-9, mode=1)
    got = wap.analyze_load(str(tmp_path / "x.hdr"))[0]
    assert np.linalg.norm(got - x) / np.linalg.norm(x) < 1e-4


def test_facade_projector_entry_points(built, orc, checker, tmp_path):
    wap = built
    n, W, H, NPj = 32, 40, 36, 8
    vol = P.ellipsoids(n, seed=26)
    ang = P.golden_angles(NPj)
    wap.analyze_save(str(tmp_path / "vol.hdr"), vol)
    (tmp_path / "angles.txt").write_text("\n".join("%.17g" % a for a in ang))
    _run(checker, "project", tmp_path / "vol.hdr", W, H, NPj, 5, 4 * n, 6 * n, tmp_path / "angles.txt",
         tmp_path / "p.hdr")
    got = wap.analyze_load(str(tmp_path / "p.hdr"))[:, 0]
    scan = O.make_scan((n, n, n), (W, H), NPj)
    img, ln, wt = orc.forward(scan, ang[5], vol)
    assert np.array_equal(got[2], wt) and np.array_equal(got[1], ln) and np.array_equal(got[0], img)
