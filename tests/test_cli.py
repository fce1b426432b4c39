"""The headless command line and the C++ facade, without a GPU: the binary's
option handling (the reference's argtable options), its error statuses, and
that the facade compiles against the reference-style template signatures
(also with the reference's own CImg<float>, when that tree is present)."""
import os
import shutil
import subprocess

import pytest

import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(REPO, "warp-and-project-tomography_gb300", "lib", "wap_tomo")
CHECK_SRC = os.path.join(REPO, "tests", "facade", "facade_check.cpp")


@pytest.fixture(scope="module")
def cli(wapmod):
    import build
    build.build()
    assert os.path.exists(CLI)
    return CLI


def run(args, **kw):
    return subprocess.run(args, capture_output=True, text=True, timeout=60, **kw)


def test_help_lists_the_reference_options(cli):
    r = run([cli, "--help"])
    assert r.returncode == 0
    for opt in ["-s, --Sigma", "-t, --Tau", "-a, --Alpha", "-o", "-v, --nframes", "-f, --XYZ", "-u, --imgUV",
                "-c, --voxelspacing", "-i, --projsvolume", "-j, --sdd", "-g, --sid", "--oxyz", "--sdg",
                "-b, --AlgorithmIter", "-p, --SartIter", "--prior", "--bp"]:
        assert opt in r.stdout, opt


@pytest.mark.parametrize("args,msg", [(["--nope"], "unknown option --nope"), (["-f"], "needs a value"),
                                      (["-f", "x"], "invalid value"), (["-f", "1", "-f", "2", "-f", "3", "-f", "4"],
                                                                      "too many occurrences"),
                                      (["-f", "16"], "missing option -i")])
def test_bad_command_lines_fail_like_argtable(cli, args, msg):
    r = run([cli] + args)
    assert r.returncode == 1
    assert msg in r.stdout


def test_no_arguments_prints_the_hint(cli):
    r = run([cli])
    assert r.returncode == 0 and "Try" in r.stdout


def test_missing_projection_file_is_an_error(cli, tmp_path):
    r = run([cli, "-f", "16", "-u", "16", "-i", str(tmp_path / "none.hdr"), "--nproj", "4"], cwd=str(tmp_path))
    assert r.returncode == 2
    assert "projection stack" in r.stderr


def test_facade_compiles_with_the_reference_signatures(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    inc = os.path.join(REPO, "include")
    r = run([gxx, "-std=c++17", "-fsyntax-only", "-I" + inc, CHECK_SRC])
    assert r.returncode == 0, r.stderr
    tree = oracle.reference_tree()
    ref = os.path.join(tree, "Project") if tree else ""
    if tree and os.path.exists(os.path.join(ref, "CImg.h")):
        r = run([gxx, "-std=c++17", "-fsyntax-only", "-w", "-I" + inc, "-I" + ref, "-DWAP_WITH_CIMG", CHECK_SRC])
        assert r.returncode == 0, r.stderr
