"""The certified float-float evaluation of the reference's double bicubic and
of the flow pyramid's double cubic growth (csrc/bp_cubic.h), checked on the
host: whenever it claims a float result,
that result equals the reference's double expression rounded to float, bit
for bit, over tens of millions of correction-image-like, cancelling, tied and
random-bit-pattern inputs.  The exact backprojection kernel takes the double
path wherever the certificate declines; the GPU parity tests compare that
kernel with the oracle."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "warp-and-project-tomography_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("proof") / "bp_cubic_check")
    src = os.path.join(HERE, "proofs", "bp_cubic_check.cpp")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC, "-o", exe, src], check=True)
    return exe


@pytest.mark.parametrize("seed", ["1", "2", "3"])
def test_certified_bicubic_matches_double(checker, seed):
    r = subprocess.run([checker, "10000000", seed], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = dict(kv.split("=") for kv in r.stdout.split()[-7:])
    assert out["cubic-mismatch"] == "0" and out["update-mismatch"] == "0", r.stdout
    assert out["grow-mismatch"] == "0", r.stdout
    # the certificates must also be useful: they decide nearly all cases
    assert int(out["cubic-claimed"]) > 0.95 * int(out["cases"]), r.stdout
    assert int(out["grow-claimed"]) > 0.95 * int(out["cases"]), r.stdout
