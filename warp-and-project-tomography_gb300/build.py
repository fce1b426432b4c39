"""Build the GB300 warp-and-project library in-tree.

Compiles every CUDA/C++ source under csrc/ for sm_103a with nvcc (one
-gencode, translation units in parallel) and links lib/libwap_gb300.so with a
static CUDA runtime.  All translation units use -fmad=false: the reference's
arithmetic has no fused multiply-add, and the parity contract depends on each
float operation rounding where the reference's does; host code gets
-ffp-contract=off for the same reason (GCC contracts to FMA by default on
aarch64, which would change the projection matrices).

Usage: python build.py [--force] [-j N]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libwap_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "wap_tomo.cpp")
CLI = os.path.join(HERE, "lib", "wap_tomo")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
          "-I" + os.path.join(REPO, "include"), "-I" + CSRC]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    inc = os.path.join(REPO, "include", "wap")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + extra + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build(force=False, jobs=None, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sources()
    hdrs = headers()
    todo = [s for s in srcs if force or _stale(os.path.join(BUILD, os.path.basename(s) + ".o"), [s] + hdrs)]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda s: _compile(s, list(extra)), todo))
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    build_cli(force)
    return LIB


def build_cli(force=False):
    """The headless command line (cli/wap_tomo.cpp) over the C++ facade,
    linked against lib/libwap_gb300.so (found next to the binary)."""
    deps = [CLI_SRC, LIB] + headers()
    if not (force or _stale(CLI, deps)):
        return CLI
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(REPO, "include"), CLI_SRC, "-o", CLI,
           "-L" + os.path.dirname(LIB), "-lwap_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return CLI


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.j))
    sys.exit(0)
