"""The ctypes mirrors of the C ABI's structs (warp-and-project-tomography_gb300/wap.py)
have the size and field offsets the C compiler gives the declarations in
include/wap/*.h: a field added on one side only fails here, on the host."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
INC = os.path.join(HERE, "..", "include")

STRUCTS = {"wap_scan_desc": "ScanDesc", "wap_schedule": "Schedule", "wap_stats": "Stats",
           "wap_job_desc": "JobDesc", "wap_job_info": "JobInfo"}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory, wapmod):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "wap/wap.h"', '#include "wap/wap_serve.h"',
             "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in getattr(wapmod, pyname)._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(d / "layout")
    subprocess.run(["gcc", "-std=c99", "-I", INC, "-o", exe, str(src)], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    return dict((l.rsplit(" ", 1)[0], int(l.rsplit(" ", 1)[1])) for l in out if l)


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_struct_matches_the_c_declaration(c_layout, wapmod, cname):
    import ctypes
    py = getattr(wapmod, STRUCTS[cname])
    assert ctypes.sizeof(py) == c_layout["%s size" % cname]
    for field, _ in py._fields_:
        assert getattr(py, field).offset == c_layout["%s.%s" % (cname, field)], field
