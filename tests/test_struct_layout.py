"""The ctypes mirrors in cudagfx_gb300 match the C structs of include/gfx.h and
include/gfx_io.h field by field: a C program compiled here (gcc, no GPU) prints
sizeof and offsetof of every field, and each mirror must agree."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C type -> the ctypes class that mirrors it
STRUCTS = {
    "gfx_functional_t": "Functional",
    "gfx_or_params": "ORParams",
    "gfx_or_result": "ORResult",
    "gfx_check_record": "CheckRecord",
    "gfx_sa_params": "SAParams",
    "gfx_therm_params": "ThermParams",
    "gfx_tuning": "Tuning",
    "gfx_copy_result": "CopyResult",
    "gfx_ildg_info": "IldgInfo",
    "gfx_slice_cksum": "SliceCksum",
    "gfx_bqcd_info": "BqcdInfo",
    "gfx_cksum_state": "CksumState",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    import cudagfx_gb300 as gfx
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gfx.h"', '#include "gfx_io.h"',
             "int main(void) {"]
    for ctype, pyname in STRUCTS.items():
        cls = getattr(gfx, pyname)
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (ctype, ctype))
        for fname, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (ctype, fname, ctype, fname))
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for ln in out.splitlines():
        ctype, field, value = ln.split()
        layout[(ctype, field)] = int(value)
    return layout


@pytest.mark.parametrize("ctype", list(STRUCTS))
def test_ctypes_mirror_matches_c_struct(c_layout, ctype):
    import ctypes

    import cudagfx_gb300 as gfx
    cls = getattr(gfx, STRUCTS[ctype])
    assert ctypes.sizeof(cls) == c_layout[(ctype, "size")], ctype
    for fname, _ in cls._fields_:
        assert getattr(cls, fname).offset == c_layout[(ctype, fname)], (ctype, fname)
