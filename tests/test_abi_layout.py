"""The Python mirror of the C ABI matches include/fdadi.h: every declared
function has as many ctypes arguments as parameters, and every struct the
bindings build has the C compiler's size and field offsets (a small C program
compiled against the header prints them). Runs without a GPU."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from fd_adi_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdadi.h")

STRUCTS = [(_lib.Tri, "fdadi_tri_t"), (_lib.Mixed, "fdadi_mixed_t"),
           (_lib.MlpNet, "fdadi_mlp_net_t"), (_lib.HestonPlan, "fdadi_heston_plan_t"),
           (_lib.HestonBatch, "fdadi_heston_batch_t"), (_lib.Gemm, "fdadi_gemm_t"),
           (_lib.BsBatch, "fdadi_bs_batch_t")]


def _declarations():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return re.findall(r"^\s*(?:int|int64_t|void)\s+(fdadi_\w+)\s*\(([^;]*?)\)\s*;", src,
                      re.M | re.S)


def test_ctypes_signatures_match_the_header():
    decls = _declarations()
    assert len(decls) >= 30
    for name, params in decls:
        params = params.strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert name in _lib.SIGNATURES, name
        assert len(_lib.SIGNATURES[name][1]) == n, (name, n, len(_lib.SIGNATURES[name][1]))
    assert set(_lib.SIGNATURES) == {d[0] for d in decls}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_struct_layouts_match_the_compiler(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fdadi.h"', 'int main(void) {']
    for cls, ctype in STRUCTS:
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (ctype, ctype))
        for field, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (ctype, field, ctype, field))
    lines += ['return 0;', '}']
    c = tmp_path / "layout.c"
    c.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(c), "-o", str(exe)],
                   check=True, capture_output=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.splitlines():
        t, key, val = line.split()
        got[(t, key)] = int(val)
    for cls, ctype in STRUCTS:
        assert got[(ctype, "size")] == ctypes.sizeof(cls), ctype
        for field, _ in cls._fields_:
            assert got[(ctype, field)] == getattr(cls, field).offset, (ctype, field)
