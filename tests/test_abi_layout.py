"""The ctypes mirror of the C-ABI structs (temporalspecklescode_gb300/config.py)
has the layout of include/sstmc.h: every field's offset and each struct's
size agree with what a C compiler makes of the header.  CPU only (gcc)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from temporalspecklescode_gb300 import config as cf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes field name -> C field name where they differ
RENAMED = {"lam": "lambda"}

STRUCTS = [("sstmc_config", cf.SstmcConfig), ("sstmc_source_cfg", cf.SourceCfg), ("sstmc_path_trace", cf.PathTrace)]


def _c_layout(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sstmc.h"', "int main(void) {"]
    for cname, cls in STRUCTS:
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            n = RENAMED.get(f[0], f[0])
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {n}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    return got


def test_ctypes_structs_match_the_header(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    got = _c_layout(tmp_path)
    for cname, cls in STRUCTS:
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])
