"""The ctypes structures of the Python binding (capi.py) have the layout of
the C ABI header (include/epscu.h): size and every field offset, checked by
compiling a probe against the header with the host C compiler (no GPU)."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import pytest

from epseon_backend_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PAIRS = [
    ("epscu_batch", capi.Batch),
    ("epscu_opts", capi.Opts),
    ("epscu_result", capi.Result),
    ("epscu_device_info", capi.DeviceInfo),
    ("epscu_stats", capi.Stats),
]


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")
def test_struct_layouts_match_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "epscu.h"', "int main(void) {"]
    for cname, cls in PAIRS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            cname, key, val = line.split()
            got[(cname, key)] = int(val)
    for cname, cls in PAIRS:
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
