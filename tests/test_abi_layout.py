"""The ctypes mirrors of the public structs have the C layout of
include/pyvr_gb300.h (sizes and every field offset), checked against a
program compiled from the header with gcc."""

import ctypes
import shutil
import subprocess

import pytest

from pyvr_gb300 import _native

STRUCTS = {"pvr_job": _native.PvrJob, "pvr_tuning": _native.PvrTuning, "pvr_diff_view": _native.PvrDiffView,
           "pvr_diff_scene": _native.PvrDiffScene, "pvr_request": _native.PvrRequest,
           "pvr_completion": _native.PvrCompletion, "pvr_server_config": _native.PvrServerConfig,
           "pvr_server_stats": _native.PvrServerStats}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_struct_layouts_match_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pyvr_gb300.h"', "int main(void) {"]
    for c, py in STRUCTS.items():
        lines.append(f'printf("{c} size %zu\\n", sizeof({c}));')
        for name, _ in py._fields_:
            lines.append(f'printf("{c} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", _native.INCLUDE, str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for c, py in STRUCTS.items():
        assert got[(c, "size")] == ctypes.sizeof(py), c
        for name, _ in py._fields_:
            assert got[(c, name)] == getattr(py, name).offset, (c, name)
