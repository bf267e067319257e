"""The structs of include/fs2d.h and include/fs3d.h as a C compiler lays
them out, against the ctypes mirrors in fluid-sim_gb300/fs2d.py (no GPU):
same size, and every field at the same offset.  A mismatch here would
corrupt every call that passes the struct."""
import os
import shutil
import subprocess

import pytest

import fs2d

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
STRUCTS = {"fs2d_config": fs2d.Config, "fs2d_options": fs2d.Options, "fs2d_state": fs2d.State,
           "fs2d_stats": fs2d.Stats, "fs2d_render": fs2d.Render, "fs3d_array": fs2d.Array3D,
           "fs3d_mac": fs2d.MACGrid3D}


def c_layout(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fs2d.h"', '#include "fs3d.h"',
             "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    table = {}
    for line in out.splitlines():
        s, f, v = line.split()
        table[(s, f)] = int(v)
    return table


def test_struct_layouts_match_ctypes(tmp_path):
    table = c_layout(tmp_path)
    for cname, py in STRUCTS.items():
        assert table[(cname, "sizeof")] == fs2d.C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert table[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
