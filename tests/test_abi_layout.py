"""The ctypes mirrors of the C ABI structs match include/elfel_gpu.h (CPU).

A small C program compiled with gcc prints sizeof/offsetof of every struct
the header declares; the ctypes Structure of the Python binding must agree
field by field (a mismatch would silently corrupt every call that passes one).
"""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "elfel_space": "Space",
    "elfel_fused_desc": "FusedDesc",
    "elfel_solve_stats": "SolveStats",
    "elfel_block_desc": "BlockDesc",
    "elfel_server_config": "ServerConfig",
    "elfel_heat_request": "HeatRequest",
    "elfel_serve_result": "ServeResult",
    "elfel_server_stats": "ServerStats",
}


def c_layout(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    import importlib.util

    spec = importlib.util.spec_from_file_location("nat", os.path.join(ROOT, "elfel.jl_gb300", "_native.py"))
    nat = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(nat)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "elfel_gpu.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        st = getattr(nat, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
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
    return nat, got


def test_struct_layouts_match_header(tmp_path):
    nat, got = c_layout(tmp_path)
    for cname, pyname in STRUCTS.items():
        st = getattr(nat, pyname)
        assert ctypes.sizeof(st) == got[(cname, "size")], cname
        for f, _ in st._fields_:
            assert getattr(st, f).offset == got[(cname, f)], (cname, f)
