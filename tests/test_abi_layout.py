"""CPU check that the ctypes mirrors of the C ABI's structs match the header:
a small C program compiled against include/gemini_gb300.h prints each
struct's size and field offsets, which must equal the ctypes layout."""
import ctypes
import os
import shutil
import subprocess

import pytest

import geminigraph_gb300 as gg

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "gg_graph_info": gg._Info,
    "gg_build_options": gg._BuildOptions,
    "gg_run_stats": gg._Stats,
    "gg_query_result": gg._QueryResult,
    "gg_server_stats": gg._ServerStats,
    "gg_tune_result": gg._TuneResult,
}


def c_layout(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gemini_gb300.h"', "int main(void) {"]
    for cname, cls in MIRRORS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for ln in out.splitlines():
        cname, field, val = ln.split()
        got[(cname, field)] = int(val)
    return got


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structs_match_header(tmp_path):
    got = c_layout(tmp_path)
    for cname, cls in MIRRORS.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, f"{cname}.{fname}"
