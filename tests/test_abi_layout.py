"""The ctypes mirror (rsieve/__init__.py) matches the C header's structures:
a small C program built against include/rsieve.h prints every structure's size
and each field's offset, and the ctypes classes must agree field by field (a
field added to the header without the mirror, or in another place, would
otherwise shift every later field silently)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {
    "rs_factor": None,
    "rs_options": "Options",
    "rs_job_info": "JobInfo",
    "rs_stats": "Stats",
    "rs_server_options": "ServerOptions",
    "rs_job_report": "JobReport",
}


def _mirror(rs, cname):
    if cname == "rs_factor":  # a numpy structured dtype in the mirror
        return None
    return getattr(rs, STRUCTS[cname])


def test_struct_layouts_match_header(rs, tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "rsieve.h"', "int main(void) {"]
    for cname in STRUCTS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        cls = _mirror(rs, cname)
        names = [f for f, _ in cls._fields_] if cls else list(rs.FACTOR_DTYPE.names)
        for f in names:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname in STRUCTS:
        cls = _mirror(rs, cname)
        if cls is None:
            dt = rs.FACTOR_DTYPE
            assert got[(cname, "size")] == dt.itemsize
            for f in dt.names:
                assert got[(cname, f)] == dt.fields[f][1], (cname, f)
            continue
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
