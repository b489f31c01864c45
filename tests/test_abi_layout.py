"""The ctypes mirrors of the C structs (openbte_gb300/_lib.py) have the header's sizes and field offsets.

A small C program compiled with the host compiler prints sizeof / offsetof of every field of every struct
in include/obte.h; the ctypes layouts must match them exactly (a mismatch would pass garbage through the
C ABI)."""
import os
import shutil
import subprocess

import pytest

from openbte_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"obte_problem": _lib.Problem, "obte_material": _lib.MaterialC, "obte_solve_opts": _lib.SolveOpts,
           "obte_solve_info": _lib.SolveInfo, "obte_fourier_problem": _lib.FourierProblem,
           "obte_fourier_opts": _lib.FourierOpts, "obte_fourier_info": _lib.FourierInfo}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs the host C compiler")
def test_struct_layouts_match_the_header(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', f'#include "{ROOT}/include/obte.h"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            s, f, v = ln.split()
            got[(s, f)] = int(v)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "size")] == C_sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)
