"""The ctypes mirrors of the C-ABI structs (tensormesh_gb300/_lib.py) have
the layout of the structs in include/tensormesh_gb300.h: every field at the
same offset and the same total size, checked by compiling a small C program
against the header with the host compiler (no GPU, no CUDA)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from tensormesh_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {
    "tm_patch_plan": _lib.PatchPlan,
    "tm_assemble_args": _lib.AssembleArgs,
    "tm_backward_args": _lib.BackwardArgs,
    "tm_batched_args": _lib.BatchedArgs,
    "tm_twolevel": _lib.TwoLevel,
}


def test_ctypes_structs_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "tensormesh_gb300.h"', "int main(void) {"]
    expected = []
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        expected.append(f"{cname} sizeof {ctypes.sizeof(cls)}")
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
            expected.append(f"{cname} {fname} {getattr(cls, fname).offset}")
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    assert [g for g in got if g] == expected
