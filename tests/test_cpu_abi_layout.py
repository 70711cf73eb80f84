"""The ctypes mirrors of the C ABI's structs have the header's layout.

`lofloat_gb300/_native.py` passes `lofgb_format`, `lofgb_round_task`,
`lofgb_gemm_task`, `lofgb_codec_format` and `lofgb_conv2d_shape` to the
library by pointer (tasks as arrays). A field out of place there would hand
the kernels wrong sizes or pointers, so this test compiles a small C program
against `include/lofgb.h` with the host C compiler, prints sizeof and every
field's offsetof, and compares them with the ctypes structures.
"""
import os
import shutil
import subprocess

import pytest

from lofloat_gb300 import _native as N

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

# C struct name -> (ctypes class, {ctypes field name: C field name})
STRUCTS = {
    "lofgb_format": (N.LofgbFormat, {}),
    "lofgb_round_task": (N.LofgbRoundTask, {"in_": "in"}),
    "lofgb_gemm_task": (N.LofgbGemmTask, {}),
    "lofgb_codec_format": (N.LofgbCodecFormat, {}),
    "lofgb_conv2d_shape": (N.LofgbConv2dShape, {}),
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lofgb.h"', "int main(void) {"]
    for cname, (cls, rename) in STRUCTS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            cf = rename.get(fname, fname)
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {cf}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        s, f, v = line.split()
        layout[(s, f)] = int(v)
    return layout


def test_ctypes_structs_match_header_layout(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, (cls, _) in STRUCTS.items():
        import ctypes as C
        assert C.sizeof(cls) == layout[(cname, "sizeof")], cname
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == layout[(cname, fname)], (cname, fname)


def test_header_gives_cpp_callers_c_linkage(tmp_path):
    """A C++ translation unit that includes `lofgb.h` and takes the address of
    every declared entry point refers to them by their plain C names (the
    header's extern "C" block), so a C++ binding links against liblofgb."""
    import re
    cxx = shutil.which("g++") or shutil.which("c++")
    nm = shutil.which("nm")
    if cxx is None or nm is None:
        pytest.skip("no host C++ compiler or nm")
    header = open(os.path.join(ROOT, "include", "lofgb.h")).read()
    names = sorted(set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(lofgb_\w+)\s*\(", header, re.M)))
    assert len(names) >= 30
    body = "\n".join(f"  (void*)&{n}," for n in names)
    src = tmp_path / "probe.cpp"
    src.write_text('#include "lofgb.h"\nvoid* table[] = {\n' + body + "\n};\n")
    obj = tmp_path / "probe.o"
    subprocess.run([cxx, "-c", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(obj)],
                   check=True, capture_output=True)
    undefined = subprocess.run([nm, "-u", str(obj)], check=True, capture_output=True,
                               text=True).stdout.split()
    for n in names:
        assert n in undefined, n
