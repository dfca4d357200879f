"""The C ABI: the library builds, loads, exports every declared entry point,
and the ctypes structure images match the C layouts."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from meraxes_gb300 import _lib
from meraxes_gb300.params import MxGlobals, MxGrids, MxParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mx_reion.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mx_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(names) == sorted(_lib.EXPORTS)


def test_struct_layouts_match_header():
    fields = {"mx_params": MxParams, "mx_grids": MxGrids, "mx_globals": MxGlobals}
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "mx_reion.h"', "int main(void) {"]
    for cname, cls in fields.items():
        src.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            src.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    src.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "l")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for cname, cls in fields.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_invalid_parameters_are_rejected_without_a_device():
    lib = _lib.load()
    from meraxes_gb300.params import ReionParams

    p = ReionParams(grid_dim=15).to_ctypes()  # odd grids are not supported
    ctx = ctypes.c_void_p()
    rc = lib.mx_create(ctypes.byref(p), b".", ctypes.byref(ctx))
    assert rc == -1 and not ctx
    assert b"invalid" in lib.mx_last_error(None)
    p = ReionParams().to_ctypes()
    p.abi_version = 99
    assert lib.mx_create(ctypes.byref(p), b".", ctypes.byref(ctx)) == -1


def test_calls_on_null_context_fail_cleanly():
    lib = _lib.load()
    g = MxGrids()
    out = MxGlobals()
    assert lib.mx_find_HII_bubbles(None, 0, ctypes.byref(g), ctypes.byref(out)) == -1
    assert lib.mx_step_device(None, 0, ctypes.byref(g), ctypes.byref(out), None) == -1
    assert lib.mx_n_sfr_histories(None) == -1
