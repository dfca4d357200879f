"""The C adapter shown in INTEGRATION.md compiles against the reference's own
headers (src/meraxes.h through the oracle shims) and this library's header.
Skipped where the reference tree is not present."""
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapter_compiles_against_reference_headers():
    from oracle.runner import REF_SRC, ref_available

    if not ref_available():
        pytest.skip("reference tree not present")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, flags=re.S)
    adapter = [b for b in blocks if "void find_HII_bubbles(int snapshot" in b]
    assert len(adapter) == 1
    # the optional functions of section 2b go into the same file
    extra = [b for b in blocks if "void construct_baryon_grids(int snapshot" in b]
    assert len(extra) == 1
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "mx_adapter.c")
        open(src, "w").write(adapter[0] + "\n" + extra[0])
        cmd = ["gcc", "-std=gnu11", "-fsyntax-only", "-Werror=implicit-function-declaration",
               "-Werror=incompatible-pointer-types", "-I", os.path.join(ROOT, "oracle", "shims"),
               "-I", os.path.join(ROOT, "oracle"), "-I", REF_SRC, "-I", os.path.join(REF_SRC, "core"),
               "-I", os.path.join(ROOT, "include"), src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
