"""The C adapter shown in INTEGRATION.md compiles against the reference's own
headers (src/meraxes.h through the oracle shims) and this library's header,
and links with libmxreion.so into a program (tests/adapter_drive.c) that sets
up run_globals and calls the three drop-in entry points.  Skipped where the
reference tree is not present."""
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


def test_adapter_links_and_reports_errors_through_abort():
    """The adapter and tests/adapter_drive.c link against libmxreion.so; with
    no CUDA device visible, the first entry point fails in mx_create and the
    adapter turns the error into the reference's ABORT (myexit), as the
    reference does on its own errors."""
    from oracle.runner import REF_SRC, ref_available

    if not ref_available():
        pytest.skip("reference tree not present")
    lib_dir = os.path.join(ROOT, "meraxes_gb300", "_lib")
    if not os.path.exists(os.path.join(lib_dir, "libmxreion.so")):
        pytest.skip("libmxreion.so not built")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, flags=re.S)
    adapter = [b for b in blocks if "void find_HII_bubbles(int snapshot" in b]
    assert len(adapter) == 1
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "mx_adapter.c")
        exe = os.path.join(d, "adapter_drive")
        open(src, "w").write(adapter[0])
        inc = ["-I", os.path.join(ROOT, "oracle", "shims"), "-I", os.path.join(ROOT, "oracle"), "-I", REF_SRC,
               "-I", os.path.join(REF_SRC, "core"), "-I", os.path.join(ROOT, "include")]
        cmd = ["gcc", "-std=gnu11", "-Werror=implicit-function-declaration", "-o", exe, src,
               os.path.join(ROOT, "tests", "adapter_drive.c")] + inc + \
            ["-L", lib_dir, "-lmxreion", "-Wl,-rpath," + lib_dir, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        from meraxes_gb300 import synthetic

        env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
        r = subprocess.run([exe, synthetic.TABLES_DIR], capture_output=True, text=True, env=env, timeout=120)
        assert r.returncode == 3, (r.returncode, r.stdout[-500:], r.stderr[-500:])
        assert "ABORT(1)" in r.stderr
