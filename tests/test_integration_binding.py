"""The reference-side binding shown in INTEGRATION.md compiles against the
reference's own headers (no GPU; skipped where the reference sources are
absent).  The block's member declarations are added to a temporary copy of
the reference's include/elliptic.h, as the maintainer would add them, and
the block is compiled with g++ -fsyntax-only beside include/olgpu.h."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("OLLIPTIC_REF_DIR", "/root/reference")


def binding_block():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    return next(b for b in blocks if "void elliptic::Vcycle_GPU()" in b)


def test_integration_binding_compiles_against_the_reference(tmp_path):
    inc = os.path.join(REF, "include")
    if not os.path.isdir(inc):
        pytest.skip("the reference sources are not present")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    block = binding_block()
    members = re.findall(r"^//\s+(interface \*gpu_oll = nullptr;|void Vcycle_GPU \(\);)", block, flags=re.M)
    assert len(members) == 2, members
    hdr = tmp_path / "include"
    shutil.copytree(inc, hdr)
    eh = (hdr / "elliptic.h").read_text()
    anchor = "void Vcycle ();"
    assert anchor in eh
    (hdr / "elliptic.h").write_text(eh.replace(anchor, anchor + "\n  " + "\n  ".join(members), 1))
    src = tmp_path / "binding.cc"
    src.write_text("#include <vector>\n#include \"elliptic.h\"\n" + block)
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-w", "-I", str(hdr), "-I",
                        os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
