"""The MeshLib-side binding (include/MRGbFastWindingNumber.h) compiles against MeshLib's own headers.

g++ -fsyntax-only in C++23 with std::expected (MeshLib's MR_USE_STD_EXPECTED build), MeshLib's
source tree on the include path and two stand-in headers for its un-vendored parallel-hashmap
submodule.  The check needs a MeshLib source tree (MESHLIB_SOURCE, else the usual checkout path)
and is skipped where there is none."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _meshlib_source():
    for p in (os.environ.get("MESHLIB_SOURCE"), "/root/reference/source"):
        if p and os.path.exists(os.path.join(p, "MRMesh", "MRFastWindingNumber.h")):
            return p
    return None


def test_binding_compiles_against_meshlib_headers():
    src = _meshlib_source()
    if src is None:
        pytest.skip("no MeshLib source tree here")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    cmd = [gxx, "-fsyntax-only", "-std=c++23", "-DMR_USE_STD_EXPECTED=1", "-Wall", "-Wextra", "-Werror=return-type",
           "-I", src, "-I", os.path.join(ROOT, "tests", "cpp", "stub"), "-I", os.path.join(ROOT, "oracle", "ref", "stub"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "meshlib_binding_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    errors = [ln for ln in r.stderr.splitlines() if "error" in ln]
    assert r.returncode == 0 and not errors, "\n".join(errors[:20]) or r.stderr[-2000:]
    # MeshLib's own headers warn under -Wall -Wextra; the binding itself must not
    ours = [ln for ln in r.stderr.splitlines() if "MRGbFastWindingNumber.h" in ln and "warning" in ln]
    assert not ours, "\n".join(ours)
