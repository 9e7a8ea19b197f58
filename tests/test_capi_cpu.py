"""CPU-only checks of the C ABI: the library builds and loads, exports exactly what include/gbfwn.h
declares, and rejects bad arguments without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"GBFWN_API\s+[\w\s\*]+?\b(gbfwn_\w+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(fwn_lib):
    import meshlib_gb300
    decl = _declared()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(fwn_lib, name), name
    assert sorted(meshlib_gb300.EXPORTED) == decl


def test_bad_arguments_rejected_without_gpu(fwn_lib):
    import meshlib_gb300 as M
    L = M.lib()
    out = ctypes.c_void_p()
    assert L.gbfwn_create(None, 3, None, 1, 0, ctypes.byref(out)) == M.INVALID
    assert b"bad arguments" in L.gbfwn_last_error()
    dims = np.array([4, 4, 4], np.int32)
    xf = np.zeros(12, np.float32)
    assert L.gbfwn_from_grid(None, dims.ctypes.data, xf.ctypes.data, 2.0, None, M.PROGRESS(), None) == M.INVALID
    assert L.gbfwn_destroy(None) == M.OK
    assert L.gbfwn_num_faces(None) == 0
    v = np.zeros((3, 3), np.float32)
    t = np.array([[0, 1, 5]], np.int32)  # vertex id out of range: reported as such even without a device
    assert L.gbfwn_create(v.ctypes.data, 3, t.ctypes.data, 1, 0, ctypes.byref(out)) == M.INVALID


def test_memory_estimators(fwn_lib):
    import meshlib_gb300 as M
    est = M.memory_estimates(655362, 1310720, dims=(512, 512, 512), npts=4_000_000)
    # the result, the signed-distance columns' hand-over words (128 B per column of >= 16 tiles, or of
    # fewer tiles while under 50 items per resident warp remain), and for closed meshes the inside
    # bits (1 bit per voxel), the crossing lists (72 B per grid column) and the paired walk's fix list
    # (16 B per two tiles of 32 voxels and per work item)
    extra = est["from_grid"] - est["mesh"] - 512 ** 3 * 4 - 512 ** 3 // 8 - 512 * 512 * 72 - 512 - 512 ** 3 // 32 * 8 - 32
    assert 0 < extra <= (512 ** 3 // 4 + 50 * 160 * 32 * 128) * (1 + 16 / 128)
    # points in and results out, Morton order and its sort scratch
    assert est["from_vector"] - est["mesh"] == 4_000_000 * 40 + 4096
    # the peak is the build: 352 B kept and up to 244 B of work arrays per face, 12 B per vertex
    L = fwn_lib
    one, two = L.gbfwn_mesh_memory(655362, 1310720), L.gbfwn_mesh_memory(655362, 2 * 1310720)
    assert (two - one) == 596 * 1310720 and one == est["mesh"]
    assert L.gbfwn_mesh_memory(2 * 655362, 1310720) - one == 12 * 655362


def test_version(fwn_lib):
    import meshlib_gb300 as M
    assert b"sm_103a" in M.lib().gbfwn_version()


def test_no_cpu_fallback_when_library_missing(tmp_path, monkeypatch):
    import meshlib_gb300 as M
    monkeypatch.setattr(M, "_lib", None)
    monkeypatch.setattr(M, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        M.lib()


def test_host_output_buffer_is_checked_before_the_library_writes():
    """A caller-supplied result array must be exactly what the library writes through its pointer."""
    import types

    import numpy as np

    import meshlib_gb300 as M
    dims, xf = (4, 3, 2), np.eye(3, 4, dtype=np.float32)
    dummy = types.SimpleNamespace()  # the check runs before any use of the handle
    bad = [np.empty(24, np.float64), np.empty(23, np.float32), np.empty(48, np.float32)[::2],
           np.empty((24, 2), np.float32)[:, 0]]
    ro = np.empty(24, np.float32)
    ro.flags.writeable = False
    for out in bad + [ro, [0.0] * 24]:
        with pytest.raises(ValueError):
            M.FastWindingNumber.calcFromGridWithDistances(dummy, dims, xf, out=out)
