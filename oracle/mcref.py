"""ctypes front-end of MeshLib's own CPU mesher, built from the reference sources into
oracle/_ref/libmcref.so by oracle/ref/build_cpu_ref.py (x86-64 hosts with a copy of the reference).

TEST INFRASTRUCTURE ONLY: used to generate tests/golden/mc_reference.npz and, where the library
exists, to re-check that fixture.  Same calling convention as oracle.marching_cubes.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_ref", "libmcref.so")
_lib = None


class McRefError(RuntimeError):
    pass


def available() -> bool:
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        L.mcref_run.restype = vp
        L.mcref_run.argtypes = [vp, vp, vp, vp, ctypes.c_float, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.mcref_num_points.restype = ctypes.c_int64
        L.mcref_num_points.argtypes = [vp]
        L.mcref_num_tris.restype = ctypes.c_int64
        L.mcref_num_tris.argtypes = [vp]
        L.mcref_error.restype = ctypes.c_char_p
        L.mcref_error.argtypes = [vp]
        L.mcref_get.argtypes = [vp, vp, vp, vp]
        L.mcref_free.argtypes = [vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def marching_cubes(vol, origin=(0.0, 0.0, 0.0), voxel_size=(1.0, 1.0, 1.0), iso=0.0, less_inside=False,
                   part_starts=None, max_vertices=2**31 - 1, layers_per_block=0):
    """MeshLib's marchingCubesAsTriMesh (whole volume, layers_per_block 0) or MarchingCubesByParts fed
    the parts that start at part_starts.  vol: (nz, ny, nx) float32.  Returns (points, tris, faceMap);
    raises McRefError with the reference's message."""
    v = np.ascontiguousarray(vol, np.float32)
    nz, ny, nx = v.shape
    dims = np.array([nx, ny, nz], np.int32)
    o = np.ascontiguousarray(origin, np.float32)
    vs = np.ascontiguousarray(voxel_size, np.float32)
    ps = None if part_starts is None else np.ascontiguousarray(part_starts, np.int32)
    L = lib()
    h = L.mcref_run(_ptr(v), _ptr(dims), _ptr(o), _ptr(vs), float(iso), int(bool(less_inside)), _ptr(ps),
                    0 if ps is None else len(ps), int(max_vertices), int(layers_per_block))
    try:
        err = L.mcref_error(h).decode()
        if err:
            raise McRefError(err)
        n, m = L.mcref_num_points(h), L.mcref_num_tris(h)
        pts = np.empty((n, 3), np.float32)
        tris = np.empty((m, 3), np.int32)
        fmap = np.empty(m, np.int32)
        L.mcref_get(h, _ptr(pts), _ptr(tris), _ptr(fmap))
        return pts, tris, fmap
    finally:
        L.mcref_free(h)
