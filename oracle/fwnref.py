"""ctypes front-end of MeshLib's own CPU winding-number / signed-distance path, built from the
reference sources into oracle/_ref/libfwnref.so by oracle/ref/build_cpu_ref.py (x86-64 hosts with a
copy of the reference).  Every call runs on one core (the TBB stand-in is serial).

TEST INFRASTRUCTURE ONLY: used to generate tests/golden/fwn_cpu_reference.npz, to re-check it where
the library exists, and to time the reference code against the oracle's port.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_ref", "libfwnref.so")
_lib = None
NODE_DTYPE = np.dtype([("min", np.float32, 3), ("max", np.float32, 3), ("l", np.int32), ("r", np.int32)])


def available() -> bool:
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        vp, i64, f32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float
        L.fwnref_create.restype = vp
        L.fwnref_create.argtypes = [vp, i64, vp, i64]
        L.fwnref_destroy.argtypes = [vp]
        L.fwnref_num_nodes.restype = i64
        L.fwnref_num_nodes.argtypes = [vp]
        L.fwnref_nodes.argtypes = [vp, vp]
        L.fwnref_dipoles.argtypes = [vp, vp]
        L.fwnref_from_grid_with_distances.argtypes = [vp, vp, vp, vp, vp]
        L.fwnref_from_grid.argtypes = [vp, vp, vp, f32, vp]
        L.fwnref_from_vector.argtypes = [vp, vp, i64, f32, ctypes.c_int32, vp]
        L.fwnref_self_intersections.argtypes = [vp, f32, vp]
        L.fwnref_grid_voxels.argtypes = [vp, vp, vp, vp, vp, i64, vp]
        L.fwnref_project.argtypes = [vp, vp, i64, f32, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _opts(minDistSq=0.0, maxDistSq=3.4028234663852886e38, nullOutsideMinMax=True, windingNumberThreshold=0.5,
          windingNumberBeta=2.0):
    return np.array([minDistSq, maxDistSq, float(bool(nullOutsideMinMax)), windingNumberThreshold, windingNumberBeta],
                    np.float32)


class Reference:
    """MR::Mesh::fromTriangles + MR::FastWindingNumber on the given triangles (face ids kept)."""

    def __init__(self, verts, faces):
        self.verts = np.ascontiguousarray(verts, np.float32)
        self.faces = np.ascontiguousarray(faces, np.int32)
        self.L = lib()
        self.h = self.L.fwnref_create(_p(self.verts), len(self.verts), _p(self.faces), len(self.faces))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fwnref_destroy(self.h)
            self.h = None

    def nodes(self):
        out = np.empty(self.L.fwnref_num_nodes(self.h), NODE_DTYPE)
        self.L.fwnref_nodes(self.h, _p(out))
        return out

    def dipoles(self):
        out = np.empty((self.L.fwnref_num_nodes(self.h), 8), np.float32)
        self.L.fwnref_dipoles(self.h, _p(out))
        return out

    def from_grid_with_distances(self, dims, xf, **opts):
        d = np.asarray(dims, np.int32)
        out = np.empty(int(np.prod(d.astype(np.int64))), np.float32)
        x = np.ascontiguousarray(xf, np.float32)
        assert self.L.fwnref_from_grid_with_distances(self.h, _p(d), _p(x), _p(_opts(**opts)), _p(out)) == 0
        return out

    def from_grid(self, dims, xf, beta=2.0):
        d = np.asarray(dims, np.int32)
        out = np.empty(int(np.prod(d.astype(np.int64))), np.float32)
        x = np.ascontiguousarray(xf, np.float32)
        assert self.L.fwnref_from_grid(self.h, _p(d), _p(x), beta, _p(out)) == 0
        return out

    def from_vector(self, pts, beta=2.0, skip_face=-1):
        p = np.ascontiguousarray(pts, np.float32)
        out = np.empty(len(p), np.float32)
        assert self.L.fwnref_from_vector(self.h, _p(p), len(p), beta, skip_face, _p(out)) == 0
        return out

    def self_intersections(self, beta=2.0):
        out = np.empty(len(self.faces), np.uint8)
        assert self.L.fwnref_self_intersections(self.h, beta, _p(out)) == 0
        return out.astype(bool)

    def grid_voxels(self, dims, xf, ids, **opts):
        d = np.asarray(dims, np.int32)
        x = np.ascontiguousarray(xf, np.float32)
        i = np.ascontiguousarray(ids, np.int64)
        out = np.empty(len(i), np.float32)
        self.L.fwnref_grid_voxels(self.h, _p(d), _p(x), _p(_opts(**opts)), _p(i), len(i), _p(out))
        return out

    def project(self, pts, up_dist_limit_sq=3.4028234663852886e38):
        """Per point: (distSq, face, point xyz, barycentric a, b, edge) of findProjection."""
        p = np.ascontiguousarray(pts, np.float32)
        out = np.empty((len(p), 8), np.float32)
        self.L.fwnref_project(self.h, _p(p), len(p), up_dist_limit_sq, _p(out))
        face = out[:, 1].view(np.int32).copy()
        edge = out[:, 7].view(np.int32).copy()
        return out[:, 0].copy(), face, out[:, 2:5].copy(), out[:, 5:7].copy(), edge
