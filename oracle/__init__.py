"""ctypes front-end of the CPU oracle (oracle/fwn_oracle.cpp, oracle/mc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py -- never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle.so")
_lib = None


class Options(ctypes.Structure):
    """Mirror of MR::DistanceToMeshOptions (MRMesh/MRDistanceToMeshOptions.h:10-33)."""
    _fields_ = [("minDistSq", ctypes.c_float), ("maxDistSq", ctypes.c_float), ("nullOutsideMinMax", ctypes.c_int),
                ("windingNumberThreshold", ctypes.c_float), ("windingNumberBeta", ctypes.c_float)]


def build(force: bool = False) -> str:
    """Compiles the oracle with the host compiler (no FMA contraction, so FP32 follows the reference)
    and the launcher of the reference's GPU kernels (oracle/mrcuda_runner.cpp)."""
    srcs = [os.path.join(_HERE, f) for f in ("fwn_oracle.cpp", "mc_oracle.cpp")]
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < max(os.path.getmtime(s) for s in srcs):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                               "-o", _SO] + srcs)
    from . import mrcuda
    mrcuda.build_runner(force)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        vp, fp, ip, dp = ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp, ip, vp, ip]
        L.orc_destroy.argtypes = [vp]
        L.orc_num_nodes.restype = ip
        L.orc_num_nodes.argtypes = [vp]
        L.orc_get_nodes.argtypes = [vp, vp]
        L.orc_get_dipoles_f.argtypes = [vp, vp]
        L.orc_get_dipoles_d.argtypes = [vp, vp]
        L.orc_solid_angle_f.restype = fp
        L.orc_solid_angle_f.argtypes = [vp, vp]
        L.orc_solid_angle_d.restype = dp
        L.orc_solid_angle_d.argtypes = [vp, vp]
        L.orc_closest_point_d.argtypes = [vp, vp, vp]
        L.orc_from_vector.argtypes = [vp, vp, ctypes.c_int64, fp, ip, ip, ip, vp]
        L.orc_self_intersections.argtypes = [vp, fp, ip, ip, vp, vp]
        L.orc_from_grid.argtypes = [vp, vp, vp, fp, ip, ip, vp]
        L.orc_from_grid_with_distances.argtypes = [vp, vp, vp, ctypes.POINTER(Options), ip, ip, vp, vp]
        L.orc_vector_with_distances.argtypes = [vp, vp, ctypes.c_int64, ctypes.POINTER(Options), ip, ip, vp]
        L.orc_grid_voxels.argtypes = [vp, vp, vp, vp, ctypes.c_int64, ctypes.POINTER(Options), ip, ip, ip, vp, vp]
        L.orc_self_intersections_at.argtypes = [vp, vp, ctypes.c_int64, fp, ip, ip, vp, vp]
        L.orc_dist_sq.argtypes = [vp, vp, ctypes.c_int64, fp, fp, ip, vp]
        L.orc_traversal_counts.argtypes = [vp, vp, ctypes.c_int64, ctypes.POINTER(Options), vp]
        L.orc_exact_wn.argtypes = [vp, vp, ctypes.c_int64, ip, vp]
        L.orc_find_projections.argtypes = [vp, vp, ctypes.c_int64, vp, vp, fp, fp, ip, vp]
        L.orc_refit.argtypes = [vp, vp, vp]
        L.orc_is_rigid.restype = ip
        L.orc_is_rigid.argtypes = [vp]
        L.orc_mc.restype = vp
        L.orc_mc.argtypes = [vp, vp, vp, vp, fp, ip, vp, ip, ctypes.c_int64]
        L.orc_mc_num_points.restype = ctypes.c_int64
        L.orc_mc_num_points.argtypes = [vp]
        L.orc_mc_num_tris.restype = ctypes.c_int64
        L.orc_mc_num_tris.argtypes = [vp]
        L.orc_mc_error.restype = ctypes.c_char_p
        L.orc_mc_error.argtypes = [vp]
        L.orc_mc_get.argtypes = [vp, vp, vp, vp]
        L.orc_mc_free.argtypes = [vp]
        L.orc_mc_plan.restype = ctypes.c_char_p
        L.orc_mc_plan.argtypes = [ip]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def make_options(minDistSq=0.0, maxDistSq=3.4028234663852886e38, nullOutsideMinMax=True, windingNumberThreshold=0.5,
                 windingNumberBeta=2.0) -> Options:
    return Options(minDistSq, maxDistSq, int(bool(nullOutsideMinMax)), windingNumberThreshold, windingNumberBeta)


class Oracle:
    """The reference CPU FastWindingNumber restated: tree, dipoles, and the four queries,
    in FP32 (prec=0, the reference arithmetic) or FP64 (prec=1)."""

    def __init__(self, verts: np.ndarray, faces: np.ndarray):
        self.verts = np.ascontiguousarray(verts, np.float32)
        self.faces = np.ascontiguousarray(faces, np.int32)
        self.L = lib()
        self.h = self.L.orc_create(_ptr(self.verts), len(self.verts), _ptr(self.faces), len(self.faces))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def nodes(self) -> np.ndarray:
        """Reference node array: structured (min float3, max float3, l int, r int)."""
        dt = np.dtype([("min", np.float32, 3), ("max", np.float32, 3), ("l", np.int32), ("r", np.int32)])
        out = np.empty(self.L.orc_num_nodes(self.h), dt)
        self.L.orc_get_nodes(self.h, _ptr(out))
        return out

    def dipoles(self, prec: int = 0) -> np.ndarray:
        n = self.L.orc_num_nodes(self.h)
        if prec == 0:
            out = np.empty((n, 8), np.float32)
            self.L.orc_get_dipoles_f(self.h, _ptr(out))
        else:
            out = np.empty((n, 8), np.float64)
            self.L.orc_get_dipoles_d(self.h, _ptr(out))
        return out

    def from_vector(self, pts, beta=2.0, skip_face=-1, prec=0, threads=None):
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.empty(len(pts), np.float64)
        self.L.orc_from_vector(self.h, _ptr(pts), len(pts), beta, skip_face, prec, threads or default_threads(), _ptr(out))
        return out

    def self_intersections(self, beta=2.0, prec=0, threads=None):
        bits = np.empty(len(self.faces), np.uint8)
        wn = np.empty(len(self.faces), np.float64)
        self.L.orc_self_intersections(self.h, beta, prec, threads or default_threads(), _ptr(bits), _ptr(wn))
        return bits.astype(bool), wn

    def from_grid(self, dims, xf, beta=2.0, prec=0, threads=None):
        d = np.asarray(dims, np.int32)
        xf = np.ascontiguousarray(xf, np.float32)
        out = np.empty(int(np.prod(d.astype(np.int64))), np.float64)
        self.L.orc_from_grid(self.h, _ptr(d), _ptr(xf), beta, prec, threads or default_threads(), _ptr(out))
        return out

    def from_grid_with_distances(self, dims, xf, opts: Options | None = None, prec=0, threads=None, want_fwn=False):
        d = np.asarray(dims, np.int32)
        xf = np.ascontiguousarray(xf, np.float32)
        n = int(np.prod(d.astype(np.int64)))
        out = np.empty(n, np.float64)
        fwn = np.empty(n, np.float64) if want_fwn else None
        o = opts or make_options()
        self.L.orc_from_grid_with_distances(self.h, _ptr(d), _ptr(xf), ctypes.byref(o), prec, threads or default_threads(),
                                            _ptr(out), _ptr(fwn) if fwn is not None else None)
        return (out, fwn) if want_fwn else out

    def grid_voxels(self, dims, xf, ids, opts: Options | None = None, distances=True, prec=0, threads=None):
        """calcFromGridWithDistances (distances=True) or calcFromGrid (False; beta from opts) at the
        voxels with linear ids `ids` (x fastest) of the dims grid; returns (values, winding numbers)."""
        d = np.asarray(dims, np.int32)
        xf = np.ascontiguousarray(xf, np.float32)
        ids = np.ascontiguousarray(ids, np.int64)
        out = np.empty(len(ids), np.float64)
        fwn = np.empty(len(ids), np.float64)
        o = opts or make_options()
        self.L.orc_grid_voxels(self.h, _ptr(d), _ptr(xf), _ptr(ids), len(ids), ctypes.byref(o), 1 if distances else 0, prec,
                               threads or default_threads(), _ptr(out), _ptr(fwn))
        return out, fwn

    def self_intersections_at(self, faces, beta=2.0, prec=0, threads=None):
        """calcSelfIntersections bits and centroid winding numbers at the given faces only."""
        faces = np.ascontiguousarray(faces, np.int32)
        bits = np.empty(len(faces), np.uint8)
        wn = np.empty(len(faces), np.float64)
        self.L.orc_self_intersections_at(self.h, _ptr(faces), len(faces), beta, prec, threads or default_threads(), _ptr(bits),
                                         _ptr(wn))
        return bits.astype(bool), wn

    def vector_with_distances(self, pts, opts: Options | None = None, prec=0, threads=None):
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.empty(len(pts), np.float64)
        o = opts or make_options()
        self.L.orc_vector_with_distances(self.h, _ptr(pts), len(pts), ctypes.byref(o), prec, threads or default_threads(), _ptr(out))
        return out

    def dist_sq(self, pts, maxDistSq=3.4028234663852886e38, minDistSq=0.0, threads=None):
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.empty(len(pts), np.float32)
        self.L.orc_dist_sq(self.h, _ptr(pts), len(pts), maxDistSq, minDistSq, threads or default_threads(), _ptr(out))
        return out

    def traversal_counts(self, pts, opts: Options | None = None):
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.zeros(4, np.uint64)
        o = opts or make_options()
        self.L.orc_traversal_counts(self.h, _ptr(pts), len(pts), ctypes.byref(o), _ptr(out))
        return out

    def find_projections(self, pts, objXf=None, refXf=None, upDistLimitSq=3.4028234663852886e38, loDistLimitSq=0.0,
                         threads=None) -> np.ndarray:
        """PointsToMeshProjector::findProjections (reference CPU arithmetic: FP64 leaf projection):
        structured records (face, point[3], edge=-1, bary[2], distSq), the MeshProjectionResult layout."""
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        dt = np.dtype([("face", np.int32), ("point", np.float32, 3), ("edge", np.int32), ("bary", np.float32, 2),
                       ("distSq", np.float32)])
        out = np.empty(len(pts), dt)
        ox = None if objXf is None else np.ascontiguousarray(objXf, np.float32).reshape(12)
        rx = None if refXf is None else np.ascontiguousarray(refXf, np.float32).reshape(12)
        self.L.orc_find_projections(self.h, _ptr(pts), len(pts), _ptr(ox) if ox is not None else None,
                                    _ptr(rx) if rx is not None else None, upDistLimitSq, loDistLimitSq,
                                    threads or default_threads(), _ptr(out))
        return out

    def refit(self, verts, changed=None):
        """AABBTree::refit + dipoles for moved vertices; changed: bool array over vertices or None (all)."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        assert v.shape == self.verts.shape
        bits = None
        if changed is not None:
            c = np.asarray(changed, bool).reshape(-1)
            b = np.zeros(((len(c) + 63) // 64) * 64, bool)
            b[:len(c)] = c
            bits = np.packbits(b, bitorder="little").view(np.uint64).copy()
        self.L.orc_refit(self.h, _ptr(v), _ptr(bits) if bits is not None else None)

    def exact_wn(self, pts, threads=None):
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.empty(len(pts), np.float64)
        self.L.orc_exact_wn(self.h, _ptr(pts), len(pts), threads or default_threads(), _ptr(out))
        return out


def solid_angle_f(p, tri) -> float:
    p = np.ascontiguousarray(p, np.float32)
    tri = np.ascontiguousarray(tri, np.float32)
    return float(lib().orc_solid_angle_f(_ptr(p), _ptr(tri)))


def solid_angle_d(p, tri) -> float:
    p = np.ascontiguousarray(p, np.float64)
    tri = np.ascontiguousarray(tri, np.float64)
    return float(lib().orc_solid_angle_d(_ptr(p), _ptr(tri)))


def is_rigid(xf) -> bool:
    """MRMatrix3Decompose.h isRigid of the 3x3 part of a 12-float transform."""
    x = np.ascontiguousarray(xf, np.float32).reshape(12)
    return bool(lib().orc_is_rigid(_ptr(x)))


def grid_points(dims, xf) -> np.ndarray:
    """Voxel centres in the reference order (x fastest), computed in float like the reference."""
    nx, ny, nz = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)
    A = np.asarray(xf[:9], np.float32).reshape(3, 3)
    b = np.asarray(xf[9:12], np.float32)
    out = np.empty_like(p)
    for r in range(3):
        out[:, r] = (p[:, 0] * A[r, 0] + p[:, 1] * A[r, 1]) + p[:, 2] * A[r, 2] + b[r]
    return out


class McError(RuntimeError):
    """An error string of the restated mesher (the reference's Expected<TriMesh> error)."""


def marching_cubes(vol, origin=(0.0, 0.0, 0.0), voxel_size=(1.0, 1.0, 1.0), iso=0.0, less_inside=False,
                   part_starts=None, max_vertices=2**31 - 1):
    """Restated MeshLib VolumeMesher (oracle/mc_oracle.cpp).  vol: (nz, ny, nx) float32 (x fastest).
    part_starts: first layer of each overlapping part (MarchingCubesByParts), None = whole volume.
    Returns (points (n, 3) float32, tris (m, 3) int32, faceMap (m,) int32); raises McError."""
    v = np.ascontiguousarray(vol, np.float32)
    nz, ny, nx = v.shape
    dims = np.array([nx, ny, nz], np.int32)
    o = np.ascontiguousarray(origin, np.float32)
    vs = np.ascontiguousarray(voxel_size, np.float32)
    ps = None if part_starts is None else np.ascontiguousarray(part_starts, np.int32)
    L = lib()
    r = L.orc_mc(_ptr(v), _ptr(dims), _ptr(o), _ptr(vs), float(iso), int(bool(less_inside)),
                 _ptr(ps) if ps is not None else None, 0 if ps is None else len(ps), int(max_vertices))
    try:
        err = L.orc_mc_error(r).decode()
        if err:
            raise McError(err)
        npt, ntr = L.orc_mc_num_points(r), L.orc_mc_num_tris(r)
        pts = np.empty((npt, 3), np.float32)
        tris = np.empty((ntr, 3), np.int32)
        fmap = np.empty(ntr, np.int32)
        L.orc_mc_get(r, _ptr(pts), _ptr(tris), _ptr(fmap))
        return pts, tris, fmap
    finally:
        L.orc_mc_free(r)


def mc_plan(config: int) -> str:
    """Triangulation plan of a cube configuration (hex digits, three per triangle)."""
    return lib().orc_mc_plan(int(config)).decode()
