"""GB300-native fast winding number / signed distance for triangle meshes.

Python front-end over the C ABI in ``include/gbfwn.h`` (library ``libgbfwn.so`` built in-tree by
``meshlib_gb300.build``).  The class :class:`FastWindingNumber` mirrors MeshLib's
``MR::IFastWindingNumber`` / ``IFastWindingNumberByParts`` (MRMesh/MRFastWindingNumber.h:11-107)
method for method -- the same names as the reference's Python bindings
(``mrcudapy.FastWindingNumber(mesh)``), numpy arrays in and out.  Errors raise
:class:`FwnError` (the reference returns ``Expected<void>``; its bindings raise).

There is no CPU fallback: every call goes to the CUDA library, and importing the module on a
machine without the built library raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbfwn.so")
FLT_MAX = 3.4028234663852886e38

OK, CANCELLED, OUT_OF_MEMORY, CUDA_ERROR, INVALID, TIMEOUT, TRAVERSAL_OVERFLOW = range(7)


class FwnError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class _DistOpts(ctypes.Structure):
    _fields_ = [("minDistSq", ctypes.c_float), ("maxDistSq", ctypes.c_float), ("nullOutsideMinMax", ctypes.c_int32),
                ("windingNumberThreshold", ctypes.c_float), ("windingNumberBeta", ctypes.c_float)]


@dataclass
class DistanceToMeshOptions:
    """MR::DistanceToMeshOptions (MRMesh/MRDistanceToMeshOptions.h:10-33), same defaults."""
    minDistSq: float = 0.0
    maxDistSq: float = FLT_MAX
    nullOutsideMinMax: bool = True
    windingNumberThreshold: float = 0.5
    windingNumberBeta: float = 2.0

    def _c(self) -> _DistOpts:
        return _DistOpts(self.minDistSq, self.maxDistSq, int(bool(self.nullOutsideMinMax)), self.windingNumberThreshold,
                         self.windingNumberBeta)


class _SurrogateOpts(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_int64), ("validation", ctypes.c_int64), ("steps", ctypes.c_int32),
                ("batch", ctypes.c_int32), ("learningRate", ctypes.c_float), ("band", ctypes.c_float),
                ("beta", ctypes.c_float), ("seed", ctypes.c_uint64)]


class _SurrogateStats(ctypes.Structure):
    _fields_ = [("trainLoss", ctypes.c_float), ("validationMaxError", ctypes.c_float), ("margin", ctypes.c_float),
                ("sampleSeconds", ctypes.c_float), ("trainSeconds", ctypes.c_float), ("steps", ctypes.c_int32),
                ("validationOverestimate", ctypes.c_float), ("limit", ctypes.c_float)]


class _BandedStats(ctypes.Structure):
    _fields_ = [("bricks", ctypes.c_int32), ("keptBricks", ctypes.c_int32), ("cullMs", ctypes.c_float),
                ("exactMs", ctypes.c_float)]


class _McParams(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("voxelSize", ctypes.c_float * 3), ("iso", ctypes.c_float),
                ("lessInside", ctypes.c_int32), ("maxVertices", ctypes.c_int64), ("wantFaceMap", ctypes.c_int32)]


class _BatchItem(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_void_p), ("dims", ctypes.c_int32 * 3), ("xf", ctypes.c_float * 12), ("opts", _DistOpts),
                ("d_out", ctypes.c_void_p)]


SURROGATE_PARAMS = 74369
SURROGATE_META = 48

PROGRESS = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_float, ctypes.c_void_p)
SLAB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                        ctypes.c_void_p)

# (name, restype, argtypes) of every exported symbol of include/gbfwn.h
_vp, _i32, _i64, _f = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
_SIGS = [
    ("gbfwn_version", ctypes.c_char_p, []),
    ("gbfwn_last_error", ctypes.c_char_p, []),
    ("gbfwn_set_precise", None, [_vp, ctypes.c_int]),
    ("gbfwn_set_sign_reuse", None, [_vp, ctypes.c_int]),
    ("gbfwn_is_closed", ctypes.c_int, [_vp]),
    ("gbfwn_create", ctypes.c_int, [_vp, _i64, _vp, _i64, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("gbfwn_create_dev", ctypes.c_int, [_vp, _i64, _vp, _i64, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("gbfwn_destroy", ctypes.c_int, [_vp]),
    ("gbfwn_num_faces", _i64, [_vp]),
    ("gbfwn_num_nodes", _i64, [_vp]),
    ("gbfwn_get_tree", ctypes.c_int, [_vp, _vp, _vp]),
    ("gbfwn_from_vector", ctypes.c_int, [_vp, _vp, _i64, _f, _i32, _vp, PROGRESS, _vp]),
    ("gbfwn_from_vector_dev", ctypes.c_int, [_vp, _vp, _i64, _f, _i32, _vp, _vp]),
    ("gbfwn_self_intersections", ctypes.c_int, [_vp, _f, _vp, _vp, PROGRESS, _vp]),
    ("gbfwn_self_intersections_dev", ctypes.c_int, [_vp, _f, _vp, _vp, _vp]),
    ("gbfwn_from_grid", ctypes.c_int, [_vp, _vp, _vp, _f, _vp, PROGRESS, _vp]),
    ("gbfwn_from_grid_dev", ctypes.c_int, [_vp, _vp, _vp, _f, _vp, _vp]),
    ("gbfwn_from_grid_with_distances", ctypes.c_int, [_vp, _vp, _vp, ctypes.POINTER(_DistOpts), _vp, PROGRESS, _vp]),
    ("gbfwn_from_grid_with_distances_dev", ctypes.c_int, [_vp, _vp, _vp, ctypes.POINTER(_DistOpts), _vp, _vp]),
    ("gbfwn_from_grid_with_distances_noalloc", ctypes.c_int,
     [_vp, _vp, _vp, ctypes.POINTER(_DistOpts), _vp, _vp]),
    ("gbfwn_vector_with_distances", ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(_DistOpts), _vp, PROGRESS, _vp]),
    ("gbfwn_vector_with_distances_dev", ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(_DistOpts), _vp, _vp]),
    ("gbfwn_from_grid_by_parts", ctypes.c_int, [_vp, _vp, _vp, _f, _i32, _i32, SLAB, _vp, PROGRESS, _vp]),
    ("gbfwn_from_grid_with_distances_by_parts", ctypes.c_int,
     [_vp, _vp, _vp, ctypes.POINTER(_DistOpts), _i32, _i32, SLAB, _vp, PROGRESS, _vp]),
    ("gbfwn_mesh_memory", ctypes.c_size_t, [_i64, _i64]),
    ("gbfwn_from_grid_memory", ctypes.c_size_t, [_i64, _i64, _vp]),
    ("gbfwn_from_vector_memory", ctypes.c_size_t, [_i64, _i64, _i64]),
    ("gbfwn_self_intersections_memory", ctypes.c_size_t, [_i64, _i64]),
    ("gbfwn_debug_fail_next_allocs", None, [ctypes.c_int]),
    ("gbfwn_debug_wait_timeout", ctypes.c_int, [ctypes.c_uint32, _vp]),
    ("gbfwn_debug_gemm_bf16", ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    ("gbfwn_batch_create", ctypes.c_int, [ctypes.POINTER(_BatchItem), _i32, ctypes.POINTER(_vp)]),
    ("gbfwn_batch_destroy", ctypes.c_int, [_vp]),
    ("gbfwn_batch_num_configs", _i32, []),
    ("gbfwn_batch_config_name", ctypes.c_char_p, [_i32]),
    ("gbfwn_batch_set_config", ctypes.c_int, [_vp, _i32]),
    ("gbfwn_batch_autotune", ctypes.c_int, [_vp, ctypes.POINTER(_i32), _vp]),
    ("gbfwn_batch_run_dev", ctypes.c_int, [_vp, _vp]),
    ("gbfwn_batch_graph_launch", ctypes.c_int, [_vp, _vp]),
    ("gbfwn_surrogate_default_opts", None, [ctypes.POINTER(_SurrogateOpts)]),
    ("gbfwn_surrogate_train", ctypes.c_int,
     [_vp, _vp, _vp, ctypes.POINTER(_SurrogateOpts), ctypes.POINTER(_vp), ctypes.POINTER(_SurrogateStats)]),
    ("gbfwn_surrogate_destroy", ctypes.c_int, [_vp]),
    ("gbfwn_surrogate_get", ctypes.c_int, [_vp, _vp, _vp]),
    ("gbfwn_surrogate_create", ctypes.c_int, [ctypes.c_int, _vp, _vp, ctypes.POINTER(_vp)]),
    ("gbfwn_surrogate_eval_dev", ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    ("gbfwn_surrogate_gradients_dev", ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _vp]),
    ("gbfwn_from_grid_with_distances_banded_dev", ctypes.c_int,
     [_vp, _vp, _vp, _vp, ctypes.POINTER(_DistOpts), _vp, ctypes.POINTER(_BandedStats), _vp]),
    ("gbfwn_from_grid_slab_dev", ctypes.c_int, [_vp, _vp, _vp, _f, _i32, _i32, _vp, _vp]),
    ("gbfwn_from_grid_with_distances_slab_dev", ctypes.c_int,
     [_vp, _vp, _vp, ctypes.POINTER(_DistOpts), _i32, _i32, _vp, _vp]),
    ("gbfwn_refit", ctypes.c_int, [_vp, _vp, _vp]),
    ("gbfwn_refit_dev", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("gbfwn_find_projections", ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _f, _f, _vp, PROGRESS, _vp]),
    ("gbfwn_find_projections_dev", ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _f, _f, _vp, _vp]),
    ("gbfwn_projections_heap_bytes", ctypes.c_size_t, [_i64]),
    ("gbfwn_make_signed_by_winding_number_dev", ctypes.c_int, [_vp, _vp, _vp, _f, _f, _vp, _vp]),
    ("gbfwn_mc_default_params", None, [ctypes.POINTER(_McParams)]),
    ("gbfwn_marching_cubes", ctypes.c_int,
     [_vp, _vp, ctypes.POINTER(_McParams), _vp, _i32, ctypes.c_int, ctypes.POINTER(_vp), PROGRESS, _vp]),
    ("gbfwn_marching_cubes_dev", ctypes.c_int,
     [_vp, _vp, ctypes.POINTER(_McParams), _vp, _i32, ctypes.c_int, ctypes.POINTER(_vp), _vp]),
    ("gbfwn_mc_release_workspace", ctypes.c_int, [ctypes.c_int]),
    ("gbfwn_release_cached_memory", ctypes.c_int, [ctypes.c_int]),
    ("gbfwn_marching_cubes_memory", ctypes.c_size_t, [_vp, _i64]),
    ("gbfwn_trimesh_sizes", ctypes.c_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    ("gbfwn_trimesh_copy", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("gbfwn_trimesh_device", ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    ("gbfwn_trimesh_destroy", ctypes.c_int, [_vp]),
    ("gbfwn_mc_parts_create", ctypes.c_int, [_vp, ctypes.POINTER(_McParams), ctypes.c_int, ctypes.POINTER(_vp)]),
    ("gbfwn_mc_parts_next_z", _i32, [_vp]),
    ("gbfwn_mc_parts_add", ctypes.c_int, [_vp, _vp, _vp]),
    ("gbfwn_mc_parts_add_dev", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("gbfwn_mc_parts_finalize", ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    ("gbfwn_mc_parts_destroy", ctypes.c_int, [_vp]),
    ("gbfwn_grid_to_mesh", ctypes.c_int,
     [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_DistOpts), ctypes.POINTER(_McParams), _vp, _i32, ctypes.POINTER(_vp),
      PROGRESS, _vp]),
]
EXPORTED = [s[0] for s in _SIGS]

_lib = None


def lib():
    """Loads ``libgbfwn.so`` (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m meshlib_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in _SIGS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(st: int):
    if st != OK:
        raise FwnError(st, lib().gbfwn_last_error().decode())


def _progress(cb: Optional[Callable[[float], bool]]):
    if cb is None:
        return PROGRESS(), None
    fn = PROGRESS(lambda p, _u: 1 if cb(float(p)) else 0)
    return fn, fn


def _stream(s) -> ctypes.c_void_p:
    """None: the handle's own stream; 0: the legacy default stream (cudaStreamLegacy); else a cudaStream_t."""
    if s is None:
        return ctypes.c_void_p(None)
    return ctypes.c_void_p(1 if int(s) == 0 else int(s))


def _xf12(xf) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(xf, np.float32).reshape(-1))
    if a.size != 12:
        raise ValueError("gridToMeshXf must be 12 floats: 3x3 rows then translation")
    return a


class FastWindingNumber:
    """GB300 implementation of ``MR::IFastWindingNumber`` + ``IFastWindingNumberByParts``.

    ``verts``: (nv, 3) float32, ``faces``: (nt, 3) int32 (a face with a negative id is invalid).
    The tree and dipoles are built on the device at construction and cached, as
    ``MR::Cuda::FastWindingNumber::prepareData_`` caches them (MRCuda/MRCudaFastWindingNumber.cpp:46-85).
    """

    def __init__(self, verts: np.ndarray, faces: np.ndarray, device: int = 0, precise: bool = True):
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        self._h = ctypes.c_void_p()
        self._L = lib()
        _check(self._L.gbfwn_create(_p(self.verts), len(self.verts), _p(self.faces), len(self.faces), device,
                                    ctypes.byref(self._h)))
        self.set_precise(precise)

    @classmethod
    def from_device(cls, d_verts_ptr: int, nv: int, d_faces_ptr: int, nt: int, device: int = 0, precise: bool = True):
        self = cls.__new__(cls)
        self.verts = self.faces = None
        self._h = ctypes.c_void_p()
        self._L = lib()
        _check(self._L.gbfwn_create_dev(ctypes.c_void_p(d_verts_ptr), nv, ctypes.c_void_p(d_faces_ptr), nt, device,
                                        ctypes.byref(self._h)))
        self.set_precise(precise)
        return self

    def close(self):
        """Frees the device data; raises (and keeps the handle) while a live Batch uses the mesh."""
        if getattr(self, "_h", None) and self._h.value:
            _check(self._L.gbfwn_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def set_precise(self, precise: bool):
        self._L.gbfwn_set_precise(self._h, 1 if precise else 0)

    def set_sign_reuse(self, enable: bool):
        """Exact signs on a closed surface (default on; gbfwn_set_sign_reuse in include/gbfwn.h): grids
        with a vertical z axis from their columns' crossings, other grids and points from the voxel
        below or one vertical ray; off evaluates every winding number, as the reference does."""
        self._L.gbfwn_set_sign_reuse(self._h, 1 if enable else 0)

    def is_closed(self) -> bool:
        """True if the valid faces form a closed oriented surface (every edge used equally often in
        both directions)."""
        return bool(self._L.gbfwn_is_closed(self._h))

    def refit(self, verts: np.ndarray, changedVerts: Optional[np.ndarray] = None):
        """MR::AABBTree::refit + dipoles for moved vertices (same triangles).  ``changedVerts``: bool
        array over vertices (None = all moved)."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        bits = None
        if changedVerts is not None:
            c = np.asarray(changedVerts, bool).reshape(-1)
            words = (len(c) + 63) // 64
            bits = np.zeros(words * 64, bool)
            bits[:len(c)] = c
            bits = np.packbits(bits, bitorder="little").view(np.uint64).copy()
        _check(self._L.gbfwn_refit(self._h, _p(v), _p(bits)))
        if self.verts is not None:
            self.verts = v

    def refit_dev(self, d_verts_ptr: int, d_changed_ptr: int = 0, stream=None):
        _check(self._L.gbfwn_refit_dev(self._h, ctypes.c_void_p(d_verts_ptr), ctypes.c_void_p(d_changed_ptr or None),
                                       _stream(stream)))

    def num_faces(self) -> int:
        return int(self._L.gbfwn_num_faces(self._h))

    def tree(self):
        """(nodes, dipoles): the reference-layout tree (structured array) and (n, 8) float32 dipoles."""
        n = int(self._L.gbfwn_num_nodes(self._h))
        dt = np.dtype([("min", np.float32, 3), ("max", np.float32, 3), ("l", np.int32), ("r", np.int32)])
        nodes = np.empty(n, dt)
        dip = np.empty((n, 8), np.float32)
        _check(self._L.gbfwn_get_tree(self._h, _p(nodes), _p(dip)))
        return nodes, dip

    # -- MR::IFastWindingNumber
    def calcFromVector(self, points: np.ndarray, beta: float = 2.0, skipFace: int = -1, cb=None) -> np.ndarray:
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.empty(len(pts), np.float32)
        c, _keep = _progress(cb)
        _check(self._L.gbfwn_from_vector(self._h, _p(pts), len(pts), beta, int(skipFace), _p(out), c, None))
        return out

    def calcSelfIntersections(self, beta: float = 2.0, cb=None, with_wn: bool = False):
        """Bool array over faces (MeshLib's FaceBitSet); optionally the centroid winding numbers too."""
        nt = self.num_faces()
        words = np.zeros((nt + 63) // 64, np.uint64)
        wn = np.empty(nt, np.float32) if with_wn else None
        c, _keep = _progress(cb)
        _check(self._L.gbfwn_self_intersections(self._h, beta, _p(words), _p(wn), c, None))
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:nt].astype(bool)
        return (bits, wn) if with_wn else bits

    def calcFromGrid(self, dims, gridToMeshXf, beta: float = 2.0, cb=None) -> np.ndarray:
        d = np.asarray(dims, np.int32)
        out = np.empty(int(np.prod(d.astype(np.int64))), np.float32)
        c, _keep = _progress(cb)
        _check(self._L.gbfwn_from_grid(self._h, _p(d), _p(_xf12(gridToMeshXf)), beta, _p(out), c, None))
        return out

    def calcFromGridWithDistances(self, dims, gridToMeshXf, options: Optional[DistanceToMeshOptions] = None, cb=None,
                                  out: Optional[np.ndarray] = None) -> np.ndarray:
        d = np.asarray(dims, np.int32)
        n = int(np.prod(d.astype(np.int64)))
        if out is None:
            out = np.empty(n, np.float32)
        elif not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.flags.c_contiguous
                  and out.flags.writeable and out.size == n):
            # the library writes n floats through the raw pointer: anything else would corrupt memory
            raise ValueError(f"out must be a writeable C-contiguous float32 array of {n} elements (dims product)")
        o = (options or DistanceToMeshOptions())._c()
        c, _keep = _progress(cb)
        _check(self._L.gbfwn_from_grid_with_distances(self._h, _p(d), _p(_xf12(gridToMeshXf)), ctypes.byref(o), _p(out),
                                                       c, None))
        return out

    def calcWithDistances(self, points: np.ndarray, options: Optional[DistanceToMeshOptions] = None, cb=None) -> np.ndarray:
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.empty(len(pts), np.float32)
        o = (options or DistanceToMeshOptions())._c()
        c, _keep = _progress(cb)
        _check(self._L.gbfwn_vector_with_distances(self._h, _p(pts), len(pts), ctypes.byref(o), _p(out), c, None))
        return out

    # -- MR::IFastWindingNumberByParts
    def calcFromGridByParts(self, resFunc, dims, gridToMeshXf, beta: float = 2.0, layerOverlap: int = 0, cb=None,
                            maxLayersPerSlab: int = 0):
        self._by_parts(resFunc, dims, gridToMeshXf, None, beta, layerOverlap, cb, maxLayersPerSlab)

    def calcFromGridWithDistancesByParts(self, resFunc, dims, gridToMeshXf, options=None, layerOverlap: int = 0, cb=None,
                                         maxLayersPerSlab: int = 0):
        self._by_parts(resFunc, dims, gridToMeshXf, options or DistanceToMeshOptions(), 2.0, layerOverlap, cb,
                       maxLayersPerSlab)

    def _by_parts(self, resFunc, dims, xf, options, beta, layerOverlap, cb, maxLayers):
        d = np.asarray(dims, np.int32)
        err = []

        def slab(data, sd, zoff, _u):
            try:
                n = int(sd[0]) * int(sd[1]) * int(sd[2])
                arr = np.ctypeslib.as_array(data, shape=(n,)).copy()
                r = resFunc(arr, (int(sd[0]), int(sd[1]), int(sd[2])), int(zoff))
                return 0 if (r is None or r is True) else int(r) or 1
            except Exception as ex:  # surfaced after the call
                err.append(ex)
                return CANCELLED

        s = SLAB(slab)
        c, _keep = _progress(cb)
        if options is None:
            st = self._L.gbfwn_from_grid_by_parts(self._h, _p(d), _p(_xf12(xf)), beta, layerOverlap, maxLayers, s, None, c,
                                                 None)
        else:
            o = options._c()
            st = self._L.gbfwn_from_grid_with_distances_by_parts(self._h, _p(d), _p(_xf12(xf)), ctypes.byref(o),
                                                                layerOverlap, maxLayers, s, None, c, None)
        if err:
            raise err[0]
        _check(st)

    # -- device-pointer variants (torch tensors or any CUDA pointer); enqueue only
    def calcFromGridWithDistances_dev(self, dims, xf, d_out_ptr: int, options=None, stream=None):
        d = np.asarray(dims, np.int32)
        o = (options or DistanceToMeshOptions())._c()
        _check(self._L.gbfwn_from_grid_with_distances_dev(self._h, _p(d), _p(_xf12(xf)), ctypes.byref(o),
                                                           ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcFromGridWithDistancesBanded_dev(self, dims, xf, d_out_ptr: int, options: "DistanceToMeshOptions",
                                            surrogate: Optional["Surrogate"] = None, stream=None) -> dict:
        """Banded signed distance (finite maxDistSq, nullOutsideMinMax) with brick culling by the
        surrogate, or by exact brick-centre distances when surrogate is None."""
        d = np.asarray(dims, np.int32)
        o = options._c()
        st = _BandedStats()
        _check(self._L.gbfwn_from_grid_with_distances_banded_dev(
            self._h, surrogate.handle if surrogate is not None else None, _p(d), _p(_xf12(xf)), ctypes.byref(o),
            ctypes.c_void_p(d_out_ptr), ctypes.byref(st), _stream(stream)))
        return {"bricks": st.bricks, "keptBricks": st.keptBricks, "cullMs": st.cullMs, "exactMs": st.exactMs}

    def gridToMesh(self, dims, origin, voxelSize, options: Optional["DistanceToMeshOptions"] = None,
                   mcParams: Optional["MarchingCubesParams"] = None, surrogate: Optional["Surrogate"] = None,
                   partStarts=None, cb=None) -> "TriMesh":
        """The volume step of ``mcOffsetMesh`` (MRVoxels/MROffset.cpp:185-226) fused on the device: the
        signed-distance grid of ``dims`` voxels centred at origin + (i + 0.5) * voxelSize, then marching
        cubes on it (mcOffsetMesh passes origin, iso = offset, lessInside = True); the grid never
        leaves the GPU.  voxelSize: a float or three floats."""
        d = np.asarray(dims, np.int32)
        o = np.ascontiguousarray(origin, np.float32)
        vs = np.ascontiguousarray(np.broadcast_to(np.asarray(voxelSize, np.float32), (3,)))
        opts = (options or DistanceToMeshOptions())._c()
        mp = mcParams or MarchingCubesParams(origin=tuple(o), voxelSize=tuple(vs))
        prm = mp._c()
        ps, nps = _parts(partStarts)
        fn, _keep = _progress(cb)
        h = ctypes.c_void_p()
        _check(self._L.gbfwn_grid_to_mesh(self._h, surrogate.handle if surrogate is not None else None, _p(d), _p(o), _p(vs),
                                          ctypes.byref(opts), ctypes.byref(prm), _p(ps), nps, ctypes.byref(h), fn, None))
        return TriMesh(h)

    def calcFromGridWithDistances_noalloc(self, dims, xf, d_out_ptr: int, options=None, stream=None):
        """Allocation-free variant of calcFromGridWithDistances_dev (see gbfwn_from_grid_with_distances_noalloc)."""
        d = np.asarray(dims, np.int32)
        o = (options or DistanceToMeshOptions())._c()
        _check(self._L.gbfwn_from_grid_with_distances_noalloc(self._h, _p(d), _p(_xf12(xf)), ctypes.byref(o),
                                                               ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcFromGridSlab_dev(self, dims, xf, z0: int, z1: int, d_out_ptr: int, beta: float = 2.0, stream=None):
        """Layers [z0, z1) of the grid into d_out (the multi-GPU shard unit)."""
        d = np.asarray(dims, np.int32)
        _check(self._L.gbfwn_from_grid_slab_dev(self._h, _p(d), _p(_xf12(xf)), beta, int(z0), int(z1),
                                                ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcFromGridWithDistancesSlab_dev(self, dims, xf, z0: int, z1: int, d_out_ptr: int, options=None, stream=None):
        d = np.asarray(dims, np.int32)
        o = (options or DistanceToMeshOptions())._c()
        _check(self._L.gbfwn_from_grid_with_distances_slab_dev(self._h, _p(d), _p(_xf12(xf)), ctypes.byref(o), int(z0),
                                                               int(z1), ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcFromGrid_dev(self, dims, xf, d_out_ptr: int, beta: float = 2.0, stream=None):
        d = np.asarray(dims, np.int32)
        _check(self._L.gbfwn_from_grid_dev(self._h, _p(d), _p(_xf12(xf)), beta, ctypes.c_void_p(d_out_ptr),
                                           _stream(stream)))

    def makeSignedByWindingNumber_dev(self, dims, xf, d_values_ptr: int, beta: float = 2.0, threshold: float = 0.5,
                                      stream=None):
        """MeshLib's makeSignedByWindingNumber on a dense device grid: values of voxels whose winding
        number exceeds `threshold` are negated in place (MRVoxels/MRVDBConversions.cpp:491-571)."""
        d = np.asarray(dims, np.int32)
        _check(self._L.gbfwn_make_signed_by_winding_number_dev(self._h, _p(d), _p(_xf12(xf)), beta, threshold,
                                                               ctypes.c_void_p(d_values_ptr), _stream(stream)))

    def calcFromVector_dev(self, d_pts_ptr: int, n: int, d_out_ptr: int, beta: float = 2.0, skipFace: int = -1,
                           stream=None):
        _check(self._L.gbfwn_from_vector_dev(self._h, ctypes.c_void_p(d_pts_ptr), n, beta, skipFace,
                                             ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcWithDistances_dev(self, d_pts_ptr: int, n: int, d_out_ptr: int, options=None, stream=None):
        o = (options or DistanceToMeshOptions())._c()
        _check(self._L.gbfwn_vector_with_distances_dev(self._h, ctypes.c_void_p(d_pts_ptr), n, ctypes.byref(o),
                                                       ctypes.c_void_p(d_out_ptr), _stream(stream)))

    def calcSelfIntersections_dev(self, d_bits_ptr: int, d_wn_ptr: int = 0, beta: float = 2.0, stream=None):
        """d_bits: ceil(faces / 64) 64-bit words; d_wn (optional): one float per face."""
        _check(self._L.gbfwn_self_intersections_dev(self._h, beta, ctypes.c_void_p(d_bits_ptr),
                                                    ctypes.c_void_p(d_wn_ptr or None), _stream(stream)))


# MR::MeshProjectionResult (MRMesh/MRMeshProject.h:17-31) as returned per point by findProjections:
# proj = PointOnFace {face, point}, mtp = MeshTriPoint {e, bary a, b} (e = -1: the caller's topology
# gives edgeWithLeft(face)), distSq.
PROJECTION_DTYPE = np.dtype([("face", np.int32), ("point", np.float32, 3), ("edge", np.int32), ("bary", np.float32, 2),
                             ("distSq", np.float32)])
assert PROJECTION_DTYPE.itemsize == 32


class PointsToMeshProjector:
    """GB300 implementation of ``MR::IPointsToMeshProjector`` (MRMesh/MRPointsToMeshProjector.h:11-30;
    the reference's GPU class is MRCuda/MRCudaPointsToMeshProjector.{h,cpp,cu}).

    ``updateMeshData(verts, faces)`` builds (or replaces) the device tree; ``findProjections`` returns
    one ``PROJECTION_DTYPE`` record per point.  Transforms are 12 floats (3x3 rows, then translation)
    or None, with the reference's meaning: ``objXf`` maps the points, ``refXf`` maps the mesh."""

    def __init__(self, device: int = 0, precise: bool = True):
        self.device = device
        self.precise = precise
        self._fwn: Optional[FastWindingNumber] = None

    def updateMeshData(self, verts: Optional[np.ndarray], faces: Optional[np.ndarray] = None):
        if self._fwn is not None:
            self._fwn.close()
            self._fwn = None
        if verts is not None:
            self._fwn = FastWindingNumber(verts, faces, device=self.device, precise=self.precise)

    @classmethod
    def from_mesh(cls, fwn: "FastWindingNumber") -> "PointsToMeshProjector":
        """Shares the tree of an existing FastWindingNumber handle (the caller keeps it alive)."""
        self = cls(precise=True)
        self._fwn = fwn
        return self

    def findProjections(self, points: np.ndarray, objXf=None, refXf=None, upDistLimitSq: float = FLT_MAX,
                        loDistLimitSq: float = 0.0, cb=None) -> np.ndarray:
        if self._fwn is None:
            raise FwnError(INVALID, "findProjections: no mesh (call updateMeshData first)")
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.empty(len(pts), PROJECTION_DTYPE)
        ox = None if objXf is None else _xf12(objXf)
        rx = None if refXf is None else _xf12(refXf)
        c, _keep = _progress(cb)
        L = self._fwn._L
        _check(L.gbfwn_find_projections(self._fwn.handle, _p(pts), len(pts), _p(ox), _p(rx), upDistLimitSq, loDistLimitSq,
                                        _p(out), c, None))
        return out

    def findProjections_dev(self, d_pts_ptr: int, n: int, d_out_ptr: int, objXf=None, refXf=None,
                            upDistLimitSq: float = FLT_MAX, loDistLimitSq: float = 0.0, stream=None):
        """Device pointers: n x 3 floats in, n x 32-byte records out (16-byte aligned)."""
        ox = None if objXf is None else _xf12(objXf)
        rx = None if refXf is None else _xf12(refXf)
        _check(self._fwn._L.gbfwn_find_projections_dev(self._fwn.handle, ctypes.c_void_p(d_pts_ptr), n, _p(ox), _p(rx),
                                                        upDistLimitSq, loDistLimitSq, ctypes.c_void_p(d_out_ptr),
                                                        _stream(stream)))

    def projectionsHeapBytes(self, numProjections: int) -> int:
        return int(lib().gbfwn_projections_heap_bytes(numProjections))



# ------------------------------------------------------------------ marching cubes (the grid's consumer)
@dataclass
class MarchingCubesParams:
    """MR::MarchingCubesParams (MRVoxels/MRMarchingCubes.h:18-61) for the default linear positioner;
    ``voxelSize`` is the volume's (SimpleVolume::voxelSize), ``outVoxelPerFaceMap`` asks for the
    face -> voxel map."""
    origin: tuple = (0.0, 0.0, 0.0)
    voxelSize: tuple = (1.0, 1.0, 1.0)
    iso: float = 0.0
    lessInside: bool = False
    maxVertices: int = 2**31 - 1
    outVoxelPerFaceMap: bool = False

    def _c(self) -> _McParams:
        c = _McParams()
        for k in range(3):
            c.origin[k] = float(self.origin[k])
            c.voxelSize[k] = float(self.voxelSize[k])
        c.iso = float(self.iso)
        c.lessInside = int(bool(self.lessInside))
        c.maxVertices = int(self.maxVertices)
        c.wantFaceMap = int(bool(self.outVoxelPerFaceMap))
        return c


class TriMesh:
    """A mesh produced on the device (MR::TriMesh: points + triangles, plus the optional
    face -> voxel map).  ``points`` / ``tris`` / ``faceMap`` copy it to host arrays; ``device_ptrs``
    gives the device arrays, valid while this object lives."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle
        self._L = lib()
        npt, ntr = _i64(), _i64()
        _check(self._L.gbfwn_trimesh_sizes(self._h, ctypes.byref(npt), ctypes.byref(ntr)))
        self.numPoints, self.numTris = int(npt.value), int(ntr.value)
        self._host = None

    def _copy(self):
        if self._host is None:
            pts = np.empty((self.numPoints, 3), np.float32)
            tris = np.empty((self.numTris, 3), np.int32)
            dp, dt, df = _vp(), _vp(), _vp()
            _check(self._L.gbfwn_trimesh_device(self._h, ctypes.byref(dp), ctypes.byref(dt), ctypes.byref(df)))
            fmap = np.empty(self.numTris, np.int32) if df.value else None
            _check(self._L.gbfwn_trimesh_copy(self._h, _p(pts), _p(tris), _p(fmap)))
            self._host = (pts, tris, fmap)
        return self._host

    @property
    def points(self) -> np.ndarray:
        return self._copy()[0]

    @property
    def tris(self) -> np.ndarray:
        return self._copy()[1]

    @property
    def faceMap(self) -> Optional[np.ndarray]:
        return self._copy()[2]

    def device_ptrs(self) -> tuple:
        dp, dt, df = _vp(), _vp(), _vp()
        _check(self._L.gbfwn_trimesh_device(self._h, ctypes.byref(dp), ctypes.byref(dt), ctypes.byref(df)))
        return dp.value, dt.value, df.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gbfwn_trimesh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _parts(partStarts):
    if partStarts is None:
        return None, 0
    a = np.ascontiguousarray(partStarts, np.int32)
    return a, len(a)


def marchingCubes(volume: np.ndarray, params: Optional[MarchingCubesParams] = None, partStarts=None, device: int = 0,
                  cb: Optional[Callable[[float], bool]] = None) -> TriMesh:
    """``MR::marchingCubesAsTriMesh(SimpleVolume, params)`` (MRVoxels/MRMarchingCubes.h:66) on the GPU.
    ``volume``: (nz, ny, nx) float32, x fastest.  ``partStarts``: first layers of the overlapping
    parts of an equivalent MarchingCubesByParts sequence (only the rounding of z changes)."""
    v = np.ascontiguousarray(volume, np.float32)
    if v.ndim != 3:
        raise ValueError("volume must be (nz, ny, nx)")
    dims = np.array([v.shape[2], v.shape[1], v.shape[0]], np.int32)
    prm = (params or MarchingCubesParams())._c()
    ps, nps = _parts(partStarts)
    fn, _keep = _progress(cb)
    h = ctypes.c_void_p()
    _check(lib().gbfwn_marching_cubes(_p(v), _p(dims), ctypes.byref(prm), _p(ps), nps, device, ctypes.byref(h), fn, None))
    return TriMesh(h)


def marchingCubes_dev(d_volume_ptr: int, dims, params: Optional[MarchingCubesParams] = None, partStarts=None,
                      device: int = 0, stream=None) -> TriMesh:
    """The same on a device volume of dims = (nx, ny, nz) floats (x fastest)."""
    d = np.asarray(dims, np.int32)
    prm = (params or MarchingCubesParams())._c()
    ps, nps = _parts(partStarts)
    h = ctypes.c_void_p()
    st = ctypes.c_void_p(None if stream is None else int(stream))
    _check(lib().gbfwn_marching_cubes_dev(ctypes.c_void_p(d_volume_ptr), _p(d), ctypes.byref(prm), _p(ps), nps, device,
                                          ctypes.byref(h), st))
    return TriMesh(h)


class MarchingCubesByParts:
    """``MR::MarchingCubesByParts`` (MRVoxels/MRMarchingCubes.h:96-122): ``addPart`` volumes of whole
    XY layers starting at ``nextZ()`` (the previous part's last layer repeated), then ``finalize``."""

    def __init__(self, dims, params: Optional[MarchingCubesParams] = None, device: int = 0):
        self._L = lib()
        d = np.asarray(dims, np.int32)
        prm = (params or MarchingCubesParams())._c()
        self._h = ctypes.c_void_p()
        _check(self._L.gbfwn_mc_parts_create(_p(d), ctypes.byref(prm), device, ctypes.byref(self._h)))

    def nextZ(self) -> int:
        return int(self._L.gbfwn_mc_parts_next_z(self._h))

    def addPart(self, part: np.ndarray):
        v = np.ascontiguousarray(part, np.float32)
        d = np.array([v.shape[2], v.shape[1], v.shape[0]], np.int32)
        _check(self._L.gbfwn_mc_parts_add(self._h, _p(v), _p(d)))

    def addPart_dev(self, d_part_ptr: int, dims, stream=None):
        d = np.asarray(dims, np.int32)
        st = ctypes.c_void_p(None if stream is None else int(stream))
        _check(self._L.gbfwn_mc_parts_add_dev(self._h, ctypes.c_void_p(d_part_ptr), _p(d), st))

    def finalize(self) -> TriMesh:
        h = ctypes.c_void_p()
        _check(self._L.gbfwn_mc_parts_finalize(self._h, ctypes.byref(h)))
        return TriMesh(h)

    def __del__(self):
        try:
            if self._h.value:
                self._L.gbfwn_mc_parts_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass


def calcOriginAndDimensions(box_min, box_max, voxelSize: float):
    """MR::calcOriginAndDimensions (MRVoxels/MRCalcDims.h:18-27): origin = box.min - 2 voxels,
    dims = int((box.max + 2 voxels - origin) / voxelSize) + 1, in float like the reference."""
    vs = np.float32(voxelSize)
    exp = np.float32(2) * vs
    lo = np.asarray(box_min, np.float32)
    hi = np.asarray(box_max, np.float32)
    origin = (lo - exp).astype(np.float32)
    dims = (((hi + exp).astype(np.float32) - origin).astype(np.float32) / vs).astype(np.float32).astype(np.int32) + 1
    return origin, dims


def memory_estimates(nv: int, nt: int, dims=None, npts: int = 0) -> dict:
    L = lib()
    d = np.asarray(dims if dims is not None else (0, 0, 0), np.int32)
    return {"mesh": int(L.gbfwn_mesh_memory(nv, nt)), "from_grid": int(L.gbfwn_from_grid_memory(nv, nt, _p(d))),
            "from_vector": int(L.gbfwn_from_vector_memory(nv, nt, npts)),
            "self_intersections": int(L.gbfwn_self_intersections_memory(nv, nt))}


class Surrogate:
    """Per-mesh signed-distance network used to cull bricks outside a distance band
    (gbfwn_surrogate_* in include/gbfwn.h)."""

    def __init__(self, handle: ctypes.c_void_p, stats: Optional[dict] = None):
        self._h = handle
        self._L = lib()
        self.stats = stats or {}

    @classmethod
    def train(cls, fwn: "FastWindingNumber", dims, xf, band: float, **kw) -> "Surrogate":
        L = lib()
        o = _SurrogateOpts()
        L.gbfwn_surrogate_default_opts(ctypes.byref(o))
        o.band = band
        for k, v in kw.items():
            setattr(o, k, v)
        h = ctypes.c_void_p()
        st = _SurrogateStats()
        d = np.asarray(dims, np.int32)
        _check(L.gbfwn_surrogate_train(fwn.handle, _p(d), _p(_xf12(xf)), ctypes.byref(o), ctypes.byref(h), ctypes.byref(st)))
        return cls(h, {f: getattr(st, f) for f, _ in _SurrogateStats._fields_})

    @classmethod
    def create(cls, params: np.ndarray, meta: np.ndarray, device: int = 0) -> "Surrogate":
        p = np.ascontiguousarray(params, np.float32)
        m = np.ascontiguousarray(meta, np.float32)
        h = ctypes.c_void_p()
        _check(lib().gbfwn_surrogate_create(device, _p(p), _p(m), ctypes.byref(h)))
        return cls(h)

    @property
    def handle(self):
        return self._h

    def parameters(self):
        p = np.empty(SURROGATE_PARAMS, np.float32)
        m = np.empty(SURROGATE_META, np.float32)
        _check(self._L.gbfwn_surrogate_get(self._h, _p(p), _p(m)))
        return p, m

    def eval_dev(self, d_pts_ptr: int, n: int, d_out_ptr: int, stream=None):
        _check(self._L.gbfwn_surrogate_eval_dev(self._h, ctypes.c_void_p(d_pts_ptr), n, ctypes.c_void_p(d_out_ptr),
                                                _stream(stream)))

    def gradients_dev(self, d_pts_ptr: int, d_targets_ptr: int, n: int):
        g = np.empty(SURROGATE_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        _check(self._L.gbfwn_surrogate_gradients_dev(self._h, ctypes.c_void_p(d_pts_ptr), ctypes.c_void_p(d_targets_ptr), n,
                                                     _p(g), _p(loss)))
        return g, float(loss[0])

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gbfwn_surrogate_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _autotune_cache_path() -> str:
    return os.environ.get("MESHLIB_GB300_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "meshlib_gb300", "autotune.json"))


def _autotune_cache_lookup(path: str, key: str, names) -> Optional[dict]:
    """The cached record for ``key`` if it names a variant this library still has at the same index;
    None when the file is missing, unreadable or the entry is stale."""
    import json
    try:
        with open(path) as fh:
            rec = json.load(fh).get(key)
        c = int(rec["config"])
        if 0 <= c < len(names) and rec.get("name") == names[c]:
            return rec
    except (OSError, ValueError, TypeError, KeyError, AttributeError):
        pass
    return None


def _autotune_cache_store(path: str, key: str, rec: dict) -> None:
    """Adds ``rec`` under ``key``; the file is replaced atomically, so concurrent writers never leave a
    torn file (the last writer wins)."""
    import json
    import tempfile
    try:
        cache = {}
        try:
            with open(path) as fh:
                cache = json.load(fh)
            if not isinstance(cache, dict):
                cache = {}
        except (OSError, ValueError):
            pass
        cache[key] = rec
        d = os.path.dirname(path) or "."
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".autotune.", dir=d)
        try:
            with os.fdopen(fd, "w") as fh:
                json.dump(cache, fh, indent=1)
            os.replace(tmp, path)
        except BaseException:
            os.unlink(tmp)
            raise
    except OSError:
        pass


class Batch:
    """Many meshes with their own grids in one persistent launch (gbfwn_batch_* in include/gbfwn.h).

    ``items``: sequence of (FastWindingNumber, dims, xf, DistanceToMeshOptions or None, device output
    pointer).  The tuned variant is remembered in a small JSON cache keyed by GPU, batch size and
    triangle / voxel totals (bucketed by powers of two)."""

    def __init__(self, items):
        self._L = lib()
        arr = (_BatchItem * len(items))()
        tris = vox = 0
        for k, (fwn, dims, xf, opts, out_ptr) in enumerate(items):
            it = arr[k]
            it.mesh = fwn.handle.value
            for j in range(3):
                it.dims[j] = int(dims[j])
            x = _xf12(xf)
            for j in range(12):
                it.xf[j] = float(x[j])
            it.opts = (opts or DistanceToMeshOptions())._c()
            it.d_out = int(out_ptr)
            tris += fwn.num_faces()
            vox += int(dims[0]) * int(dims[1]) * int(dims[2])
        self._items = arr
        self._meshes = [it[0] for it in items]  # the batch points into their trees: keep them alive
        self._h = ctypes.c_void_p()
        _check(self._L.gbfwn_batch_create(arr, len(items), ctypes.byref(self._h)))
        self.key = f"n{len(items)}_t{max(tris, 1).bit_length()}_v{max(vox, 1).bit_length()}"

    @staticmethod
    def configs():
        L = lib()
        return [L.gbfwn_batch_config_name(i).decode() for i in range(L.gbfwn_batch_num_configs())]

    def set_config(self, c: int):
        _check(self._L.gbfwn_batch_set_config(self._h, c))

    def autotune(self, use_cache: bool = True) -> dict:
        try:
            import torch
            gpu = torch.cuda.get_device_name()
        except Exception:
            gpu = "gpu"
        key = f"{gpu}|{self.key}"
        path = _autotune_cache_path()
        names = self.configs()
        if use_cache:
            rec = _autotune_cache_lookup(path, key, names)
            if rec is not None:
                self.set_config(int(rec["config"]))
                return dict(rec, cached=True)
        times = (ctypes.c_float * len(names))()
        best = ctypes.c_int32()
        _check(self._L.gbfwn_batch_autotune(self._h, ctypes.byref(best), times))
        rec = {"config": int(best.value), "name": names[best.value], "times_ms": [float(t) for t in times]}
        if use_cache:
            _autotune_cache_store(path, key, rec)
        return dict(rec, cached=False)

    def run_dev(self, stream=None):
        _check(self._L.gbfwn_batch_run_dev(self._h, _stream(stream)))

    def graph_launch(self, stream=None):
        _check(self._L.gbfwn_batch_graph_launch(self._h, _stream(stream)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gbfwn_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
