"""The reference's own GPU kernels (MRCuda/MRCudaFastWindingNumber.cu), run on the same GPU.

TEST / BENCH INFRASTRUCTURE ONLY: the parity tests compare the library with this path, and the
benchmark times it as the "plain MRCuda" line.  The product never imports it.

The device code is built from the reference sources by oracle/ref/build_ref.py into oracle/_ref/
(cubin, plus PTX as a fallback) and launched by oracle/mrcuda_runner.cpp through the driver API,
one thread per query and 32 threads per block, as the reference's launchers do
(MRCudaFastWindingNumber.cu:245-274).  The mesh data are what the reference's host class uploads
(MRCudaFastWindingNumber.cpp:42-80): the CPU-built AABB tree and FP32 dipoles (here from the
oracle, whose tree and dipoles are the reference's), the vertex array and the triangle array.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "libmrcuda_runner.so")
_CUBIN = os.path.join(_HERE, "_ref", "mrcuda_fwn.cubin")
_PTX = os.path.join(_HERE, "_ref", "mrcuda_fwn.ptx")
_PCUBIN = os.path.join(_HERE, "_ref", "mrcuda_proj.cubin")
_PPTX = os.path.join(_HERE, "_ref", "mrcuda_proj.ptx")
_lib = None


def _cuda_include() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH") or "/usr/local/cuda"
    return os.path.join(home, "include")


def build_runner(force: bool = False) -> str:
    src = os.path.join(_HERE, "mrcuda_runner.cpp")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + _cuda_include(), "-o", _SO, src,
                               "-ldl"])
    return _SO


def kernels_present() -> bool:
    """True when the reference kernels were built (they need the reference sources at build time)."""
    return os.path.exists(_CUBIN) or os.path.exists(_PTX)


def _load(device: int):
    global _lib
    if _lib is None:
        build_runner()
        L = ctypes.CDLL(_SO)
        vp, fp, ip, u64 = ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_uint64
        L.mrc_last_error.restype = ctypes.c_char_p
        L.mrc_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ip]
        L.mrc_signed_distance.argtypes = [vp, vp, ip, vp, vp, vp, vp, vp, fp, fp, ip, fp, fp, u64, u64, vp]
        L.mrc_from_grid.argtypes = [vp, vp, ip, vp, vp, vp, vp, vp, fp, u64, u64, vp]
        L.mrc_from_vector.argtypes = [vp, vp, vp, vp, vp, vp, fp, ip, u64, vp]
        L.mrc_from_mesh.argtypes = [vp, vp, vp, vp, vp, fp, u64, u64, vp]
        L.mrc_load_projector.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.mrc_project.argtypes = [vp, vp, vp, vp, vp, vp, vp, fp, fp, u64, vp]
        _lib = L
    r = _lib.mrc_load(_CUBIN.encode() if os.path.exists(_CUBIN) else b"", _PTX.encode() if os.path.exists(_PTX) else b"",
                      device)
    if r:
        raise RuntimeError("reference kernels: " + _lib.mrc_last_error().decode())
    return _lib


def _fold(objXf, refXf, is_rigid):
    """(point map, tree map) as MRCudaPointsToMeshProjector.cpp:75-102 derives them, in float64 -> float32
    (the reference composes in float; the tests compare with tolerances)."""
    def m(x):
        x = np.asarray(x, np.float64).reshape(12)
        A = np.eye(4)
        A[:3, :3] = x[:9].reshape(3, 3)
        A[:3, 3] = x[9:]
        return A

    def back(A):
        return np.concatenate([A[:3, :3].reshape(-1), A[:3, 3]]).astype(np.float32)

    if refXf is not None and not is_rigid(refXf):
        return (None if objXf is None else np.asarray(objXf, np.float32)), np.asarray(refXf, np.float32)
    if refXf is None:
        return (None if objXf is None else np.asarray(objXf, np.float32)), None
    A = np.linalg.inv(m(refXf))
    if objXf is not None:
        A = A @ m(objXf)
    return back(A), None


def _identity(xf) -> bool:
    return bool(np.array_equal(np.asarray(xf, np.float32), np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float32)))


class RefKernels:
    """Device copies of one mesh in the reference layouts plus the four reference kernels."""

    def __init__(self, verts, faces, nodes: np.ndarray, dipoles: np.ndarray, device: int = 0):
        import torch

        if not kernels_present():
            raise RuntimeError("reference kernels not built (oracle/ref/build_ref.py needs the reference sources)")
        self.torch = torch
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        torch.zeros(1, device=self.dev)  # make the primary context current on this thread
        self.L = _load(device)
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt).reshape(-1)).to(self.dev)
        self.points = t(verts, np.float32)
        self.faces = t(faces, np.int32)
        self.nodes = torch.from_numpy(np.ascontiguousarray(nodes).view(np.uint8).reshape(-1)).to(self.dev)
        self.dipoles = t(dipoles, np.float32)
        assert self.nodes.numel() == 32 * len(nodes) and self.dipoles.numel() == 8 * len(dipoles)

    def _p(self, x):
        return ctypes.c_void_p(x.data_ptr())

    def _check(self, r):
        if r:
            raise RuntimeError("reference kernel launch: " + self.L.mrc_last_error().decode())

    def signed_distance(self, dims, xf, minDistSq=0.0, maxDistSq=3.4028234663852886e38, nullOutsideMinMax=True,
                        threshold=0.5, beta=2.0, out=None, stream=None):
        """signedDistanceKernel over the whole grid in one chunk (a GB300 holds any grid here)."""
        d = np.asarray(dims, np.int32)
        n = int(np.prod(d.astype(np.int64)))
        out = out if out is not None else self.torch.empty(n, dtype=self.torch.float32, device=self.dev)
        x = np.ascontiguousarray(xf, np.float32)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        self._check(self.L.mrc_signed_distance(d.ctypes.data, x.ctypes.data, int(_identity(x)), self._p(self.dipoles),
                                               self._p(self.nodes), self._p(self.points), self._p(self.faces),
                                               self._p(out), minDistSq, maxDistSq, int(nullOutsideMinMax), threshold,
                                               beta, n, 0, ctypes.c_void_p(s)))
        return out

    # The reference's winding-number kernels add into their output element (processPoint takes
    # resVec[index] by reference, MRCudaFastWindingNumber.cu:30-62 and :135-201) instead of starting
    # from zero, so the output is zero-filled first, as the reference's freshly allocated result
    # buffer is in practice.  (Its chunked host loop reuses that buffer: a second chunk would add onto
    # the first one's values; the single-chunk launches here never reach that.)
    def from_grid(self, dims, xf, beta=2.0, out=None, stream=None):
        d = np.asarray(dims, np.int32)
        n = int(np.prod(d.astype(np.int64)))
        out = out if out is not None else self.torch.empty(n, dtype=self.torch.float32, device=self.dev)
        out.zero_()
        x = np.ascontiguousarray(xf, np.float32)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        self._check(self.L.mrc_from_grid(d.ctypes.data, x.ctypes.data, int(_identity(x)), self._p(self.dipoles),
                                         self._p(self.nodes), self._p(self.points), self._p(self.faces), self._p(out),
                                         beta, n, 0, ctypes.c_void_p(s)))
        return out

    def from_vector(self, pts, beta=2.0, skip_face=-1, stream=None):
        q = pts if hasattr(pts, "data_ptr") else self.torch.from_numpy(np.ascontiguousarray(pts, np.float32).reshape(-1)).to(self.dev)
        n = q.numel() // 3
        out = self.torch.zeros(n, dtype=self.torch.float32, device=self.dev)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        self._check(self.L.mrc_from_vector(self._p(q), self._p(self.dipoles), self._p(self.nodes), self._p(self.points),
                                           self._p(self.faces), self._p(out), beta, skip_face, n, ctypes.c_void_p(s)))
        return out

    def project(self, pts, objXf=None, refXf=None, upDistLimitSq=3.4028234663852886e38, loDistLimitSq=0.0, stream=None,
                out=None):
        """The reference's GPU projector (MRCuda/MRCudaPointsToMeshProjector.cu:6-111) with its host
        class's transform handling (.cpp:75-102): a rigid refXf is folded into the point map, a
        non-rigid one is applied to the tree.  Returns a uint8 tensor of n x 32-byte records
        (face, point xyz, edge = -1, bary a b, distSq)."""
        from . import is_rigid
        if not (os.path.exists(_PCUBIN) or os.path.exists(_PPTX)):
            raise RuntimeError("reference projector kernel not built")
        if self.L.mrc_load_projector(_PCUBIN.encode() if os.path.exists(_PCUBIN) else b"",
                                     _PPTX.encode() if os.path.exists(_PPTX) else b""):
            raise RuntimeError("reference projector: " + self.L.mrc_last_error().decode())
        xf_pt, xf_tree = _fold(objXf, refXf, is_rigid)
        q = pts if hasattr(pts, "data_ptr") else self.torch.from_numpy(np.ascontiguousarray(pts, np.float32).reshape(-1)).to(self.dev)
        n = q.numel() // 3
        out = out if out is not None else self.torch.empty(32 * n, dtype=self.torch.uint8, device=self.dev)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        a = None if xf_pt is None else np.ascontiguousarray(xf_pt, np.float32)
        b = None if xf_tree is None else np.ascontiguousarray(xf_tree, np.float32)
        self._check(self.L.mrc_project(self._p(q), self._p(self.nodes), self._p(self.points), self._p(self.faces), self._p(out),
                                       a.ctypes.data if a is not None else None, b.ctypes.data if b is not None else None,
                                       upDistLimitSq, loDistLimitSq, n, ctypes.c_void_p(s)))
        return out

    def from_mesh(self, beta=2.0, stream=None):
        """Winding number at every face centroid with that face skipped (the self-intersection
        query, MRCudaFastWindingNumber.cpp:129-173); the host then flags wn < 0 or wn > 1."""
        nf = self.faces.numel() // 3
        out = self.torch.zeros(nf, dtype=self.torch.float32, device=self.dev)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        self._check(self.L.mrc_from_mesh(self._p(self.dipoles), self._p(self.nodes), self._p(self.points),
                                         self._p(self.faces), self._p(out), beta, nf, 0, ctypes.c_void_p(s)))
        return out
