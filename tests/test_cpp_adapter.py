"""The header-only C++ adapter (include/gbfwn.hpp) built against the library and run on the GPU;
its results must equal the Python front-end's on the same mesh."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from meshlib_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "adapter_check")
    subprocess.check_call(["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"),
                           "-o", exe, lib, f"-Wl,-rpath,{os.path.dirname(lib)}"])
    return exe


def test_adapter_compiles(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_adapter_matches_python(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout.strip()
    assert out.startswith("OK"), out
    kv = dict(x.split("=") for x in out.split()[1:])
    import meshlib_gb300 as M
    nu, nv = 24, 12
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    u, v = 2 * np.pi * i / nu, 2 * np.pi * j / nv
    verts = np.stack([(1 + 0.3 * np.cos(v)) * np.cos(u), (1 + 0.3 * np.cos(v)) * np.sin(u), 0.3 * np.sin(v)], -1)
    verts = verts.reshape(-1, 3).astype(np.float32)
    a = (i * nv + j).ravel(); b = (((i + 1) % nu) * nv + j).ravel()
    c = (((i + 1) % nu) * nv + (j + 1) % nv).ravel(); d = (i * nv + (j + 1) % nv).ravel()
    tris = np.stack([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], 1).reshape(-1, 3).astype(np.int32)
    g = M.FastWindingNumber(verts, tris)
    xf = np.array([0.18, 0, 0, 0, 0.18, 0, 0, 0, 0.1, -1.4, -1.4, -0.4], np.float32)
    sd = g.calcFromGridWithDistances((16, 16, 8), xf)
    wn = g.calcFromGrid((16, 16, 8), xf)
    assert abs(float(kv["sum_sd"]) - float(sd.astype(np.float64).sum())) < 1e-3
    assert abs(float(kv["sum_wn"]) - float(wn.astype(np.float64).sum())) < 1e-3
    assert int(kv["neg"]) == int((sd < 0).sum())
    assert kv["parts_equal"] == "1"
    assert int(kv["selfint"]) == 0
    assert int(kv["cancel_status"]) == M.CANCELLED
    # projector adapter: closest-point distances equal |signed distance| at the same points
    assert float(kv["proj_max_diff"]) < 1e-5
    # marching-cubes adapter: the same mesh as the Python front-end; by parts and fused give the same
    # triangles (points of parts differ only in the rounding of z)
    assert kv["mc_same"] == "1"
    # knobs: the torus is a closed surface; switching sign reuse off gives the same grid
    assert kv["closed"] == "1" and kv["reuse_same"] == "1"
    prm = M.MarchingCubesParams(origin=tuple(xf[9:12] - 0.5 * xf[[0, 4, 8]]), voxelSize=tuple(xf[[0, 4, 8]]),
                                lessInside=True)
    tm = M.marchingCubes(sd.reshape(8, 16, 16), prm)
    assert int(kv["mc_tris"]) == tm.numTris > 0 and int(kv["mc_points"]) == tm.numPoints
