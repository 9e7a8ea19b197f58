"""Generates tests/golden/mc_reference.npz: outputs of MeshLib's own CPU mesher
(MRVoxels/MRMarchingCubes.cpp, compiled from the reference sources by oracle/ref/build_cpu_ref.py and
called through oracle/mcref.py) on small seeded volumes.

Run on an x86-64 machine with a copy of the reference:
    python tests/golden/make_mc_golden.py [output path, default tests/golden/mc_reference.npz]

Every case stores its input volume and parameters beside the reference's outputs, so the tests need
neither the generator nor the reference:
  <name>/vol        float32 (nz, ny, nx), x fastest
  <name>/params     float64 [origin xyz, voxel size xyz, iso, lessInside, maxVertices, layersPerBlock]
  <name>/parts      int32 first layer of each part (MarchingCubesByParts), empty = whole volume
  <name>/points     float32 (n, 3)   \
  <name>/tris       int32 (m, 3)      > the reference's TriMesh and face -> voxel map
  <name>/faceMap    int32 (m,)       /
  <name>/error      the reference's error message (empty when it returned a mesh)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "mc_reference.npz")


def _noisy_sphere(shape=(20, 17, 23), seed=0):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    d = np.sqrt((x - 11.2) ** 2 + (y - 8.1) ** 2 + (z - 9.7) ** 2) - 6.3 + 0.3 * rng.standard_normal(x.shape)
    return d.astype(np.float32)


def _sphere(n, r):
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pos = np.stack([x, y, z], -1).astype(np.float32)
    return (np.sqrt(((np.float32(n // 2) - pos) ** 2).sum(-1, dtype=np.float32)) - np.float32(r)).astype(np.float32)


def cases():
    """(name, vol, dict(origin, voxel_size, iso, less_inside, part_starts, max_vertices, layers_per_block))"""
    out = []
    # the reference's own test input (MRTest/MRMarchingCubesTests.cpp): a 10^3 occupancy sphere, iso 0.5
    z, y, x = np.meshgrid(np.arange(10), np.arange(10), np.arange(10), indexing="ij")
    occ = ((x - 4.5) ** 2 + (y - 4.5) ** 2 + (z - 4.5) ** 2 < 16).astype(np.float32)
    out.append(("reference_test_sphere", occ, dict(iso=0.5)))
    ns = _noisy_sphere()
    geo = dict(origin=(0.1, -0.2, 0.3), voxel_size=(0.5, 0.7, 0.9))
    out.append(("distance_volume", ns, dict(geo, iso=0.0, less_inside=True)))
    out.append(("dense_volume", ns, dict(geo, iso=0.5, less_inside=False)))
    out.append(("blocks_of_3_layers", ns, dict(geo, iso=0.0, less_inside=True, layers_per_block=3)))
    out.append(("three_parts", ns, dict(geo, iso=0.0, less_inside=True, part_starts=[0, 6, 13])))
    out.append(("two_parts_blocks_of_2", ns, dict(geo, iso=0.25, less_inside=True, part_starts=[0, 5], layers_per_block=2)))
    rng = np.random.default_rng(9)
    nan = rng.normal(size=(16, 15, 17)).astype(np.float32)
    nan[rng.random(nan.shape) < 0.15] = np.nan
    nan[6:8] = np.nan
    nan[:, 5, :] = np.nan
    out.append(("nan_voxels", nan, dict(origin=(1, 2, 3), voxel_size=(0.5, 0.5, 0.25), iso=-0.1)))
    for shape in ((2, 2, 2), (3, 5, 7), (9, 8, 17)):
        r = np.random.default_rng(sum(shape)).normal(size=shape).astype(np.float32)
        out.append((f"random_{shape[0]}x{shape[1]}x{shape[2]}", r,
                    dict(origin=(0.25, -3.0, 1.5), voxel_size=(0.3, 0.7, 0.11), iso=0.2)))
    pm = np.where(np.random.default_rng(5).random((14, 14, 14)) < 0.5, -1.0, 1.0).astype(np.float32)  # all 254 crossing cubes
    out.append(("every_configuration", pm, dict(iso=0.0, less_inside=True)))
    sp = _sphere(31, 12.0)
    out.append(("two_layer_parts", sp, dict(voxel_size=(0.02,) * 3, iso=0.0, less_inside=True,
                                            part_starts=list(range(30)))))
    out.append(("uneven_parts", sp, dict(voxel_size=(0.02,) * 3, iso=0.0, less_inside=True,
                                         part_starts=[0, 7, 15, 16, 25])))
    small = np.random.default_rng(1).normal(size=(6, 5, 5)).astype(np.float32)
    out.append(("one_layer", small[:1], dict()))
    out.append(("part_of_one_layer", small, dict(part_starts=[0, 2, 5])))
    out.append(("flat_xy", np.random.default_rng(3).normal(size=(4, 1, 6)).astype(np.float32), dict()))
    out.append(("empty_volume", np.zeros((0, 4, 4), np.float32), dict()))
    out.append(("no_crossing_zero_limit", np.ones((3, 3, 3), np.float32), dict(max_vertices=0)))
    out.append(("vertex_limit_zero", small, dict(max_vertices=0)))
    out.append(("vertex_limit_exact", small, dict(max_vertices=193)))  # the mesh of `small` has 193 vertices
    out.append(("vertex_limit_one_short", small, dict(max_vertices=192)))
    return out


def main(path=OUT):
    import oracle.mcref as R
    from oracle.ref import build_cpu_ref
    if not build_cpu_ref.build(targets=("libmcref.so",)):
        raise SystemExit("the reference mesher could not be built here (no copy of the reference)")
    arrays = {}
    names = []
    for name, vol, kw in cases():
        p = dict(origin=(0.0, 0.0, 0.0), voxel_size=(1.0, 1.0, 1.0), iso=0.0, less_inside=False, part_starts=None,
                 max_vertices=2**31 - 1, layers_per_block=0)
        p.update(kw)
        try:
            pts, tris, fmap = R.marching_cubes(vol, **p)
            err = ""
        except R.McRefError as e:
            pts, tris, fmap, err = np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32), np.zeros(0, np.int32), str(e)
        arrays[f"{name}/vol"] = vol
        arrays[f"{name}/params"] = np.array(list(p["origin"]) + list(p["voxel_size"]) + [
            p["iso"], float(p["less_inside"]), float(p["max_vertices"]), float(p["layers_per_block"])], np.float64)
        arrays[f"{name}/parts"] = np.array(p["part_starts"] or [], np.int32)
        arrays[f"{name}/points"] = pts
        arrays[f"{name}/tris"] = tris
        arrays[f"{name}/faceMap"] = fmap
        arrays[f"{name}/error"] = np.array(err)
        names.append(name)
        print(f"{name:28s} {str(vol.shape):16s} points {len(pts):6d} tris {len(tris):6d} {err}")
    arrays["cases"] = np.array(names)
    np.savez_compressed(path, **arrays)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(*sys.argv[1:])
