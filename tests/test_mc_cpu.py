"""Marching-cubes oracle (oracle/mc_oracle.cpp) against the reference's own mesher tests, and the
table invariants; host-side helpers of the mesher front-end.  No GPU needed.

Reference tests mirrored:
  source/MRTest/MRMarchingCubesTests.cpp:9-50        sphere indicator volume, iso 0.5: a non-empty mesh
  source/MRTest/MRVolumeToMeshByPartsTests.cpp:16-160 sphere distance volume (101^3, radius 50 voxels of
                                                     0.01): mesh volume within 0.001 of 4/3 pi r^3, also
                                                     when the volume arrives in 2-layer parts
"""
import numpy as np
import pytest

import oracle as O

CORNER_BIT = [0, 1, 3, 2, 4, 5, 7, 6]
EDGE_CORNER = [0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2]
EDGE_DIR = [0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2]


def mesh_volume(p, t):
    a, b, c = (p[t[:, k]].astype(np.float64) for k in range(3))
    return np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6


def closed_oriented(t):
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    fwd = set(map(tuple, e.tolist()))
    return len(fwd) == len(e) and all((b, a) in fwd for a, b in e.tolist())


def sphere_volume(n=101, r=50.0):
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pos = np.stack([x, y, z], -1).astype(np.float32)
    return (np.sqrt(((np.float32(n // 2) - pos) ** 2).sum(-1, dtype=np.float32)) - np.float32(r)).astype(np.float32)


def test_table_edges_cross_the_surface():
    """Every edge of every plan joins an inside corner to an outside one, and the plan count is the
    classic one (no triangles for the empty and full cubes)."""
    for config in range(256):
        plan = O.mc_plan(config)
        assert len(plan) % 3 == 0 and len(plan) <= 15
        inside = [bool(config >> CORNER_BIT[i] & 1) for i in range(8)]
        for ch in plan:
            e = int(ch, 16)
            c0 = EDGE_CORNER[e]
            c1 = c0 | (1 << EDGE_DIR[e])
            assert inside[c0] != inside[c1], (config, plan, e)
    assert O.mc_plan(0) == "" and O.mc_plan(255) == ""


def test_sphere_indicator_mesh():
    z, y, x = np.meshgrid(np.arange(10), np.arange(10), np.arange(10), indexing="ij")
    vol = ((x - 4.5) ** 2 + (y - 4.5) ** 2 + (z - 4.5) ** 2 < 16).astype(np.float32)
    p, t, f = O.marching_cubes(vol, iso=0.5)
    assert len(t) > 0 and closed_oriented(t)
    assert (t >= 0).all() and (t < len(p)).all()


def test_sphere_distance_volume_whole_and_by_parts():
    vol = sphere_volume()
    expected = 4 * np.pi * 0.5 ** 3 / 3
    p, t, f = O.marching_cubes(vol, voxel_size=(0.01,) * 3, iso=0.0, less_inside=True)
    assert abs(mesh_volume(p, t) - expected) < 1e-3
    assert closed_oriented(t)
    p2, t2, f2 = O.marching_cubes(vol, voxel_size=(0.01,) * 3, iso=0.0, less_inside=True, part_starts=np.arange(100))
    assert abs(mesh_volume(p2, t2) - expected) < 1e-3
    # parts only change the rounding of z (relative to each part's first layer)
    assert np.array_equal(t, t2) and np.array_equal(f, f2)
    assert np.array_equal(p[:, :2], p2[:, :2])
    assert np.abs(p[:, 2] - p2[:, 2]).max() <= 2 * np.spacing(np.float32(1.0))
    # lessInside flips the orientation only
    p3, t3, _ = O.marching_cubes(vol, voxel_size=(0.01,) * 3, iso=0.0, less_inside=False)
    assert np.array_equal(p3, p) and np.array_equal(t3, t[:, [0, 2, 1]])


def test_vertices_on_cell_edges_with_nans():
    """With NaN voxels: every triangle's vertices lie on edges of the cell faceMap names, and no
    vertex sits on an edge with a NaN end."""
    rng = np.random.default_rng(3)
    vol = rng.normal(size=(12, 11, 13)).astype(np.float32)
    vol[rng.random(vol.shape) < 0.1] = np.nan
    vol[5] = np.nan
    p, t, f = O.marching_cubes(vol, origin=(0.5, -1.0, 2.0), voxel_size=(0.5, 0.25, 2.0), iso=0.1)
    assert len(t) > 0
    nz, ny, nx = vol.shape
    vs = np.array([0.5, 0.25, 2.0], np.float32)
    org = np.array([0.5, -1.0, 2.0], np.float32)
    cx, cy, cz = f % nx, (f // nx) % ny, f // (nx * ny)
    lo = org + (np.stack([cx, cy, cz], 1) + 0.5) * vs
    for k in range(3):
        q = p[t[:, k]]
        assert ((q >= lo - 1e-5) & (q <= lo + vs + 1e-5)).all()
    assert not np.isnan(p).any()


def test_errors_and_empty():
    vol = np.zeros((1, 4, 4), np.float32)
    with pytest.raises(O.McError, match="at least two Z slices"):
        O.marching_cubes(vol)
    vol = np.random.default_rng(0).normal(size=(6, 5, 5)).astype(np.float32)
    with pytest.raises(O.McError, match="at least two Z slices"):
        O.marching_cubes(vol, part_starts=[0, 2, 5])
    with pytest.raises(O.McError, match="exceeds whole volume"):
        O.marching_cubes(vol, part_starts=[0, 7])
    p, t, f = O.marching_cubes(vol)
    with pytest.raises(O.McError, match="Vertices number limit exceeded"):
        O.marching_cubes(vol, max_vertices=len(p) - 1)
    assert len(O.marching_cubes(vol, max_vertices=len(p))[0]) == len(p)
    p, t, f = O.marching_cubes(np.zeros((0, 3, 3), np.float32))
    assert len(p) == 0 and len(t) == 0


def test_calc_origin_and_dimensions():
    import meshlib_gb300 as M
    o, d = M.calcOriginAndDimensions([-1, -0.5, 0], [1, 0.5, 2], 0.1)
    assert np.allclose(o, [-1.2, -0.7, -0.2]) and o.dtype == np.float32
    assert d.tolist() == [25, 15, 25]


def test_mesher_memory_estimate():
    """The mesher's memory estimator (pure host arithmetic): about 3 bytes per voxel of work arrays,
    plus the output for the expected triangles; 0 for an empty volume."""
    import meshlib_gb300 as M
    L = M.lib()
    dims = np.array([512, 512, 512], np.int32)
    w = L.gbfwn_marching_cubes_memory(dims.ctypes.data, 0)
    assert 3 * 512 ** 3 <= w <= 3.1 * 512 ** 3
    assert L.gbfwn_marching_cubes_memory(dims.ctypes.data, 1_000_000) == w + 30 * 1_000_000
    assert L.gbfwn_marching_cubes_memory(np.array([0, 4, 4], np.int32).ctypes.data, 10) == 0


def test_vertex_limit_zero_like_reference():
    """maxVertices = 0: any vertex exceeds the limit (VolumeMesher::finalize), an empty mesh does not."""
    vol = np.random.default_rng(2).normal(size=(4, 4, 4)).astype(np.float32)
    with pytest.raises(O.McError, match="Vertices number limit exceeded"):
        O.marching_cubes(vol, max_vertices=0)
    assert len(O.marching_cubes(np.ones((3, 3, 3), np.float32), max_vertices=0)[0]) == 0


def _one_cell(vals):
    """2x2x2 volume from corner values indexed x + 2y + 4z."""
    v = np.empty((2, 2, 2), np.float32)
    for i, val in enumerate(vals):
        v[i >> 2, (i >> 1) & 1, i & 1] = val
    return v


def test_hand_worked_single_cell():
    """Corner 0 below iso, the rest above: configuration 1 (plan edges 0, 8, 3), vertices on corner
    0's +X, +Y, +Z edges in that order at the midpoints (ratio 0.5), one triangle (X, Z, Y); lessInside
    reverses it (MRMarchingCubes.cpp:610-646, 1030-1045)."""
    vol = _one_cell([-1, 1, 1, 1, 1, 1, 1, 1])
    p, t, f = O.marching_cubes(vol, iso=0.0)
    assert p.tolist() == [[1.0, 0.5, 0.5], [0.5, 1.0, 0.5], [0.5, 0.5, 1.0]]
    assert t.tolist() == [[0, 2, 1]] and f.tolist() == [0]
    p2, t2, _ = O.marching_cubes(vol, iso=0.0, less_inside=True)
    assert np.array_equal(p2, p) and t2.tolist() == [[0, 1, 2]]
    # iso between: ratio (iso - v0) / (v1 - v0) from the lower-id end of each edge
    p3, _, _ = O.marching_cubes(_one_cell([-1, 3, 3, 3, 3, 3, 3, 3]), iso=0.0)
    assert np.allclose(p3, [[0.75, 0.5, 0.5], [0.5, 0.75, 0.5], [0.5, 0.5, 0.75]])


def test_hand_worked_nan_corner():
    """Corner 0 NaN takes corner 1's side (first valid neighbour: x, then y, z, ...), giving
    configuration 3; its plan needs a vertex on corner 0's +Z edge, which a NaN end cannot have, so the
    cell emits nothing (MRMarchingCubes.cpp:913-1032) -- while corner 1's +Y and +Z vertices exist."""
    vol = _one_cell([np.nan, -1, 1, 1, 1, 1, 1, 1])
    p, t, f = O.marching_cubes(vol, iso=0.0)
    assert p.tolist() == [[1.5, 1.0, 0.5], [1.5, 0.5, 1.0]]
    assert len(t) == 0
    # with corner 0 valid and below iso the same cell is configuration 3 and meshes fully
    p2, t2, _ = O.marching_cubes(_one_cell([-1, -1, 1, 1, 1, 1, 1, 1]), iso=0.0)
    assert len(t2) == 2 and O.mc_plan(3) == "183981"
