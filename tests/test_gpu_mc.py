"""Marching cubes on the GPU against the restated reference mesher (oracle/mc_oracle.cpp), bit for
bit: the same points (every float equal), the same triangles in the same order, the same face map.
Covers the reference's cases: NaN voxels (nullOutsideMinMax bands), parts (MarchingCubesByParts),
both orientations, odd sizes, the vertex limit, and the fused distance-grid -> mesh call; and, through
tests/golden/mc_reference.npz, the outputs of MeshLib's own mesher compiled from its sources."""
import os

import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300


def _same(tm, ref):
    p, t, f = ref
    assert tm.numPoints == len(p) and tm.numTris == len(t)
    assert np.array_equal(tm.points.view(np.uint32), p.view(np.uint32))
    assert np.array_equal(tm.tris, t)
    if tm.faceMap is not None:
        assert np.array_equal(tm.faceMap, f)


def _sphere(n=101, r=50.0):
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pos = np.stack([x, y, z], -1).astype(np.float32)
    return (np.sqrt(((np.float32(n // 2) - pos) ** 2).sum(-1, dtype=np.float32)) - np.float32(r)).astype(np.float32)


@pytest.mark.parametrize("less_inside", [False, True])
def test_sphere_vs_oracle(M, less_inside):
    vol = _sphere()
    prm = M.MarchingCubesParams(voxelSize=(0.01,) * 3, iso=0.0, lessInside=less_inside, outVoxelPerFaceMap=True)
    ref = O.marching_cubes(vol, voxel_size=(0.01,) * 3, iso=0.0, less_inside=less_inside)
    _same(M.marchingCubes(vol, prm), ref)


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 5, 7), (17, 16, 33), (40, 37, 48)])
def test_random_fields_odd_sizes(M, shape):
    rng = np.random.default_rng(sum(shape))
    vol = rng.normal(size=shape).astype(np.float32)
    org, vs = (0.25, -3.0, 1.5), (0.3, 0.7, 0.11)
    prm = M.MarchingCubesParams(origin=org, voxelSize=vs, iso=0.2, outVoxelPerFaceMap=True)
    _same(M.marchingCubes(vol, prm), O.marching_cubes(vol, origin=org, voxel_size=vs, iso=0.2))


def test_every_configuration(M):
    """A random +-1 volume meets all 256 cube configurations (checked on the oracle's face map)."""
    rng = np.random.default_rng(5)
    vol = np.where(rng.random((48, 48, 48)) < 0.5, -1.0, 1.0).astype(np.float32)
    ref = O.marching_cubes(vol, iso=0.0, less_inside=True)
    z, y, x = np.unravel_index(ref[2], vol.shape)
    cfg = np.zeros(len(z), np.int64)
    for i, bit in enumerate([0, 1, 3, 2, 4, 5, 7, 6]):
        cfg |= (vol[z + (i >> 2), y + ((i >> 1) & 1), x + (i & 1)] < 0).astype(np.int64) << bit
    assert len(np.unique(cfg)) == 254  # all but the empty and the full cube
    _same(M.marchingCubes(vol, M.MarchingCubesParams(iso=0.0, lessInside=True, outVoxelPerFaceMap=True)), ref)


def test_nan_voxels(M):
    rng = np.random.default_rng(9)
    vol = rng.normal(size=(30, 29, 31)).astype(np.float32)
    vol[rng.random(vol.shape) < 0.15] = np.nan
    vol[10:12] = np.nan
    vol[:, 5, :] = np.nan
    prm = M.MarchingCubesParams(origin=(1, 2, 3), voxelSize=(0.5, 0.5, 0.25), iso=-0.1, outVoxelPerFaceMap=True)
    ref = O.marching_cubes(vol, origin=(1, 2, 3), voxel_size=(0.5, 0.5, 0.25), iso=-0.1)
    assert len(ref[1]) > 0
    _same(M.marchingCubes(vol, prm), ref)
    allnan = np.full((4, 4, 4), np.nan, np.float32)
    tm = M.marchingCubes(allnan, prm)
    assert tm.numPoints == 0 and tm.numTris == 0


def test_parts_and_by_parts_object(M):
    vol = _sphere(61, 25.0)
    prm = M.MarchingCubesParams(voxelSize=(0.02,) * 3, iso=0.0, lessInside=True, outVoxelPerFaceMap=True)
    for starts in (np.arange(60), [0, 7, 30, 31, 50]):
        ref = O.marching_cubes(vol, voxel_size=(0.02,) * 3, iso=0.0, less_inside=True, part_starts=starts)
        _same(M.marchingCubes(vol, prm, partStarts=starts), ref)
    # MarchingCubesByParts: 2-layer parts as in the reference's test, then uneven parts from device memory
    ref = O.marching_cubes(vol, voxel_size=(0.02,) * 3, iso=0.0, less_inside=True, part_starts=np.arange(60))
    mc = M.MarchingCubesByParts((61, 61, 61), prm)
    for z in range(60):
        assert mc.nextZ() == z
        mc.addPart(vol[z:z + 2])
    _same(mc.finalize(), ref)
    import torch
    dv = torch.from_numpy(vol).cuda()
    mc = M.MarchingCubesByParts((61, 61, 61), prm)
    starts = [0, 7, 30, 31, 50]
    for a, b in zip(starts, starts[1:] + [60]):
        mc.addPart_dev(dv[a:b + 1].data_ptr(), (61, 61, b + 1 - a))
    ref = O.marching_cubes(vol, voxel_size=(0.02,) * 3, iso=0.0, less_inside=True, part_starts=starts)
    _same(mc.finalize(), ref)


def test_errors(M):
    vol = np.random.default_rng(1).normal(size=(6, 5, 5)).astype(np.float32)
    with pytest.raises(M.FwnError, match="at least two Z slices"):
        M.marchingCubes(vol[:1])
    with pytest.raises(M.FwnError, match="at least two Z slices"):
        M.marchingCubes(vol, partStarts=[0, 2, 5])
    n = len(O.marching_cubes(vol)[0])
    with pytest.raises(M.FwnError, match="Vertices number limit exceeded"):
        M.marchingCubes(vol, M.MarchingCubesParams(maxVertices=n - 1))
    assert M.marchingCubes(vol, M.MarchingCubesParams(maxVertices=n)).numPoints == n
    with pytest.raises(M.FwnError, match="Vertices number limit exceeded"):
        M.marchingCubes(vol, M.MarchingCubesParams(maxVertices=0))
    assert M.marchingCubes(np.ones((3, 3, 3), np.float32), M.MarchingCubesParams(maxVertices=0)).numPoints == 0
    assert M.marchingCubes(np.zeros((0, 4, 4), np.float32)).numTris == 0
    mc = M.MarchingCubesByParts((5, 5, 6))
    with pytest.raises(M.FwnError, match="XY dimensions"):
        mc.addPart(np.zeros((2, 5, 4), np.float32))
    with pytest.raises(M.FwnError, match="at least two Z slices"):
        mc.addPart(np.zeros((1, 5, 5), np.float32))
    mc.addPart(vol[:3])
    with pytest.raises(M.FwnError, match="exceeds whole volume"):
        mc.addPart(vol[:5])
    with pytest.raises(M.FwnError, match="do not cover"):
        mc.finalize()


@pytest.mark.parametrize("banded", [False, True])
def test_grid_to_mesh_vs_host_pipeline(M, banded):
    """mcOffsetMesh's volume step fused on the device == our distance grid copied to the host and
    meshed by the oracle (the reference's flow), at an offset of 2 voxels."""
    v, f = mg.noisy_torus(seed=1)
    g = M.FastWindingNumber(v, f)
    vsz = 0.02
    off = 2 * vsz
    lo, hi = v.min(0) - off, v.max(0) + off
    origin, dims = M.calcOriginAndDimensions(lo, hi, vsz)
    opts = M.DistanceToMeshOptions()
    if banded:
        opts.minDistSq = max(off - 1.001 * vsz, 0.0) ** 2
        opts.maxDistSq = (off + 1.001 * vsz) ** 2
        opts.nullOutsideMinMax = True
    prm = M.MarchingCubesParams(origin=tuple(origin), voxelSize=(vsz,) * 3, iso=off, lessInside=True,
                                outVoxelPerFaceMap=True)
    tm = g.gridToMesh(dims, origin, vsz, opts, prm)
    basis = np.array([vsz, 0, 0, 0, vsz, 0, 0, 0, vsz, 0, 0, 0], np.float32)
    basis[9:] = (origin + np.float32(0.5) * np.float32(vsz)).astype(np.float32)
    grid = g.calcFromGridWithDistances(dims, basis, opts).reshape(dims[2], dims[1], dims[0])
    ref = O.marching_cubes(grid, origin=origin, voxel_size=(vsz,) * 3, iso=off, less_inside=True)
    assert len(ref[1]) > 1000
    _same(tm, ref)
    if not banded:  # a clean offset surface of a closed mesh is closed
        t = tm.tris
        e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
        assert len(set(map(tuple, e.tolist()))) == len(e)


def test_grid_to_mesh_large(M):
    """256^3 offset grid of the 1.31 M-triangle icosphere: the fused call against the oracle mesher
    on the same device grid."""
    import torch
    v, f = mg.noisy_icosphere(seed=0, level=8)
    g = M.FastWindingNumber(v, f)
    ext = (v.max(0) - v.min(0)).max()
    vsz = float(ext) / 240
    off = 3 * vsz
    origin, dims = M.calcOriginAndDimensions(v.min(0) - off, v.max(0) + off, vsz)
    prm = M.MarchingCubesParams(origin=tuple(origin), voxelSize=(vsz,) * 3, iso=off, lessInside=True)
    tm = g.gridToMesh(dims, origin, vsz, M.DistanceToMeshOptions(), prm)
    basis = np.array([vsz, 0, 0, 0, vsz, 0, 0, 0, vsz, 0, 0, 0], np.float32)
    basis[9:] = (origin + np.float32(0.5) * np.float32(vsz)).astype(np.float32)
    out = torch.empty(int(np.prod(dims)), device="cuda")
    g.calcFromGridWithDistances_dev(dims, basis, out.data_ptr())
    torch.cuda.synchronize()
    grid = out.cpu().numpy().reshape(dims[2], dims[1], dims[0])
    ref = O.marching_cubes(grid, origin=origin, voxel_size=(vsz,) * 3, iso=off, less_inside=True)
    _same(tm, ref)


def test_cancel_and_allocation_failure(M):
    """Progress callbacks cancel (MeshLib's unexpectedOperationCanceled); a failed device allocation
    (host-side injection) is reported as out of memory and leaves the library usable."""
    vol = _sphere(41, 15.0)
    prm = M.MarchingCubesParams(iso=0.0, lessInside=True)
    with pytest.raises(M.FwnError) as ei:
        M.marchingCubes(vol, prm, cb=lambda p: p < 0.2)
    assert ei.value.status == M.CANCELLED
    seen = []
    tm = M.marchingCubes(vol, prm, cb=lambda p: seen.append(p) or True)
    assert tm.numTris > 0 and seen[0] == 0.0 and seen[-1] == 1.0
    M.lib().gbfwn_debug_fail_next_allocs(1)
    with pytest.raises(M.FwnError) as ei:
        M.marchingCubes(vol, prm)
    assert ei.value.status == M.OUT_OF_MEMORY
    again = M.marchingCubes(vol, prm)
    assert np.array_equal(again.tris, tm.tris)
    v, f = mg.noisy_torus(seed=1)
    g = M.FastWindingNumber(v, f)
    origin, dims = M.calcOriginAndDimensions(v.min(0) - 0.05, v.max(0) + 0.05, 0.02)
    with pytest.raises(M.FwnError) as ei:
        g.gridToMesh(dims, origin, 0.02, cb=lambda p: p < 0.5)
    assert ei.value.status == M.CANCELLED
    assert g.gridToMesh(dims, origin, 0.02).numTris > 0


def test_offset_flow_by_parts(M):
    """mcOffsetMesh's own flow (MRVoxels/MROffset.cpp:194-226): the banded distance grid produced by
    parts with one overlapping layer (IFastWindingNumberByParts) feeds MarchingCubesByParts slab by
    slab.  The GPU mesher by parts == the fused call given the same part starts == the oracle."""
    v, f = mg.noisy_torus(seed=4)
    g = M.FastWindingNumber(v, f)
    vsz = 0.02
    off = 2 * vsz
    origin, dims = M.calcOriginAndDimensions(v.min(0) - off, v.max(0) + off, vsz)
    opts = M.DistanceToMeshOptions(minDistSq=max(off - 1.001 * vsz, 0.0) ** 2, maxDistSq=(off + 1.001 * vsz) ** 2,
                                   nullOutsideMinMax=True)
    prm = M.MarchingCubesParams(origin=tuple(origin), voxelSize=(vsz,) * 3, iso=off, lessInside=True,
                                outVoxelPerFaceMap=True)
    basis = np.array([vsz, 0, 0, 0, vsz, 0, 0, 0, vsz, 0, 0, 0], np.float32)
    basis[9:] = (origin + np.float32(0.5) * np.float32(vsz)).astype(np.float32)
    mc = M.MarchingCubesByParts(dims, prm)
    starts = []

    def part(arr, sd, zoff):
        assert zoff == mc.nextZ()
        starts.append(zoff)
        mc.addPart(arr.reshape(sd[2], sd[1], sd[0]))

    g.calcFromGridWithDistancesByParts(part, dims, basis, opts, layerOverlap=1, maxLayersPerSlab=7)
    assert len(starts) > 2
    tm = mc.finalize()
    assert tm.numTris > 1000
    fused = g.gridToMesh(dims, origin, vsz, opts, prm, partStarts=starts)
    _same(fused, (tm.points, tm.tris, tm.faceMap))
    grid = g.calcFromGridWithDistances(dims, basis, opts).reshape(dims[2], dims[1], dims[0])
    _same(tm, O.marching_cubes(grid, origin=origin, voxel_size=(vsz,) * 3, iso=off, less_inside=True,
                               part_starts=starts))


def test_more_than_2_31_voxels(M):
    """1300^3 = 2.2e9 voxels (64-bit voxel and flag indices): a sphere of radius 200 voxels gives a
    closed, consistently oriented genus-0 mesh (V - E + F = 2) whose volume is the ball's within
    1e-3; the face map is refused (32-bit voxel ids), as the reference's VoxelId would overflow."""
    import torch
    n, r = 1300, 200.0
    vol = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
    ax = torch.arange(n, device="cuda", dtype=torch.float32) - (n - 1) / 2
    yy, xx = torch.meshgrid(ax, ax, indexing="ij")
    rxy = yy * yy + xx * xx
    for z0 in range(0, n, 100):
        zz = ax[z0:z0 + 100].view(-1, 1, 1)
        vol[z0:z0 + 100] = torch.sqrt(rxy.unsqueeze(0) + zz * zz) - r
    del yy, xx, rxy
    prm = M.MarchingCubesParams(iso=0.0, lessInside=True)
    tm = M.marchingCubes_dev(vol.data_ptr(), (n, n, n), prm)
    with pytest.raises(M.FwnError, match="32 bits"):
        M.marchingCubes_dev(vol.data_ptr(), (n, n, n), M.MarchingCubesParams(outVoxelPerFaceMap=True))
    del vol
    torch.cuda.empty_cache()
    p, t = tm.points.astype(np.float64), tm.tris.astype(np.int64)
    assert tm.numTris > 500_000 and (t >= 0).all() and (t < len(p)).all()
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    key = e[:, 0] * len(p) + e[:, 1]
    rkey = e[:, 1] * len(p) + e[:, 0]
    ks = np.sort(key)
    assert (np.diff(ks) > 0).all()  # every directed edge once
    assert np.isin(rkey, ks).all()  # and its reverse present: closed and consistently oriented
    assert len(p) - len(e) // 2 + len(t) == 2
    a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    volume = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6
    assert abs(volume / (4 / 3 * np.pi * r ** 3) - 1) < 1e-3


def test_release_cached_memory(M):
    """Handles created one per call reuse the library's pooled staging memory; releasing the cache
    (pool and mesher workspace) leaves every call working and the results unchanged."""
    v, f = mg.noisy_torus(seed=2)
    dims, xf = mg.grid_for(v, 24)
    first = M.FastWindingNumber(v, f).calcFromGridWithDistances(dims, xf)
    tm = M.marchingCubes(first.reshape(dims[2], dims[1], dims[0]), M.MarchingCubesParams(lessInside=True))
    assert M.lib().gbfwn_release_cached_memory(0) == M.OK
    again = M.FastWindingNumber(v, f).calcFromGridWithDistances(dims, xf)
    assert np.array_equal(first, again)
    tm2 = M.marchingCubes(again.reshape(dims[2], dims[1], dims[0]), M.MarchingCubesParams(lessInside=True))
    assert np.array_equal(tm.tris, tm2.tris)


@pytest.mark.parametrize("vals", [[-1, 1, 1, 1, 1, 1, 1, 1], [np.nan, -1, 1, 1, 1, 1, 1, 1], [-1, -1, 1, 1, 1, 1, 1, 1],
                                  [1, -1, -1, 1, -1, 1, 1, -1], [np.nan, np.nan, -1, 1, 1, np.nan, 1, -1]])
def test_single_cells(M, vals):
    """The hand-worked cells of the oracle tests (and two ambiguous / NaN-heavy ones) on the GPU."""
    vol = np.empty((2, 2, 2), np.float32)
    for i, val in enumerate(vals):
        vol[i >> 2, (i >> 1) & 1, i & 1] = val
    for li in (False, True):
        _same(M.marchingCubes(vol, M.MarchingCubesParams(lessInside=li, outVoxelPerFaceMap=True)),
              O.marching_cubes(vol, less_inside=li))


_GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mc_reference.npz"))


@pytest.mark.parametrize("name", [str(c) for c in _GOLDEN["cases"]])
def test_matches_reference_mesher(M, name):
    """The CUDA mesher against the outputs of MeshLib's own mesher (MRVoxels/MRMarchingCubes.cpp,
    compiled from its sources) stored in tests/golden/mc_reference.npz: points bit for bit, the same
    triangles in the same order, the same face map, and the reference's error messages."""
    p = _GOLDEN[f"{name}/params"]
    parts = _GOLDEN[f"{name}/parts"]
    vol = _GOLDEN[f"{name}/vol"]
    prm = M.MarchingCubesParams(origin=tuple(p[0:3]), voxelSize=tuple(p[3:6]), iso=float(p[6]), lessInside=bool(p[7]),
                                maxVertices=int(p[8]), outVoxelPerFaceMap=True)
    err = str(_GOLDEN[f"{name}/error"])
    starts = parts if len(parts) else None
    if err:
        with pytest.raises(M.FwnError, match=err.rstrip(".")):
            M.marchingCubes(vol, prm, partStarts=starts)
        return
    tm = M.marchingCubes(vol, prm, partStarts=starts)
    ref = (_GOLDEN[f"{name}/points"], _GOLDEN[f"{name}/tris"], _GOLDEN[f"{name}/faceMap"])
    assert tm.numPoints == len(ref[0]) and tm.numTris == len(ref[1])
    if len(ref[0]):
        _same(tm, ref)
