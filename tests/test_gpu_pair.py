"""The paired walks (two voxels per lane through one packet traversal): winding-number grids equal the
one-query walk's values at the same points bit for bit, in both arithmetic modes and for slabs."""
import numpy as np
import pytest

from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precise", [True, False])
def test_paired_winding_numbers_equal_point_queries(fwn_lib, precise):
    import meshlib_gb300 as M
    v, f = mg.noisy_icosphere(seed=3, level=7)
    g = M.FastWindingNumber(v, f, precise=precise)
    dims, xf = mg.grid_for(v, 256)  # work items of several tiles: the paired walk
    xf = np.asarray(xf, np.float32)
    wn = g.calcFromGrid(dims, xf).reshape(dims[2], dims[1], dims[0])
    rng = np.random.default_rng(0)
    idx = rng.integers(0, [dims[0], dims[1], dims[2]], (200_000, 3))
    # the voxel centres as the grid computes them (left-to-right dots, FP32)
    fx, fy, fz = (idx[:, k].astype(np.float32) for k in range(3))
    pts = np.stack([((xf[0] * fx + xf[1] * fy) + xf[2] * fz) + xf[9], ((xf[3] * fx + xf[4] * fy) + xf[5] * fz) + xf[10],
                    ((xf[6] * fx + xf[7] * fy) + xf[8] * fz) + xf[11]], 1).astype(np.float32)
    at = g.calcFromVector(pts)
    grid_at = wn[idx[:, 2], idx[:, 1], idx[:, 0]]
    assert np.array_equal(grid_at.view(np.uint32), at.view(np.uint32))
    # slabs of the same grid
    import torch
    z0, z1 = 37, 171
    sl = torch.empty((z1 - z0) * dims[0] * dims[1], device="cuda")
    g.calcFromGridSlab_dev(dims, xf, z0, z1, sl.data_ptr(), stream=0)
    torch.cuda.synchronize()
    assert np.array_equal(sl.cpu().numpy().reshape(z1 - z0, dims[1], dims[0]).view(np.uint32), wn[z0:z1].view(np.uint32))


@pytest.mark.parametrize("precise", [True, False])
def test_paired_point_winding_numbers(fwn_lib, precise):
    """Large point sets (Morton-ordered, two tiles per walk) give each point the same winding number as
    small batches of the same points (one tile per walk), bit for bit."""
    import meshlib_gb300 as M
    v, f = mg.noisy_icosphere(seed=8, level=6)
    g = M.FastWindingNumber(v, f, precise=precise)
    rng = np.random.default_rng(4)
    pts = np.concatenate([v[rng.integers(0, len(v), 60_000)] * rng.uniform(0.99, 1.01, (60_000, 1)),
                          rng.uniform(-1.3, 1.3, (40_001, 3))]).astype(np.float32)
    whole = g.calcFromVector(pts)
    parts = np.concatenate([g.calcFromVector(pts[i:i + 5000]) for i in range(0, len(pts), 5000)])
    assert np.array_equal(whole.view(np.uint32), parts.view(np.uint32))


@pytest.mark.parametrize("precise", [True, False])
def test_paired_signed_distance_slabs(fwn_lib, precise):
    """Slabs of a 256^3 signed-distance grid (paired walk, its fix-up pass and the column signs over
    each slab's own range) stack to the whole grid, bit for bit, unbanded and banded."""
    import torch

    import meshlib_gb300 as M
    v, f = mg.noisy_icosphere(seed=9, level=7)
    g = M.FastWindingNumber(v, f, precise=precise)
    dims, xf = mg.grid_for(v, 256)
    n = int(np.prod(dims))
    for opts in (None, M.DistanceToMeshOptions(maxDistSq=(0.02 * mg.diag(v)) ** 2)):
        whole = torch.empty(n, device="cuda")
        g.calcFromGridWithDistances_dev(dims, xf, whole.data_ptr(), options=opts, stream=0)
        parts = []
        for z0, z1 in ((0, 90), (90, 200), (200, 256)):
            t = torch.empty((z1 - z0) * dims[0] * dims[1], device="cuda")
            g.calcFromGridWithDistancesSlab_dev(dims, xf, z0, z1, t.data_ptr(), options=opts, stream=0)
            parts.append(t)
        torch.cuda.synchronize()
        assert torch.equal(torch.cat(parts).view(torch.int32), whole.view(torch.int32))


@pytest.mark.parametrize("precise", [True, False])
def test_ordered_point_distances(fwn_lib, precise):
    """Signed distances at large point sets (Morton-ordered and walked in that order) equal those of
    small batches of the same points (unordered), bit for bit: shell points, points in the box, the
    mesh's own vertices (on the surface) and, for a self-intersecting closed mesh, points inside both
    parts.  (A paired walk for points, two tiles per walk with paired rays, measured slower: 4 M shell
    points 3.94 -> 4.13 ms, so points keep one tile per walk for distances.)"""
    import meshlib_gb300 as M
    rng = np.random.default_rng(5)
    for v, f in (mg.noisy_icosphere(seed=10, level=6), mg.overlapping_spheres(seed=5, level=5)):
        g = M.FastWindingNumber(v, f, precise=precise)
        pts = np.concatenate([v[rng.integers(0, len(v), 50_000)] * rng.uniform(0.995, 1.005, (50_000, 1)),
                              rng.uniform(v.min(0) - 0.2, v.max(0) + 0.2, (40_000, 3)), v[:10_000]]).astype(np.float32)
        rng.shuffle(pts)
        for opts in (None, M.DistanceToMeshOptions(maxDistSq=0.01)):
            whole = g.calcWithDistances(pts, opts)
            parts = np.concatenate([g.calcWithDistances(pts[i:i + 5000], opts) for i in range(0, len(pts), 5000)])
            assert np.array_equal(np.isnan(whole), np.isnan(parts))
            m = ~np.isnan(whole)
            assert np.array_equal(whole[m].view(np.uint32), parts[m].view(np.uint32))
            assert (whole[m] == 0).any()
