"""Sign reuse in signed-distance grids of closed surfaces (gbfwn_set_sign_reuse, include/gbfwn.h).

The closedness fingerprint recognises closed oriented surfaces (also self-intersecting ones and
disjoint unions) and rejects open ones, flipped faces and holes.  On closed meshes the grids with
sign reuse equal the grids that evaluate every voxel's winding number, bit for bit, for both
arithmetic modes, with and without a band, far from the origin, and on the bricks of the banded
path; where it does not apply (open meshes, a threshold near an integer, beta < 2) the call is the
plain one.  The parity tests against the oracle and the reference's kernels run with it on."""
import numpy as np
import pytest

from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300


def _grids(M, v, f, n, opts=None, precise=True):
    g = M.FastWindingNumber(v, f, precise=precise)
    dims, xf = mg.grid_for(v, n)
    g.set_sign_reuse(True)
    on = g.calcFromGridWithDistances(dims, xf, opts)
    g.set_sign_reuse(False)
    off = g.calcFromGridWithDistances(dims, xf, opts)
    return g, on, off


def _same(a, b):
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    assert np.array_equal(a[m].view(np.uint32), b[m].view(np.uint32))


def test_closedness(M):
    v, f = mg.noisy_torus(seed=0)
    assert M.FastWindingNumber(v, f).is_closed()
    sv, sf = mg.overlapping_spheres(seed=0, level=3)  # self-intersecting, still closed
    assert M.FastWindingNumber(sv, sf).is_closed()
    assert not M.FastWindingNumber(v, f[1:]).is_closed()  # a hole
    flipped = f.copy()
    flipped[7] = flipped[7][::-1]
    assert not M.FastWindingNumber(v, flipped).is_closed()
    invalid = f.copy()
    invalid[3] = -1  # an invalid face is not part of the surface: a hole
    assert not M.FastWindingNumber(v, invalid).is_closed()
    two = np.concatenate([f, f + len(v)])
    assert M.FastWindingNumber(np.concatenate([v, v + 5.0]), two).is_closed()
    assert not M.FastWindingNumber(v[:3].copy(), np.array([[0, 1, 2]], np.int32)).is_closed()


@pytest.mark.parametrize("precise", [True, False])
def test_reuse_identical_on_closed_meshes(M, precise):
    v, f = mg.noisy_torus(seed=1)
    g, on, off = _grids(M, v, f, 64, precise=precise)
    _same(on, off)
    vi, fi = mg.noisy_icosphere(seed=3, level=6)
    _, on, off = _grids(M, vi, fi, 128, precise=precise)
    _same(on, off)
    sv, sf = mg.overlapping_spheres(seed=2, level=5)
    _, on, off = _grids(M, sv, sf, 96, precise=precise)
    _same(on, off)
    assert (on < 0).any() and (on > 0).any()


def test_reuse_identical_with_bands_and_far_from_origin(M):
    v, f = mg.noisy_icosphere(seed=4, level=6)
    diag = mg.diag(v)
    for opts in (M.DistanceToMeshOptions(maxDistSq=(0.05 * diag) ** 2),
                 M.DistanceToMeshOptions(minDistSq=(0.01 * diag) ** 2, maxDistSq=(0.2 * diag) ** 2),
                 M.DistanceToMeshOptions(minDistSq=(0.01 * diag) ** 2, maxDistSq=(0.1 * diag) ** 2, nullOutsideMinMax=False)):
        _, on, off = _grids(M, v, f, 96, opts)
        _same(on, off)
    far = (v + np.float32(3.0e3)).astype(np.float32)  # coordinates ~3000x the voxel pitch's scale
    _, on, off = _grids(M, far, f, 96)
    _same(on, off)


def test_reuse_identical_on_banded_bricks(M):
    import torch
    v, f = mg.noisy_icosphere(seed=5, level=7)
    dims, xf = mg.grid_for(v, 128)
    band = 0.02 * mg.diag(v)
    g = M.FastWindingNumber(v, f)
    o = M.DistanceToMeshOptions(maxDistSq=band * band)
    res = []
    for enable in (True, False):
        g.set_sign_reuse(enable)
        out = torch.empty(int(np.prod(dims)), device="cuda")
        g.calcFromGridWithDistancesBanded_dev(dims, xf, out.data_ptr(), o, None, stream=0)
        torch.cuda.synchronize()
        res.append(out.cpu().numpy())
    _same(*res)
    assert np.isfinite(res[0]).any()


def test_not_applied_where_it_does_not_hold(M):
    v, f = mg.noisy_torus(seed=2)
    open_f = f[:-40]
    _, on, off = _grids(M, v, open_f, 48)
    _same(on, off)
    for opts in (M.DistanceToMeshOptions(windingNumberThreshold=0.9), M.DistanceToMeshOptions(windingNumberBeta=1.5)):
        _, on, off = _grids(M, v, f, 48, opts)
        _same(on, off)


def test_reuse_identical_at_benchmark_scale(M):
    """The 1,310,720-triangle icosphere on a 256^3 grid: with the sign reuse and the column hand-over
    the grid equals the grid that evaluates every voxel's winding number, unbanded and banded."""
    import torch
    v, f = mg.noisy_icosphere(seed=0, level=8)
    dims, xf = mg.grid_for(v, 256)
    g = M.FastWindingNumber(v, f)
    assert g.is_closed()
    band = 0.01 * mg.diag(v)
    for opts in (None, M.DistanceToMeshOptions(maxDistSq=band * band)):
        res = []
        for enable in (True, False):
            g.set_sign_reuse(enable)
            out = torch.empty(int(np.prod(dims)), device="cuda")
            g.calcFromGridWithDistances_dev(dims, xf, out.data_ptr(), options=opts, stream=0)
            torch.cuda.synchronize()
            res.append(out.cpu().numpy())
        _same(*res)
    g.set_sign_reuse(True)


@pytest.mark.parametrize("precise", [True, False])
def test_self_intersection_bits_by_rays(M, precise):
    """calcSelfIntersections without winding numbers takes a closed mesh's bits from ray crossings; they
    equal the bits of the winding-number walk (with_wn=True) on self-intersecting and clean closed
    meshes, and open meshes keep the walk."""
    cases = [mg.overlapping_spheres(seed=0, level=5), mg.overlapping_spheres(seed=1, level=6), mg.noisy_icosphere(seed=2, level=6)]
    v, f = mg.noisy_torus(seed=3)
    cases.append((v, f))
    cases.append((v, f[:-50]))  # open
    flagged = 0
    for v, f in cases:
        g = M.FastWindingNumber(v, f, precise=precise)
        fast = g.calcSelfIntersections()
        walk, _ = g.calcSelfIntersections(with_wn=True)
        assert np.array_equal(fast, walk)
        flagged += int(fast.sum())
    assert flagged > 0
