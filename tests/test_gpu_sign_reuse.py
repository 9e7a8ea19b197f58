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


def _signed_pass(M, g, dims, xf, vals, enable, thr=0.5):
    import torch
    g.set_sign_reuse(enable)
    d = torch.from_numpy(vals.copy()).cuda()
    g.makeSignedByWindingNumber_dev(dims, xf, d.data_ptr(), threshold=thr, stream=0)
    torch.cuda.synchronize()
    g.set_sign_reuse(True)
    return d.cpu().numpy()


@pytest.mark.parametrize("precise", [True, False])
def test_sign_columns_identical(M, precise):
    """makeSignedByWindingNumber on a closed mesh with the grid's z axis vertical takes each column's
    signs from its crossings (the signed count of crossings above each voxel; the columns' crossing lists
    filled from the triangles); the negated voxels equal those of the winding-number walk at every
    voxel: clean, self-intersecting (winding number 2), far from the origin, a stack of 16 spheres (32
    crossings per column: more than a list holds, those columns cast their own ray, more than a ray
    keeps, they take the walk), coarse meshes (a cube, an 80-face sphere: triangles over many
    columns), ragged, z-scaled and turned (about z) grids, thresholds 0.5 and 0.3, and tilted grids
    (the walk)."""
    rng = np.random.default_rng(11)
    v, f = mg.noisy_icosphere(seed=1, level=5)
    stack_v = np.concatenate([v * 0.4 + np.float32([0, 0, 1.0 * k]) for k in range(16)]).astype(np.float32)
    stack_f = np.concatenate([f + k * len(v) for k in range(16)]).astype(np.int32)
    cube_v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32)
    cube_f = np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4], [2, 6, 7], [2, 7, 3], [0, 4, 6],
                       [0, 6, 2], [1, 3, 7], [1, 7, 5]], np.int32)
    iv, iff = mg.icosphere(1)
    cases = [mg.noisy_torus(seed=4), mg.overlapping_spheres(seed=3, level=5), ((v + np.float32(3.0e3)).astype(np.float32), f),
             (stack_v, stack_f), (cube_v, cube_f), (iv.astype(np.float32), iff.astype(np.int32))]
    negated = 0
    for cv, cf in cases:
        g = M.FastWindingNumber(cv, cf, precise=precise)
        assert g.is_closed()
        dims, xf = mg.grid_for(cv, 72)
        xf = np.asarray(xf, np.float32).copy()
        grids = [(tuple(dims), xf)]
        ragged = xf.copy()
        ragged[8] *= 0.5  # z pitch halved, twice the layers
        grids.append(((dims[0] - 5, dims[1] - 3, 2 * dims[2] + 1), ragged))
        turned = xf.copy()  # columns still vertical, the grid turned about z
        c, s = np.float32(np.cos(0.4)), np.float32(np.sin(0.4))
        turned[:9] = (np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], np.float32) @ turned[:9].reshape(3, 3)).reshape(-1)
        turned[9:] = 0.5 * (cv.min(0) + cv.max(0)) - turned[:9].reshape(3, 3) @ (0.5 * np.array(dims, np.float32))
        grids.append((tuple(dims), turned))
        for gd, gx in grids:
            vals = rng.uniform(0.1, 1.0, int(np.prod(gd))).astype(np.float32)
            for thr in (0.5, 0.3):
                a = _signed_pass(M, g, gd, gx, vals, True, thr)
                b = _signed_pass(M, g, gd, gx, vals, False, thr)
                assert np.array_equal(a, b)
                negated += int((a < 0).sum())
    assert negated > 0
    # a rotated grid keeps the walk (and the same result either way)
    cv, cf = cases[0]
    g = M.FastWindingNumber(cv, cf, precise=precise)
    dims, xf = mg.grid_for(cv, 40)
    c, s = np.float32(np.cos(0.3)), np.float32(np.sin(0.3))
    rot = np.asarray(xf, np.float32).copy()
    rot[:9] = (rot[:9].reshape(3, 3) @ np.array([[1, 0, 0], [0, c, -s], [0, s, c]], np.float32)).reshape(-1)
    vals = rng.uniform(0.1, 1.0, int(np.prod(dims))).astype(np.float32)
    assert np.array_equal(_signed_pass(M, g, dims, rot, vals, True), _signed_pass(M, g, dims, rot, vals, False))


def test_sign_columns_identical_at_benchmark_scale(M):
    """The 1,310,720-triangle icosphere, 256^3: the column rays negate the same voxels as the walk."""
    v, f = mg.noisy_icosphere(seed=0, level=8)
    dims, xf = mg.grid_for(v, 256)
    g = M.FastWindingNumber(v, f)
    vals = np.random.default_rng(2).uniform(0.1, 1.0, int(np.prod(dims))).astype(np.float32)
    a = _signed_pass(M, g, dims, xf, vals, True)
    b = _signed_pass(M, g, dims, xf, vals, False)
    assert np.array_equal(a, b) and (a < 0).any()


@pytest.mark.parametrize("precise", [True, False])
def test_reuse_and_rays_identical_on_tilted_grids(M, precise):
    """A grid whose z axis is not vertical has no column rays: its signs come from sign reuse and one
    ray per voxel, and equal the winding-number walk's, with and without a band."""
    for v, f in (mg.noisy_torus(seed=6), mg.overlapping_spheres(seed=4, level=5)):
        g = M.FastWindingNumber(v, f, precise=precise)
        dims, xf = mg.grid_for(v, 64)
        c, s = np.float32(np.cos(0.2)), np.float32(np.sin(0.2))
        tilt = np.asarray(xf, np.float32).copy()
        tilt[:9] = (tilt[:9].reshape(3, 3) @ np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)).reshape(-1)
        band = 0.03 * mg.diag(v)
        for opts in (None, M.DistanceToMeshOptions(maxDistSq=band * band)):
            res = []
            for enable in (True, False):
                g.set_sign_reuse(enable)
                res.append(g.calcFromGridWithDistances(dims, tilt, opts))
            g.set_sign_reuse(True)
            _same(*res)
            assert (res[0] < 0).any()


def test_signed_distance_grids_from_column_lists(M):
    """Signed-distance grids whose signs come from the columns' crossing lists equal the grids whose
    every sign comes from the winding-number walk: a turned (about z) grid, a coarse cube, 16 stacked
    spheres (overflowing lists), a band, and the slab calls of the same grid."""
    import torch
    v, f = mg.noisy_icosphere(seed=5, level=5)
    stack_v = np.concatenate([v * 0.4 + np.float32([0, 0, 1.0 * k]) for k in range(16)]).astype(np.float32)
    stack_f = np.concatenate([f + k * len(v) for k in range(16)]).astype(np.int32)
    cube_v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32) * np.float32(1.7)
    cube_f = np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4], [2, 6, 7], [2, 7, 3], [0, 4, 6],
                       [0, 6, 2], [1, 3, 7], [1, 7, 5]], np.int32)
    for cv, cf in ((v, f), (cube_v, cube_f), (stack_v, stack_f)):
        g = M.FastWindingNumber(cv, cf)
        dims, xf = mg.grid_for(cv, 60)
        dims = (dims[0] + 3, dims[1] - 2, dims[2] + 1)
        turned = np.asarray(xf, np.float32).copy()
        c, s = np.float32(np.cos(0.7)), np.float32(np.sin(0.7))
        turned[:9] = (np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], np.float32) @ turned[:9].reshape(3, 3)).reshape(-1)
        turned[9:] = 0.5 * (cv.min(0) + cv.max(0)) - turned[:9].reshape(3, 3) @ (0.5 * np.array(dims, np.float32))
        band = 0.05 * mg.diag(cv)
        for gx in (np.asarray(xf, np.float32), turned):
            for opts in (None, M.DistanceToMeshOptions(maxDistSq=band * band)):
                res = []
                for enable in (True, False):
                    g.set_sign_reuse(enable)
                    res.append(g.calcFromGridWithDistances(dims, gx, opts))
                g.set_sign_reuse(True)
                _same(*res)
        n = int(np.prod(dims))
        whole = torch.empty(n, device="cuda")
        g.calcFromGridWithDistances_dev(dims, turned, whole.data_ptr(), stream=0)
        parts = []
        for z0, z1 in ((0, 7), (7, 30), (30, dims[2])):
            t = torch.empty((z1 - z0) * dims[0] * dims[1], device="cuda")
            g.calcFromGridWithDistancesSlab_dev(dims, turned, z0, z1, t.data_ptr(), stream=0)
            parts.append(t)
        torch.cuda.synchronize()
        assert torch.equal(torch.cat(parts).view(torch.int32), whole.view(torch.int32))
        assert (whole < 0).any()


def test_column_signs_on_small_and_outlying_grids(M):
    """Column signs on grids of one voxel, of fewer than 32 voxels per row, wholly inside and wholly
    outside the mesh, and reaching far past it: the same grids as the winding-number walk."""
    v, f = mg.noisy_torus(seed=9)
    g = M.FastWindingNumber(v, f)
    lo, hi = v.min(0), v.max(0)
    mid = 0.5 * (lo + hi)
    cases = []
    for dims, pitch, origin in (((1, 1, 1), 0.1, mid), ((5, 3, 2), 0.05, lo), ((31, 2, 40), 0.02, lo),
                                ((8, 8, 8), 0.01, np.float32([hi[0] + 1.0, mid[1], mid[2]])),  # outside, beside the mesh
                                ((16, 16, 64), 0.2, lo - 3.0)):  # reaching far past it
        xf = np.zeros(12, np.float32)
        xf[0] = xf[4] = xf[8] = pitch
        xf[9:12] = origin
        cases.append((dims, xf))
    # a grid around a point inside the torus tube
    vi, fi = mg.noisy_icosphere(seed=2, level=5)
    gi = M.FastWindingNumber(vi, fi)
    xf = np.zeros(12, np.float32)
    xf[0] = xf[4] = xf[8] = 0.01
    xf[9:12] = -0.05
    for gg, dims, x in [(g, d, x) for d, x in cases] + [(gi, (10, 10, 10), xf)]:
        res = []
        for enable in (True, False):
            gg.set_sign_reuse(enable)
            res.append(gg.calcFromGridWithDistances(dims, x))
        gg.set_sign_reuse(True)
        _same(*res)
    assert (res[0] < 0).all()  # the last grid lies inside the sphere


def test_column_signs_with_vertices_on_column_centres(M):
    """A cube and an octahedron whose vertices, edges and faces lie exactly on voxel centres and grid
    columns (rays through vertices and along edges, vertical faces in the rays' planes, voxels on the
    faces): the column signs equal the winding-number walk's at every voxel."""
    cube_v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32) * np.float32(1.5) + np.float32(0.5)
    cube_f = np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4], [2, 6, 7], [2, 7, 3], [0, 4, 6],
                       [0, 6, 2], [1, 3, 7], [1, 7, 5]], np.int32)
    octa_v = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32) + np.float32(1.25)
    octa_f = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]], np.int32)
    xf = np.zeros(12, np.float32)
    xf[0] = xf[4] = xf[8] = 0.25  # voxel centres at multiples of 0.25, the vertices among them
    flipped = 0
    for cv, cf in ((cube_v, cube_f), (octa_v, octa_f)):
        g = M.FastWindingNumber(cv, cf)
        assert g.is_closed()
        for opts in (None, M.DistanceToMeshOptions(maxDistSq=0.3 ** 2)):
            res = []
            for enable in (True, False):
                g.set_sign_reuse(enable)
                res.append(g.calcFromGridWithDistances((11, 11, 11), xf, opts))
            g.set_sign_reuse(True)
            _same(*res)
            flipped += int((res[0] < 0).sum())
        vals = np.random.default_rng(1).uniform(0.1, 1.0, 11 ** 3).astype(np.float32)
        assert np.array_equal(_signed_pass(M, g, (11, 11, 11), xf, vals, True), _signed_pass(M, g, (11, 11, 11), xf, vals, False))
    assert flipped > 0


def test_column_signs_on_mirrored_grids(M):
    """Grids mirrored along x (column signs, the index map's determinant negative) and along z (no
    column signs: z must point up): the same grids as the winding-number walk, and the mirrored grids
    hold the unmirrored one's values in mirrored order."""
    v, f = mg.noisy_torus(seed=10)
    g = M.FastWindingNumber(v, f)
    dims, xf = mg.grid_for(v, 48)
    xf = np.asarray(xf, np.float32)
    plain = g.calcFromGridWithDistances(dims, xf).reshape(dims[2], dims[1], dims[0])
    mx = xf.copy()
    mx[0] = -xf[0]
    mx[9] = xf[9] + xf[0] * (dims[0] - 1)
    mz = xf.copy()
    mz[8] = -xf[8]
    mz[11] = xf[11] + xf[8] * (dims[2] - 1)
    for gx, flip in ((mx, 2), (mz, 0)):
        res = []
        for enable in (True, False):
            g.set_sign_reuse(enable)
            res.append(g.calcFromGridWithDistances(dims, gx))
        g.set_sign_reuse(True)
        _same(*res)
        mirrored = res[0].reshape(dims[2], dims[1], dims[0])
        assert np.array_equal(np.signbit(np.flip(mirrored, axis=flip)), np.signbit(plain))


@pytest.mark.parametrize("precise", [True, False])
def test_paired_walk_with_voxels_on_the_surface(M, precise):
    """The paired walk (grids large enough for work items of several tiles) on a cube whose faces
    hold 256^2-voxel layers and on the noisy sphere: voxels on the surface make the precise walk list
    their pair steps for the fix-up pass; the grids equal the one-voxel walk's with the winding-number
    signs, bit for bit, unbanded and banded."""
    cube_v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32) * np.float32(1.5) + np.float32(0.5)
    cube_f = np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4], [2, 6, 7], [2, 7, 3], [0, 4, 6],
                       [0, 6, 2], [1, 3, 7], [1, 7, 5]], np.int32)
    xf = np.zeros(12, np.float32)
    xf[0] = xf[4] = xf[8] = 0.0125  # voxel centres at multiples of 1/80: the faces at 40 and 160
    dims = (208, 208, 416)
    v, f = mg.noisy_icosphere(seed=6, level=6)
    dims2, xf2 = mg.grid_for(v, 256)
    for cv, cf, d, x in ((cube_v, cube_f, dims, xf), (v, f, dims2, xf2)):
        g = M.FastWindingNumber(cv, cf, precise=precise)
        for opts in (None, M.DistanceToMeshOptions(maxDistSq=(0.02 * mg.diag(cv)) ** 2)):
            res = []
            for enable in (True, False):
                g.set_sign_reuse(enable)
                res.append(g.calcFromGridWithDistances(d, x, opts))
            g.set_sign_reuse(True)
            _same(*res)
            assert (res[0] == 0).any() or cf is f
            if opts is not None:  # the banded bricks (exact cull): paired walk over brick runs, fix-up
                import torch
                out = torch.full((int(np.prod(d)),), 7.0, device="cuda")
                g.calcFromGridWithDistancesBanded_dev(d, x, out.data_ptr(), opts, None, stream=0)
                torch.cuda.synchronize()
                _same(out.cpu().numpy(), res[1])
