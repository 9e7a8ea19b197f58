"""CUDA path vs the CPU oracle (the reference's FastWindingNumber restated), through the C ABI.

Tolerances (stated once, used throughout):
  * tree nodes and dipoles: bit-exact (the GPU builds the reference's tree with the reference's
    float arithmetic);
  * winding numbers: |w_gpu - w_oracle| <= WN_TOL (FP32 sums of a few hundred terms, different
    summation order, atan2f last-ulp differences);
  * inside/outside sign of signed distances and self-intersection bits: exact, except where the
    oracle's winding number lies within TAU of the threshold (those are counted, not failed);
  * distances: |d_gpu - d_oracle| <= 1e-5 * bbox diagonal (the contract's tolerance).
"""
import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

WN_TOL = 5e-5
TAU = 1e-3


@pytest.fixture(scope="module")
def fwncls(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300.FastWindingNumber


def _sign_ok(d_gpu, d_ref, wn_ref, thr=0.5):
    both = np.isfinite(d_gpu) & np.isfinite(d_ref)
    mism = both & (np.signbit(d_gpu) != np.signbit(d_ref))  # signbit keeps the sign of a zero distance
    near = np.abs(wn_ref - thr) < TAU
    return int((mism & ~near).sum()), int((mism & near).sum())


def test_tree_and_dipoles_bit_exact(fwncls, torus):
    v, f = torus
    o = O.Oracle(v, f)
    g = fwncls(v, f)
    nodes, dip = g.tree()
    ref = o.nodes()
    assert len(nodes) == 2 * len(f) - 1
    assert np.array_equal(nodes.view(np.uint8), ref.view(np.uint8))
    assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32))


def test_tree_bit_exact_large(fwncls):
    v, f = mg.noisy_icosphere(seed=5, level=6)  # 81,920 triangles
    o = O.Oracle(v, f)
    g = fwncls(v, f)
    nodes, dip = g.tree()
    assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8))
    assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32))


def _plane_grid(n):
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    v = np.stack([i.ravel(), j.ravel(), np.zeros((n + 1) ** 2)], 1).astype(np.float32) / n
    a = (i[:-1, :-1] * (n + 1) + j[:-1, :-1]).ravel()
    f = np.concatenate([np.stack([a, a + n + 1, a + n + 2], 1), np.stack([a, a + n + 2, a + 1], 1)]).astype(np.int32)
    return v, f


@pytest.mark.parametrize("n, dup", [(20, 2), (110, 2), (64, 1)])
def test_tree_bit_exact_with_ties(fwncls, n, dup):
    """Flat grids (every box centre ties in z) with duplicated faces (identical boxes: only the face
    id breaks the tie); the larger cases go through the multi-level radix-select path."""
    v, f = _plane_grid(n)
    f = np.concatenate([f] * dup)
    o = O.Oracle(v, f)
    g = fwncls(v, f)
    nodes, dip = g.tree()
    assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8))
    assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32))


def test_tree_bit_exact_sizes(fwncls):
    """Leaf counts around the shared-memory threshold and odd sizes."""
    for level, keep in [(3, 1), (5, 1023), (5, 1024), (5, 1025), (6, 2049), (6, 4095), (4, 1), (4, 2), (4, 3)]:
        v, f = mg.noisy_icosphere(seed=level, level=level)
        f = f[:keep]
        o = O.Oracle(v, f)
        nodes, dip = fwncls(v, f).tree()
        assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8)), (level, keep)
        assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32)), (level, keep)


@pytest.mark.parametrize("precise", [False, True])
def test_from_grid_matches_oracle(fwncls, torus, precise):
    v, f = torus
    dims, xf = mg.grid_for(v, 24)
    o = O.Oracle(v, f)
    ref = o.from_grid(dims, xf, prec=1 if precise else 0)
    g = fwncls(v, f, precise=precise)
    w = g.calcFromGrid(dims, xf)
    err = np.abs(w - ref)
    assert err.max() <= WN_TOL, f"max {err.max()} rms {np.sqrt((err**2).mean())}"


def test_from_grid_ragged_dims(fwncls, small_sphere):
    v, f = small_sphere
    dims = (13, 7, 5)  # not multiples of the 4x4x2 warp tile
    _, xf = mg.grid_for(v, 13)
    o = O.Oracle(v, f)
    ref = o.from_grid(dims, xf)
    w = fwncls(v, f, precise=False).calcFromGrid(dims, xf)
    assert np.abs(w - ref).max() <= WN_TOL


@pytest.mark.parametrize("precise", [False, True])
def test_signed_distance_grid(fwncls, torus, precise):
    v, f = torus
    dims, xf = mg.grid_for(v, 32)
    o = O.Oracle(v, f)
    ref, wref = o.from_grid_with_distances(dims, xf, prec=1, want_fwn=True)
    g = fwncls(v, f, precise=precise)
    d = g.calcFromGridWithDistances(dims, xf)
    assert np.isfinite(d).all()
    diag = mg.diag(v)
    err = np.abs(np.abs(d) - np.abs(ref))
    assert err.max() <= 1e-5 * diag, f"distance max err {err.max()} vs {1e-5 * diag}"
    bad, near = _sign_ok(d, ref, wref)
    assert bad == 0, f"{bad} sign mismatches away from the threshold ({near} near it)"


def test_signed_distance_banded(fwncls, small_sphere):
    """Reference's own banded request (MRVoxels/MROffset.cpp:176-183): NaN outside [min, max)."""
    v, f = small_sphere
    dims, xf = mg.grid_for(v, 32)
    band = 0.05 * mg.diag(v)
    vox = float(xf[0])
    opts_o = O.make_options(minDistSq=(band - 1.001 * vox) ** 2, maxDistSq=(band + 1.001 * vox) ** 2)
    from meshlib_gb300 import DistanceToMeshOptions
    opts = DistanceToMeshOptions(minDistSq=opts_o.minDistSq, maxDistSq=opts_o.maxDistSq)
    o = O.Oracle(v, f)
    ref, wref = o.from_grid_with_distances(dims, xf, opts_o, prec=1, want_fwn=True)
    d = fwncls(v, f).calcFromGridWithDistances(dims, xf, opts)
    fin_g, fin_r = np.isfinite(d), np.isfinite(ref)
    # the NaN pattern may differ only where |d| sits on the band edge within the tolerance
    diff = fin_g != fin_r
    edge = np.minimum(np.abs(np.abs(np.where(fin_g, d, ref)) - np.sqrt(opts_o.minDistSq)),
                      np.abs(np.abs(np.where(fin_g, d, ref)) - np.sqrt(opts_o.maxDistSq)))
    assert (diff & (edge > 1e-5 * mg.diag(v))).sum() == 0
    both = fin_g & fin_r
    assert both.sum() > 100
    assert np.abs(np.abs(d[both]) - np.abs(ref[both])).max() <= 1e-5 * mg.diag(v)
    bad, _ = _sign_ok(d, ref, wref)
    assert bad == 0


def test_not_null_outside(fwncls, small_sphere):
    v, f = small_sphere
    dims, xf = mg.grid_for(v, 16)
    from meshlib_gb300 import DistanceToMeshOptions
    opts = DistanceToMeshOptions(maxDistSq=0.01, nullOutsideMinMax=False)
    d = fwncls(v, f).calcFromGridWithDistances(dims, xf, opts)
    ref = O.Oracle(v, f).from_grid_with_distances(dims, xf, O.make_options(maxDistSq=0.01, nullOutsideMinMax=False), prec=1)
    assert np.isfinite(d).all()
    assert np.abs(np.abs(d) - np.abs(ref)).max() <= 1e-5 * mg.diag(v)


@pytest.mark.parametrize("precise", [False, True])
def test_from_vector_and_skip_face(fwncls, small_sphere, precise):
    v, f = small_sphere
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1.3, 1.3, (3000, 3)).astype(np.float32)
    o = O.Oracle(v, f)
    g = fwncls(v, f, precise=precise)
    w = g.calcFromVector(pts)
    ref = o.from_vector(pts, prec=1 if precise else 0)
    assert np.abs(w - ref).max() <= WN_TOL
    # skipFace: query at face centroids of one face, skipping it
    c = v[f[17]].mean(0, dtype=np.float64).astype(np.float32)[None]
    ws = g.calcFromVector(c, skipFace=17)
    rs = o.from_vector(c, skip_face=17, prec=1 if precise else 0)
    assert abs(ws[0] - rs[0]) <= WN_TOL


def test_shell_points_with_distances(fwncls, small_sphere):
    v, f = small_sphere
    pts = mg.shell_points(v, f, 20000, width=1e-3, seed=2)
    o = O.Oracle(v, f)
    ref = o.vector_with_distances(pts, prec=1)
    wref = o.from_vector(pts, prec=1)
    d = fwncls(v, f).calcWithDistances(pts)
    assert np.abs(np.abs(d) - np.abs(ref)).max() <= 1e-5 * mg.diag(v)
    bad, near = _sign_ok(d, ref, wref)
    assert bad == 0


@pytest.mark.parametrize("precise", [False, True])
def test_self_intersections(fwncls, precise):
    v, f = mg.figure8_torus(nu=48, nv=40)
    o = O.Oracle(v, f)
    bits_ref, wn_ref = o.self_intersections(prec=1 if precise else 0)
    g = fwncls(v, f, precise=precise)
    bits, wn = g.calcSelfIntersections(with_wn=True)
    assert np.abs(wn - wn_ref).max() <= WN_TOL
    near = (np.abs(wn_ref) < TAU) | (np.abs(wn_ref - 1) < TAU)
    assert ((bits != bits_ref) & ~near).sum() == 0
    assert bits.sum() > 0


def test_self_intersections_overlapping_spheres(fwncls):
    v, f = mg.overlapping_spheres(seed=2, level=4, offset=0.6)
    o = O.Oracle(v, f)
    bits_ref, wn_ref = o.self_intersections(prec=1)
    bits, wn = fwncls(v, f).calcSelfIntersections(with_wn=True)
    near = (np.abs(wn_ref) < TAU) | (np.abs(wn_ref - 1) < TAU)
    assert ((bits != bits_ref) & ~near).sum() == 0
    assert 0.1 * len(f) < bits.sum() < 0.5 * len(f)


def test_self_intersections_clean_and_invalid_faces(fwncls, torus):
    v, f = torus
    f2 = f.copy()
    f2[5] = -1  # an invalid face: excluded from the tree, never reported
    bits, wn = fwncls(v, f2).calcSelfIntersections(with_wn=True)
    assert not bits.any()
    assert np.isnan(wn[5]) and np.isfinite(np.delete(wn, 5)).all()
    o = O.Oracle(v, f2)
    g = fwncls(v, f2, precise=False)
    nodes, _ = g.tree()
    assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8))
    pts = np.array([[1.0, 0, 0], [0, 0, 0], [1.3, 0.2, 0.0]], np.float32)
    assert np.abs(g.calcFromVector(pts) - o.from_vector(pts)).max() <= WN_TOL


def test_by_parts_equals_whole(fwncls, small_sphere):
    v, f = small_sphere
    dims, xf = mg.grid_for(v, 20)
    g = fwncls(v, f)
    whole = g.calcFromGridWithDistances(dims, xf)
    nx, ny, nz = dims
    got = np.full(nx * ny * nz, np.nan, np.float32)
    seen = []

    def cb(data, sd, z0):
        seen.append((z0, sd[2]))
        got[z0 * nx * ny:(z0 + sd[2]) * nx * ny] = data
        return None

    g.calcFromGridWithDistancesByParts(cb, dims, xf, layerOverlap=1, maxLayersPerSlab=6)
    assert seen[0][0] == 0 and sum(1 for _ in seen) >= 3
    for (za, na), (zb, _) in zip(seen, seen[1:]):
        assert zb == za + na - 1  # one shared layer
    assert np.array_equal(got, whole)
    wgot = np.full(nx * ny * nz, np.nan, np.float32)

    def cb2(data, sd, z0):
        wgot[z0 * nx * ny:(z0 + sd[2]) * nx * ny] = data

    g.calcFromGridByParts(cb2, dims, xf, layerOverlap=0, maxLayersPerSlab=7)
    assert np.array_equal(wgot, g.calcFromGrid(dims, xf))


def test_cancel_and_errors(fwncls, small_sphere):
    import meshlib_gb300 as M
    v, f = small_sphere
    g = fwncls(v, f)
    dims, xf = mg.grid_for(v, 16)
    with pytest.raises(M.FwnError) as ei:
        g.calcFromGrid(dims, xf, cb=lambda p: p < 0.5)
    assert ei.value.status == M.CANCELLED
    with pytest.raises(M.FwnError) as ei:
        g.calcFromGrid((0, 4, 4), xf)
    assert ei.value.status == M.INVALID
    bad = f.copy()
    bad[0, 0] = len(v) + 5
    with pytest.raises(M.FwnError) as ei:
        fwncls(v, bad)
    assert ei.value.status == M.INVALID
    M.lib().gbfwn_debug_fail_next_allocs(1)
    with pytest.raises(M.FwnError) as ei:
        fwncls(v, f)
    assert ei.value.status == M.OUT_OF_MEMORY
    # the handle still works after the failures
    assert np.isfinite(g.calcFromGrid((4, 4, 4), xf)).all()


def test_tiny_meshes(fwncls):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.int32)
    g = fwncls(v, f, precise=False)
    o = O.Oracle(v, f)
    pts = np.array([[0.2, 0.2, 0.5], [0.2, 0.2, -0.5], [3, 3, 3], [0.2, 0.2, 0]], np.float32)
    assert np.abs(g.calcFromVector(pts) - o.from_vector(pts)).max() <= WN_TOL
    d = g.calcWithDistances(pts)
    ref = o.vector_with_distances(pts, prec=1)
    assert np.allclose(np.abs(d), np.abs(ref), atol=1e-6)
    # empty mesh: winding number 0, distance never below maxDistSq -> NaN
    e = fwncls(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    assert (e.calcFromVector(pts) == 0).all()
    assert np.isnan(e.calcWithDistances(pts)).all()
    # 1x1x1 grid, identity transform
    w1 = g.calcFromGrid((1, 1, 1), [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0])
    assert w1.shape == (1,)


def test_c1_config_parity(fwncls):
    """The reference's CPU-runnable workload: noisy torus, 16,384 triangles, 64^3 grid."""
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 64)
    o = O.Oracle(v, f)
    ref, wref = o.from_grid_with_distances(dims, xf, prec=1, want_fwn=True)
    d = fwncls(v, f).calcFromGridWithDistances(dims, xf)
    diag = mg.diag(v)
    err = np.abs(np.abs(d) - np.abs(ref))
    assert err.max() <= 1e-5 * diag
    bad, near = _sign_ok(d, ref, wref)
    assert bad == 0


def test_from_vector_large_ordered(fwncls, small_sphere):
    """>= 8192 points are processed in Morton order and scattered back: same values as the oracle."""
    v, f = small_sphere
    rng = np.random.default_rng(9)
    pts = rng.uniform(-1.3, 1.3, (30000, 3)).astype(np.float32)
    g = fwncls(v, f, precise=False)
    o = O.Oracle(v, f)
    assert np.abs(g.calcFromVector(pts) - o.from_vector(pts)).max() <= WN_TOL
    d = g.calcWithDistances(pts)
    ref = o.vector_with_distances(pts, prec=1)
    assert np.abs(np.abs(d) - np.abs(ref)).max() <= 1e-5 * mg.diag(v)


def test_grid_beyond_2_31_voxels(fwncls):
    """64-bit voxel indexing: a 1400 x 1400 x 1100 grid (2.16e9 voxels, 8.6 GB) on a 16k-triangle torus,
    computed in one device call; sampled voxels match the oracle's distances and signs."""
    import torch

    v, f = mg.noisy_torus(seed=0)
    dims = (1400, 1400, 1100)
    lo, hi = v.min(0) - 0.05, v.max(0) + 0.05
    vox = (hi - lo) / np.array(dims)
    xf = np.array([vox[0], 0, 0, 0, vox[1], 0, 0, 0, vox[2], *(lo + 0.5 * vox)], np.float32)
    n = int(np.prod(np.array(dims, np.int64)))
    assert n > 2 ** 31
    g = fwncls(v, f, precise=False)
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.integers(0, n, 3000), np.array([0, n - 1, 2 ** 31 - 1, 2 ** 31, 2 ** 31 + 1])])
    got = out[torch.from_numpy(idx).cuda()].cpu().numpy()
    z, rem = np.divmod(idx, dims[0] * dims[1])
    y, x = np.divmod(rem, dims[0])
    # voxel centres exactly as the grid computes them (row dots, then + b, in float)
    pts = (np.stack([x, y, z], 1).astype(np.float32) * np.array([xf[0], xf[4], xf[8]], np.float32)).astype(np.float32) + xf[9:]
    o = O.Oracle(v, f)
    ref = o.vector_with_distances(pts.astype(np.float32), prec=1)
    diag = mg.diag(v)
    assert np.abs(np.abs(got) - np.abs(ref)).max() <= 1e-5 * diag
    mism = np.signbit(got) != np.signbit(ref)
    if mism.any():
        wn = o.exact_wn(pts[mism])
        assert (np.abs(wn - 0.5) < TAU).all()
    del out


def test_host_grid_into_populated_and_fresh_buffers(fwn_lib):
    """Whole-grid host calls write straight into a caller buffer whose pages are populated (where the
    GPU can access pageable host memory) and go through a device buffer and a copy otherwise; both
    give the device entry point's grid bit for bit."""
    import torch

    import meshlib_gb300 as M
    v, f = mg.noisy_torus(seed=4)
    g = M.FastWindingNumber(v, f)
    dims = (37, 29, 23)
    _, xf = mg.grid_for(v, 37)
    n = int(np.prod(dims))
    d = torch.empty(n, device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, d.data_ptr(), stream=0)
    w = torch.empty(n, device="cuda")
    g.calcFromGrid_dev(dims, xf, w.data_ptr(), stream=0)
    torch.cuda.synchronize()
    ref_d, ref_w = d.cpu().numpy(), w.cpu().numpy()
    for make in (lambda: np.full(n, 7.0, np.float32), lambda: np.empty(n, np.float32)):
        out = make()
        g.calcFromGridWithDistances(dims, xf, out=out)
        assert np.array_equal(out.view(np.int32), ref_d.view(np.int32))
    assert np.array_equal(g.calcFromGrid(dims, xf).view(np.int32), ref_w.view(np.int32))
