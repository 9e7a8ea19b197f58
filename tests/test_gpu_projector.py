"""Points-to-mesh projection (MR::IPointsToMeshProjector) on the GPU vs the CPU oracle and the
reference's own GPU projector, through the C ABI.

Tolerances:
  * distance: |sqrt(d2_gpu) - sqrt(d2_oracle)| <= 1e-5 * bbox diagonal (the contract's tolerance);
  * face: equal to the oracle's, or (equidistant faces, e.g. a point whose closest mesh point is a
    vertex or an edge: the faces around it tie exactly, and which one a search meets first depends on
    its visiting order) a face whose exact FP64 distance equals the oracle's minimum within that
    tolerance, at the same closest point;
  * projected point: within 1e-5 * diagonal of the oracle's when the faces agree, and always equal to
    (1-a-b) v0 + a v1 + b v2 of the returned face and barycentrics.
"""
import math

import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300


def _points(v, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = v.min(0), v.max(0)
    ext = hi - lo
    box = rng.uniform(lo - 0.3 * ext, hi + 0.3 * ext, (n, 3))
    far = rng.normal(size=(n // 8, 3)) * 5 * ext.max()
    return np.concatenate([box, far]).astype(np.float32)


def _exact_face_dist2(v, f, pts, faces):
    out = np.empty(len(pts))
    for i, (p, fc) in enumerate(zip(pts.astype(np.float64), faces)):
        q = np.empty(3)
        O.lib().orc_closest_point_d(p.ctypes.data, np.ascontiguousarray(v[f[fc]].astype(np.float64)).ctypes.data, q.ctypes.data)
        out[i] = float(((q - p) ** 2).sum())
    return out


def _check(v, f, got, ref, pts_mapped, mesh_v=None):
    """got / ref: projection records; pts_mapped: the queries in the projection space."""
    mv = v if mesh_v is None else mesh_v
    diag = mg.diag(mv)
    found = ref["face"] >= 0
    assert np.array_equal(got["face"] >= 0, found)
    assert (got["edge"] == -1).all()
    dg, dr = np.sqrt(got["distSq"][found].astype(np.float64)), np.sqrt(ref["distSq"][found].astype(np.float64))
    assert np.abs(dg - dr).max(initial=0) <= 1e-5 * diag
    diff = np.flatnonzero(found & (got["face"] != ref["face"]))
    if len(diff):  # ties only: the returned face is as close as the oracle's
        d_ours = np.sqrt(_exact_face_dist2(mv, f, pts_mapped[diff], got["face"][diff]))
        assert np.abs(d_ours - np.sqrt(ref["distSq"][diff].astype(np.float64))).max() <= 1e-5 * diag
        # and almost always it is the same mesh point (a vertex or an edge shared by the tied faces);
        # a different point means a query equidistant (within the tolerance) from two parts of the
        # surface, e.g. near the centre of a sphere, where which one a search keeps is arbitrary
        moved = np.abs(got["point"][diff] - ref["point"][diff]).max(1) > 1e-5 * diag
        assert moved.sum() <= max(2, len(got) // 100), f"{int(moved.sum())} ties with different closest points"
    same = np.flatnonzero(found & (got["face"] == ref["face"]))
    assert np.abs(got["point"][same] - ref["point"][same]).max(initial=0) <= 1e-5 * diag
    tri = mv[f[got["face"][found]]].astype(np.float64)
    a, b = got["bary"][found, 0:1].astype(np.float64), got["bary"][found, 1:2].astype(np.float64)
    recon = (1 - a - b) * tri[:, 0] + a * tri[:, 1] + b * tri[:, 2]
    assert np.abs(recon - got["point"][found]).max(initial=0) <= 1e-5 * diag
    return len(diff)


@pytest.mark.parametrize("precise", [False, True])
def test_projection_vs_oracle(M, precise):
    v, f = mg.noisy_icosphere(seed=3, level=4)
    pts = _points(v, 6000, 1)
    o = O.Oracle(v, f)
    ref = o.find_projections(pts)
    pr = M.PointsToMeshProjector(precise=precise)
    pr.updateMeshData(v, f)
    got = pr.findProjections(pts)
    _check(v, f, got, ref, pts)


def test_projection_morton_path_and_shell(M):
    """>= 8192 points go through the Morton-ordered path; shell points sit within 1e-3 of the surface."""
    v, f = mg.noisy_torus(seed=2)
    pts = np.concatenate([mg.shell_points(v, f, 20000, width=1e-3, seed=4), _points(v, 4000, 2)])
    ref = O.Oracle(v, f).find_projections(pts)
    pr = M.PointsToMeshProjector()
    pr.updateMeshData(v, f)
    _check(v, f, pr.findProjections(pts), ref, pts)


def test_projection_transforms(M):
    v, f = mg.noisy_icosphere(seed=5, level=4)
    pts = _points(v, 3000, 3)
    o = O.Oracle(v, f)
    pr = M.PointsToMeshProjector()
    pr.updateMeshData(v, f)
    c, s = math.cos(0.4), math.sin(0.4)
    obj = np.array([1.5 * c, -1.5 * s, 0, 1.5 * s, 1.5 * c, 0, 0, 0, 1.5, 0.2, 0.1, -0.3], np.float32)  # scales the points
    rigid = np.array([c, 0, s, 0, 1, 0, -s, 0, c, -0.1, 0.4, 0.2], np.float32)
    shear = np.array([1.2, 0.3, 0, 0, 0.9, 0, 0.1, 0, 1.05, 0.05, 0, 0], np.float32)
    assert O.is_rigid(rigid) and not O.is_rigid(shear)

    def mapped(xf, p):
        return (p.astype(np.float64) @ xf[:9].reshape(3, 3).T.astype(np.float64) + xf[9:]).astype(np.float32)

    # point map only
    _check(v, f, pr.findProjections(pts, objXf=obj), o.find_projections(pts, objXf=obj), mapped(obj, pts))
    # rigid mesh map (folded into the point map)
    got = pr.findProjections(pts, objXf=obj, refXf=rigid)
    ref = o.find_projections(pts, objXf=obj, refXf=rigid)
    A = rigid[:9].reshape(3, 3).astype(np.float64)
    back = ((mapped(obj, pts).astype(np.float64) - rigid[9:]) @ A).astype(np.float32)
    _check(v, f, got, ref, back)
    # non-rigid mesh map (applied to the mesh on the fly)
    got = pr.findProjections(pts, refXf=shear)
    ref = o.find_projections(pts, refXf=shear)
    _check(v, f, got, ref, pts, mesh_v=mapped(shear, v))


def test_projection_limits_and_edges(M):
    v, f = mg.noisy_icosphere(seed=6, level=3)
    pts = _points(v, 2000, 5)
    o = O.Oracle(v, f)
    pr = M.PointsToMeshProjector()
    pr.updateMeshData(v, f)
    full = o.find_projections(pts)
    up = float(np.quantile(full["distSq"], 0.5))
    got = pr.findProjections(pts, upDistLimitSq=up)
    inside = full["distSq"] < up * (1 - 1e-5)
    outside = full["distSq"] >= up * (1 + 1e-5)
    assert (got["face"][inside] >= 0).all()
    assert (got["face"][outside] == -1).all() and (got["distSq"][outside] == np.float32(up)).all()
    # early exit: any triangle within sqrt(lo) will do
    lo = float(np.quantile(full["distSq"], 0.3))
    got = pr.findProjections(pts, loDistLimitSq=lo)
    near = full["distSq"] <= lo
    assert (got["distSq"][near] <= lo * (1 + 1e-5)).all()
    assert np.allclose(got["distSq"][~near], full["distSq"][~near], rtol=1e-4, atol=1e-8)
    # empty input and a missing mesh
    assert len(pr.findProjections(np.zeros((0, 3), np.float32))) == 0
    with pytest.raises(M.FwnError):
        M.PointsToMeshProjector().findProjections(pts)
    assert pr.projectionsHeapBytes(1000) >= 1000 * 44


def test_projection_vs_mrcuda(M):
    """Against the reference's own GPU projector kernel (FP32 projection, -use_fast_math)."""
    from oracle import mrcuda
    if not mrcuda.kernels_present():
        pytest.skip("reference kernels not built here")
    v, f = mg.noisy_icosphere(seed=3, level=4)
    pts = _points(v, 6000, 7)
    o = O.Oracle(v, f)
    rk = mrcuda.RefKernels(v, f, o.nodes(), o.dipoles(0))
    raw = rk.project(pts).cpu().numpy()
    import meshlib_gb300
    ref = raw.view(meshlib_gb300.PROJECTION_DTYPE)
    pr = M.PointsToMeshProjector()
    pr.updateMeshData(v, f)
    got = pr.findProjections(pts)
    _check(v, f, got, ref, pts)


def test_projection_many_points_seeded(M):
    """10 M Morton-ordered points (enough for two tiles per work item): warps walk consecutive tiles
    and seed each lane's search with its previous point's triangle; sampled results match the oracle,
    with and without an upper distance limit (a seed beyond the limit must not leak into the output)."""
    import torch

    v, f = mg.noisy_icosphere(seed=7, level=5)
    rng = np.random.default_rng(11)
    lo, hi = v.min(0), v.max(0)
    pts = rng.uniform(lo - 0.3 * (hi - lo), hi + 0.3 * (hi - lo), (10_000_000, 3)).astype(np.float32)
    g = M.FastWindingNumber(v, f)
    pr = M.PointsToMeshProjector.from_mesh(g)
    o = O.Oracle(v, f)
    sidx = rng.integers(0, len(pts), 20000)
    full = o.find_projections(pts[sidx])
    up = float(np.quantile(full["distSq"], 0.4))
    for limit in (None, up):
        got = pr.findProjections(pts) if limit is None else pr.findProjections(pts, upDistLimitSq=limit)
        ref = full if limit is None else o.find_projections(pts[sidx], upDistLimitSq=limit)
        g_s = got[sidx]
        if limit is not None:
            clear_in = ref["distSq"] < limit * (1 - 1e-5)
            clear_out = ref["distSq"] >= limit * (1 + 1e-5)
            assert (g_s["face"][clear_in] >= 0).all() and (g_s["face"][clear_out] == -1).all()
            keep = clear_in | clear_out
            g_s, ref = g_s[keep], ref[keep]
        _check(v, f, g_s, ref, pts[sidx] if limit is None else pts[sidx][keep])
    # signed distances at the same points through the seeded vector path
    d = torch.from_numpy(pts).cuda()
    out = torch.empty(len(pts), device="cuda")
    g.calcWithDistances_dev(d.data_ptr(), len(pts), out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    dd = out.cpu().numpy()[sidx]
    ref_d = o.vector_with_distances(pts[sidx], prec=1)
    assert np.abs(np.abs(dd) - np.abs(ref_d)).max() <= 1e-5 * mg.diag(v)
