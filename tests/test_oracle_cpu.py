"""CPU-only checks of the oracle against the reference's own known answers, and oracle self-consistency.

Known answers restated from the reference's tests:
  * MRTest/MRDipoleTests.cpp:25-51 -- triangle solid angle: -2pi / +2pi just above / below the
    centroid (tolerance 1e-3), exactly 0 at the vertices and at in-plane exterior points;
  * MRTest/MRAABBTreeTests.cpp:10-27 -- 2n-1 nodes, root box = mesh bounding box expanded by one
    ulp each way (Box::insignificantlyExpanded), both root children valid, a 1-face tree has 1 node.
"""
import math

import numpy as np

import oracle as O
from meshlib_gb300 import meshgen as mg

TRI = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)


def test_solid_angle_known_answers():
    c = TRI.mean(0)
    above = O.solid_angle_f(c + np.float32([0, 0, 1e-5]), TRI)
    below = O.solid_angle_f(c - np.float32([0, 0, 1e-5]), TRI)
    assert abs(above - (-2 * math.pi)) < 1e-3
    assert abs(below - (2 * math.pi)) < 1e-3
    for i in range(3):
        assert O.solid_angle_f(TRI[i], TRI) == 0.0
    assert O.solid_angle_f(TRI[1] + TRI[2], TRI) == 0.0
    assert O.solid_angle_f(-TRI[1], TRI) == 0.0
    assert O.solid_angle_f(-TRI[2], TRI) == 0.0
    # FP64 oracle agrees
    assert abs(O.solid_angle_d(c.astype(np.float64) + [0, 0, 1e-5], TRI.astype(np.float64)) + 2 * math.pi) < 1e-3


def test_tree_known_answers():
    v, f = mg.noisy_torus(seed=4, nu=16, nv=8)
    o = O.Oracle(v, f)
    nodes = o.nodes()
    assert len(nodes) == 2 * len(f) - 1
    lo = np.nextafter(v.min(0), np.float32(-np.inf))
    hi = np.nextafter(v.max(0), np.float32(np.inf))
    assert np.array_equal(nodes[0]["min"], lo) and np.array_equal(nodes[0]["max"], hi)
    assert nodes[0]["l"] == 1 and nodes[0]["r"] > 1
    one = O.Oracle(v, f[:1])
    assert len(one.nodes()) == 1 and one.nodes()[0]["r"] < 0


def test_tree_structure_invariants():
    v, f = mg.noisy_icosphere(seed=2, level=3)
    nodes = O.Oracle(v, f).nodes()
    leaves = nodes[nodes["r"] < 0]
    assert sorted(leaves["l"].tolist()) == list(range(len(f)))
    internal = np.nonzero(nodes["r"] >= 0)[0]
    for i in internal:
        l, r = nodes[i]["l"], nodes[i]["r"]
        assert l == i + 1
        for c in (l, r):
            assert (nodes[c]["min"] >= nodes[i]["min"]).all() and (nodes[c]["max"] <= nodes[i]["max"]).all()


def test_dipole_sums():
    v, f = mg.noisy_torus(seed=1)
    o = O.Oracle(v, f)
    d = o.dipoles(1)
    a, b, c = (v[f[:, k]].astype(np.float64) for k in range(3))
    da = 0.5 * np.cross(b - a, c - a)
    assert abs(d[0, 3] - np.linalg.norm(da, axis=1).sum()) < 1e-9 * d[0, 3]
    assert np.allclose(d[0, 4:7], da.sum(0), atol=1e-9)
    df = o.dipoles(0)
    assert np.allclose(df[:, :7], d[:, :7], rtol=1e-4, atol=1e-5)


def test_fwn_closed_mesh_far_field():
    v, f = mg.noisy_torus(seed=0)
    o = O.Oracle(v, f)
    pts = np.array([[1.0, 0, 0], [-1, 0, 0], [0, 1, 0], [0, 0, 0], [3, 0, 0], [0, 0, 2]], np.float32)
    ex = o.exact_wn(pts)
    assert np.allclose(ex, [1, 1, 1, 0, 0, 0], atol=1e-9)
    w = o.from_vector(pts, prec=1)
    assert np.abs(w - ex).max() < 0.1  # beta=2 dipole approximation
    w32 = o.from_vector(pts, prec=0)
    assert np.abs(w32 - w).max() < 1e-5


def test_fp32_vs_fp64_grid():
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 16)
    o = O.Oracle(v, f)
    d32 = o.from_grid_with_distances(dims, xf, prec=0)
    d64 = o.from_grid_with_distances(dims, xf, prec=1)
    assert np.abs(d32 - d64).max() < 1e-6
    g32 = o.from_grid(dims, xf, prec=0)
    g64 = o.from_grid(dims, xf, prec=1)
    assert np.abs(g32 - g64).max() < 1e-5


def test_distance_is_brute_force_min():
    v, f = mg.noisy_icosphere(seed=1, level=2)
    o = O.Oracle(v, f)
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1.5, 1.5, (50, 3)).astype(np.float32)
    dsq = o.dist_sq(pts)
    brute = np.empty(len(pts))
    for i, p in enumerate(pts.astype(np.float64)):
        best = np.inf
        for t in f:
            q = np.empty(3)
            O.lib().orc_closest_point_d(p.ctypes.data, np.ascontiguousarray(v[t].astype(np.float64)).ctypes.data, q.ctypes.data)
            best = min(best, float(((q - p) ** 2).sum()))
        brute[i] = best
    assert np.allclose(dsq, brute, rtol=1e-5, atol=1e-9)


def test_grid_points_convention():
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 8)
    p = O.grid_points(dims, xf)
    assert p.shape == (512, 3)
    assert np.allclose(p[0], xf[9:12]) and np.allclose(p[1] - p[0], [xf[0], 0, 0])


def test_self_intersections_known():
    v, f = mg.figure8_torus()
    bits, wn = O.Oracle(v, f).self_intersections()
    assert bits.any() and not bits.all()
    v2, f2 = mg.noisy_torus(seed=0)
    b2, _ = O.Oracle(v2, f2).self_intersections()
    assert not b2.any()


def test_traversal_counts():
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 8)
    o = O.Oracle(v, f)
    c = o.traversal_counts(O.grid_points(dims, xf))
    assert all(int(x) > 0 for x in c)


def test_mlp_oracle_gradients_finite_differences(monkeypatch):
    """The surrogate's CPU oracle: analytic gradients equal central finite differences (bf16
    rounding switched off so the loss is smooth)."""
    import math

    from oracle import mlp_oracle as MO
    monkeypatch.setattr(MO, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(0)
    p = np.concatenate([rng.normal(0, 0.1, int(np.prod(s))) for _, s in MO.SIZES])
    m = np.zeros(40)
    m[3] = 1
    m[4:36] = [math.pi * 2 ** (k / 5) for k in range(32)]
    m[36] = 10
    pts = rng.uniform(-1, 1, (64, 3)).astype(np.float32)
    t = rng.normal(0, 0.3, 64)
    _, g = MO.loss_and_grads(p, m, pts, t)
    for idx in [5, 24600, 41100, 57700, 74200, 74368, 30000, 24577]:
        e = np.zeros_like(p)
        e[idx] = 1e-6
        fd = (MO.loss_and_grads(p + e, m, pts, t)[0] - MO.loss_and_grads(p - e, m, pts, t)[0]) / 2e-6
        assert abs(g[idx] - fd) <= 1e-6 + 1e-5 * abs(fd), (idx, g[idx], fd)


def _brute_dist2(v, f, p):
    """FP64 squared distance from p to every face (the reference's closestPointInTriangle)."""
    out = np.empty(len(f))
    pd = np.ascontiguousarray(p, np.float64)
    for k, t in enumerate(f):
        q = np.empty(3)
        O.lib().orc_closest_point_d(pd.ctypes.data, np.ascontiguousarray(v[t].astype(np.float64)).ctypes.data, q.ctypes.data)
        out[k] = float(((q - pd) ** 2).sum())
    return out


def test_projection_known_answers():
    """One triangle: a point above the interior projects straight down with its barycentrics; a point
    beyond a vertex lands on it (bary (1, 0) for the second vertex)."""
    o = O.Oracle(TRI, np.array([[0, 1, 2]], np.int32))
    r = o.find_projections(np.array([[0.25, 0.25, 2.0], [3.0, -1.0, 0.0]], np.float32))
    assert r["face"].tolist() == [0, 0] and r["edge"].tolist() == [-1, -1]
    assert np.allclose(r["point"][0], [0.25, 0.25, 0]) and np.allclose(r["bary"][0], [0.25, 0.25])
    assert r["distSq"][0] == np.float32(4.0)
    assert np.array_equal(r["point"][1], [1, 0, 0]) and np.array_equal(r["bary"][1], [1, 0])
    assert r["distSq"][1] == np.float32(5.0)
    # nothing closer than the upper limit: face -1 and distSq = the limit
    r = o.find_projections(np.array([[0.25, 0.25, 2.0]], np.float32), upDistLimitSq=1.0)
    assert r["face"][0] == -1 and r["distSq"][0] == np.float32(1.0)


def test_projection_brute_force_and_transforms():
    v, f = mg.noisy_icosphere(seed=1, level=2)
    o = O.Oracle(v, f)
    rng = np.random.default_rng(3)
    pts = rng.uniform(-1.5, 1.5, (40, 3)).astype(np.float32)
    r = o.find_projections(pts)
    for i, p in enumerate(pts):
        d = _brute_dist2(v, f, p)
        assert abs(float(r["distSq"][i]) - d.min()) <= 1e-5 * d.min() + 1e-9
        assert abs(d[r["face"][i]] - d.min()) <= 1e-9 * max(1.0, d.min())
        a, b = r["bary"][i]
        tri = v[f[r["face"][i]]].astype(np.float64)
        assert np.allclose((1 - a - b) * tri[0] + a * tri[1] + b * tri[2], r["point"][i], atol=1e-5)
    # a rigid mesh map folds into the points: projecting through refXf = projecting the mapped-back points
    c, s = math.cos(0.7), math.sin(0.7)
    rot = np.array([c, -s, 0, s, c, 0, 0, 0, 1, 0.3, -0.2, 0.5], np.float32)
    assert O.is_rigid(rot)
    r_rot = o.find_projections(pts, refXf=rot)
    A, b = rot[:9].reshape(3, 3).astype(np.float64), rot[9:].astype(np.float64)
    back = ((pts.astype(np.float64) - b) @ A).astype(np.float32)  # A^-1 = A^T
    r_back = o.find_projections(back)
    assert np.allclose(r_rot["distSq"], r_back["distSq"], rtol=1e-4, atol=1e-7)
    # a non-rigid mesh map is applied to the mesh: same as projecting onto the mapped mesh
    sc = np.array([1.3, 0.2, 0, 0, 0.8, 0, 0, 0, 1.1, 0.1, 0, 0], np.float32)
    assert not O.is_rigid(sc)
    r_sc = o.find_projections(pts, refXf=sc)
    vm = (v.astype(np.float64) @ sc[:9].reshape(3, 3).T.astype(np.float64) + sc[9:]).astype(np.float32)
    r_m = O.Oracle(vm, f).find_projections(pts)
    assert np.allclose(r_sc["distSq"], r_m["distSq"], rtol=1e-4, atol=1e-7)
    assert (r_sc["face"] == r_m["face"]).mean() > 0.9


def test_refit_keeps_topology_and_bounds():
    """AABBTree::refit (MRAABBTree.cpp:62-94): same topology, every leaf box holds its moved face
    (one ulp wider), every internal box is the union of its children, distances equal a rebuild's."""
    v, f = mg.noisy_icosphere(seed=4, level=3)
    o = O.Oracle(v, f)
    before = o.nodes().copy()
    rng = np.random.default_rng(2)
    moved = rng.random(len(v)) < 0.3
    v2 = v.copy()
    v2[moved] += rng.normal(scale=0.05, size=(int(moved.sum()), 3)).astype(np.float32)
    o.refit(v2, moved)
    after = o.nodes()
    assert np.array_equal(after["l"], before["l"]) and np.array_equal(after["r"], before["r"])
    leaf = after["r"] < 0
    tri = v2[f[after["l"][leaf]]]
    assert (after["min"][leaf] < tri.min(1)).all() and (after["max"][leaf] > tri.max(1)).all()
    inner = np.flatnonzero(~leaf)
    l, r = after["l"][inner], after["r"][inner]
    assert np.array_equal(after["min"][inner], np.minimum(after["min"][l], after["min"][r]))
    assert np.array_equal(after["max"][inner], np.maximum(after["max"][l], after["max"][r]))
    # untouched faces keep their boxes
    touched = moved[f[after["l"][leaf]]].any(1)
    assert np.array_equal(after["min"][leaf][~touched], before["min"][leaf][~touched])
    pts = rng.uniform(-1.4, 1.4, (200, 3)).astype(np.float32)
    assert np.allclose(o.dist_sq(pts), O.Oracle(v2, f).dist_sq(pts), rtol=1e-6, atol=1e-9)
