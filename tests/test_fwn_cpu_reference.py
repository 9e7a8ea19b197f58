"""The oracle (CPU, bit for bit) and the library (GPU, at the parity bars) against MeshLib's own CPU
winding-number / signed-distance code.

tests/golden/fwn_cpu_reference.npz holds outputs of the reference's MRMesh/MRFastWindingNumber.cpp
with its AABB tree, dipoles and findProjection, compiled from the reference sources
(oracle/ref/build_cpu_ref.py) and run by tests/golden/make_fwn_cpu_golden.py: the tree and dipoles,
signed-distance grids (unbanded and banded), a winding-number grid, winding numbers and projections
at points of the 16,384-triangle torus; self-intersection bits of two overlapping spheres; and 2,048
voxels of the 512^3 grid, winding numbers and projections at 1,024 shell points of the
1,310,720-triangle icosphere.  The oracle restates that code in the same FP32 operations without
FMA contraction, so it must reproduce every float.  The library computes with compensated sums and
FP64 near-degenerate fallbacks, so it is held to the parity bars: distances within 1e-5 x diagonal,
signs / bits exact except within TAU of the threshold (decided by the FP64 oracle), winding numbers
within WN_TOL.  Reference: MRMesh/MRFastWindingNumber.cpp:28-94, MRMesh/MRDipole.cpp:11-128,
MRMesh/MRAABBTreeMaker.hpp:51-165, MRMesh/MRMeshProject.cpp:13-104."""
import os
import sys

import numpy as np
import pytest

import oracle as O
import oracle.fwnref as FR
from meshlib_gb300 import meshgen as mg

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_fwn_cpu_golden as G  # noqa: E402

TAU = 1e-3
WN_TOL = 2e-4


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "fwn_cpu_reference.npz"))


@pytest.fixture(scope="module")
def torus(gold):
    v, f, dims, xf, pts = G.torus_inputs()
    assert str(gold["digest_torus"]) == G.digest(v, f, pts), "mesh generator changed: regenerate the fixture"
    return v, f, dims, xf, pts


@pytest.fixture(scope="module")
def ico(gold):
    v, f, dims, xf = G.ico_inputs()
    assert str(gold["digest_ico"]) == G.digest(v, f), "mesh generator changed: regenerate the fixture"
    return v, f, dims, xf


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _band(diag):
    return dict(minDistSq=(0.01 * diag) ** 2, maxDistSq=(0.05 * diag) ** 2)


def test_oracle_bit_identical_torus(gold, torus):
    v, f, dims, xf, pts = torus
    o = O.Oracle(v, f)
    diag = mg.diag(v)
    assert G.digest(o.nodes()) == str(gold["torus_nodes_digest"])
    assert G.digest(o.dipoles(0).astype(np.float32)) == str(gold["torus_dipoles_digest"])
    assert np.array_equal(_bits(o.from_grid_with_distances(dims, xf, prec=0)), _bits(gold["torus_sdf"]))
    band = o.from_grid_with_distances(dims, xf, O.make_options(**_band(diag)), prec=0)
    assert np.isnan(gold["torus_sdf_band"]).any() and np.isfinite(gold["torus_sdf_band"]).any()
    assert np.array_equal(_bits(band), _bits(gold["torus_sdf_band"]))
    assert np.array_equal(_bits(o.from_grid(dims, xf, prec=0)), _bits(gold["torus_fwn"]))
    assert np.array_equal(_bits(o.from_vector(pts, skip_face=11, prec=0)), _bits(gold["torus_fwn_pts"]))
    assert np.array_equal(_bits(o.dist_sq(pts)), _bits(gold["torus_proj_dsq"]))


def test_oracle_bit_identical_self_intersections(gold):
    sv, sf = G.spheres_inputs()
    assert str(gold["digest_spheres"]) == G.digest(sv, sf)
    bits, _ = O.Oracle(sv, sf).self_intersections(prec=0)
    assert gold["spheres_selfint"].sum() > 0
    assert np.array_equal(bits, gold["spheres_selfint"].astype(bool))


def test_oracle_bit_identical_icosphere(gold, ico):
    v, f, dims, xf = ico
    o = O.Oracle(v, f)
    assert G.digest(o.nodes()) == str(gold["ico_nodes_digest"])
    assert G.digest(o.dipoles(0).astype(np.float32)) == str(gold["ico_dipoles_digest"])
    d, _ = o.grid_voxels(dims, xf, gold["ico_ids"], prec=0)
    assert np.array_equal(_bits(d), _bits(gold["ico_sdf"]))
    assert np.array_equal(_bits(o.from_vector(gold["ico_pts"], prec=0)), _bits(gold["ico_fwn_pts"]))
    assert np.array_equal(_bits(o.dist_sq(gold["ico_pts"])), _bits(gold["ico_proj_dsq"]))


@pytest.mark.skipif(not FR.available(), reason="the reference library is built only where a copy of the reference is")
def test_fixture_rederived_from_reference(gold, torus):
    v, f, dims, xf, pts = torus
    R = FR.Reference(v, f)
    assert np.array_equal(_bits(R.from_grid_with_distances(dims, xf)), _bits(gold["torus_sdf"]))
    assert np.array_equal(_bits(R.from_vector(pts, skip_face=11)), _bits(gold["torus_fwn_pts"]))
    assert np.array_equal(R.project(pts)[1], gold["torus_proj_face"])


# ------------------------------------------------------------------------------- the library (GPU)

def _check_signed(d, d_ref, sign_wn, diag, band=None):
    """d: ours; d_ref: the reference's; sign_wn(idx) -> FP64 winding numbers deciding sign disagreements.
    With a band, a voxel may be kept by one side and dropped by the other only at the band's edges."""
    fin, fin_ref = np.isfinite(d), np.isfinite(d_ref)
    flip = np.flatnonzero(fin != fin_ref)
    if len(flip):
        assert band is not None, f"NaN pattern differs at {len(flip)} places"
        dist = np.where(fin[flip], np.abs(d[flip]), np.abs(d_ref[flip]))
        edge = np.minimum(np.abs(dist - np.sqrt(band["minDistSq"])), np.abs(dist - np.sqrt(band["maxDistSq"])))
        assert (edge <= 1e-5 * diag).all(), f"{int((edge > 1e-5 * diag).sum())} voxels in / out of the band away from its edges"
    fin = fin & fin_ref
    err = np.abs(np.abs(d[fin]) - np.abs(d_ref[fin]))
    assert err.max() <= 1e-5 * diag, f"max |d - d_ref| {err.max():.3e}"
    mism = np.flatnonzero((np.signbit(d) != np.signbit(d_ref)) & fin)
    if len(mism):
        wn = sign_wn(mism)
        assert (np.abs(wn - 0.5) < TAU).all(), f"{int((np.abs(wn - 0.5) >= TAU).sum())} sign mismatches"


@pytest.mark.gpu
def test_library_matches_cpu_reference_torus(gold, torus, fwn_lib):
    import meshlib_gb300 as M
    v, f, dims, xf, pts = torus
    diag = mg.diag(v)
    o = O.Oracle(v, f)
    gp = O.grid_points(dims, xf)
    for precise in (False, True):
        g = M.FastWindingNumber(v, f, precise=precise)
        nodes, dip = g.tree()
        assert G.digest(nodes) == str(gold["torus_nodes_digest"]), "tree differs from the reference's"
        assert G.digest(np.ascontiguousarray(dip, np.float32)) == str(gold["torus_dipoles_digest"])
        _check_signed(g.calcFromGridWithDistances(dims, xf), gold["torus_sdf"], lambda i: o.exact_wn(gp[i]), diag)
        band = g.calcFromGridWithDistances(dims, xf, M.DistanceToMeshOptions(**_band(diag)))
        _check_signed(band, gold["torus_sdf_band"], lambda i: o.exact_wn(gp[i]), diag, _band(diag))
        assert np.abs(g.calcFromGrid(dims, xf) - gold["torus_fwn"]).max() <= WN_TOL
        assert np.abs(g.calcFromVector(pts, skipFace=11) - gold["torus_fwn_pts"]).max() <= WN_TOL
        pr = M.PointsToMeshProjector.from_mesh(g).findProjections(pts)
        dd = np.abs(np.sqrt(pr["distSq"].astype(np.float64)) - np.sqrt(gold["torus_proj_dsq"].astype(np.float64)))
        assert dd.max() <= 1e-5 * diag
        # a different face is a tie at the same closest point (a shared vertex or edge) but for queries
        # equidistant from two parts of the surface within FP32 precision
        diff = pr["face"] != gold["torus_proj_face"]
        moved = np.abs(pr["point"][diff] - gold["torus_proj_point"][diff]).max(1) > 1e-5 * diag
        assert moved.sum() <= max(2, len(pts) // 500)


@pytest.mark.gpu
def test_library_matches_cpu_reference_self_intersections(gold, fwn_lib):
    import meshlib_gb300 as M
    sv, sf = G.spheres_inputs()
    _, wn64 = O.Oracle(sv, sf).self_intersections(prec=1)
    ref = gold["spheres_selfint"].astype(bool)
    for precise in (False, True):
        bits = M.FastWindingNumber(sv, sf, precise=precise).calcSelfIntersections()
        diff = np.flatnonzero(bits != ref)
        assert ((np.abs(wn64[diff]) < TAU) | (np.abs(wn64[diff] - 1) < TAU)).all()


@pytest.mark.gpu
def test_library_matches_cpu_reference_icosphere(gold, ico, fwn_lib):
    import torch

    import meshlib_gb300 as M
    v, f, dims, xf = ico
    diag = mg.diag(v)
    o = O.Oracle(v, f)
    g = M.FastWindingNumber(v, f)
    nodes, dip = g.tree()
    assert G.digest(nodes) == str(gold["ico_nodes_digest"]), "tree differs from the reference's"
    assert G.digest(np.ascontiguousarray(dip, np.float32)) == str(gold["ico_dipoles_digest"])
    out = torch.empty(int(np.prod(dims)), device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    ids = gold["ico_ids"]
    d = out[torch.from_numpy(ids).cuda()].cpu().numpy()
    del out
    _check_signed(d, gold["ico_sdf"], lambda i: o.grid_voxels(dims, xf, ids[i], prec=1)[1], diag)
    pts = gold["ico_pts"]
    wn = g.calcFromVector(pts)
    assert np.abs(wn - gold["ico_fwn_pts"]).max() <= WN_TOL
    pr = M.PointsToMeshProjector.from_mesh(g).findProjections(pts)
    dd = np.abs(np.sqrt(pr["distSq"].astype(np.float64)) - np.sqrt(gold["ico_proj_dsq"].astype(np.float64)))
    assert dd.max() <= 1e-5 * diag
