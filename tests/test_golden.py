"""The oracle (CPU) and the library (GPU) against golden outputs of the reference's own GPU kernels.

tests/golden/mrcuda_small.npz holds outputs of MRCuda/MRCudaFastWindingNumber.cu and
MRCuda/MRCudaPointsToMeshProjector.cu (built from the reference sources, run on a GB300 by
tests/golden/make_golden.py) on seeded inputs that the tests regenerate.  The reference kernels compute
in FP32 with -use_fast_math, so the bars are those of tests/test_gpu_mrcuda.py: distances within
1e-5 x bbox diagonal, winding numbers within 2e-4, signs / bits exact except within TAU of the
threshold (decided with the unapproximated FP64 winding number), projection faces equal except exact
ties at the same closest point.
"""
import os
import sys

import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

TAU = 1e-3
WN_TOL = 2e-4


@pytest.fixture(scope="module")
def gold():
    d = np.load(os.path.join(HERE, "golden", "mrcuda_small.npz"))
    v, f, dims, xf, pts, sv, sf = make_golden.inputs()
    assert str(d["digest_torus"]) == make_golden.digest(v, f), "mesh generator changed: regenerate the fixture"
    assert str(d["digest_spheres"]) == make_golden.digest(sv, sf)
    assert np.array_equal(d["pts"], pts) and np.array_equal(d["xf"], xf)
    return d, (v, f, dims, xf, pts, sv, sf)


def _check_sdf(got, ref, o, dims, xf, diag):
    assert np.abs(np.abs(got) - np.abs(ref)).max() <= 1e-5 * diag
    mism = np.flatnonzero(np.signbit(got) != np.signbit(ref))
    if len(mism):
        wn = o.exact_wn(O.grid_points(dims, xf)[mism])
        assert (np.abs(wn - 0.5) < TAU).all(), f"{int((np.abs(wn - 0.5) >= TAU).sum())} sign mismatches"


def _check_bits(wn_got, wn_ref, wn_exact):
    b_got, b_ref = (wn_got < 0) | (wn_got > 1), (wn_ref < 0) | (wn_ref > 1)
    diff = np.flatnonzero(b_got != b_ref)
    near = (np.abs(wn_exact[diff]) < TAU) | (np.abs(wn_exact[diff] - 1) < TAU)
    assert near.all()
    assert b_ref.sum() > 0


def _check_proj(got, ref, v, f, diag):
    dt = np.dtype([("face", np.int32), ("point", np.float32, 3), ("edge", np.int32), ("bary", np.float32, 2),
                   ("distSq", np.float32)])
    ref = np.ascontiguousarray(ref).view(dt)
    assert np.array_equal(got["face"] >= 0, ref["face"] >= 0)
    assert np.abs(np.sqrt(got["distSq"].astype(np.float64)) - np.sqrt(ref["distSq"].astype(np.float64))).max() <= 1e-5 * diag
    # a different face is a tie: almost always at the same closest point (a shared vertex or edge);
    # a different point means a query equidistant from two parts of the surface within FP32 precision
    diff = got["face"] != ref["face"]
    moved = np.abs(got["point"][diff] - ref["point"][diff]).max(1) > 1e-5 * diag
    assert moved.sum() <= max(2, len(got) // 500)


def test_oracle_matches_reference_golden(gold):
    d, (v, f, dims, xf, pts, sv, sf) = gold
    o = O.Oracle(v, f)
    diag = mg.diag(v)
    _check_sdf(o.from_grid_with_distances(dims, xf, prec=0), d["sdf_grid"], o, dims, xf, diag)
    assert np.abs(o.from_grid(dims, xf, prec=0) - d["fwn_grid"]).max() <= WN_TOL
    assert np.abs(o.from_vector(pts, skip_face=11, prec=0) - d["fwn_pts"]).max() <= WN_TOL
    os_ = O.Oracle(sv, sf)
    _, wn = os_.self_intersections(prec=0)
    _, wn64 = os_.self_intersections(prec=1)
    _check_bits(wn, d["selfint_wn"], wn64)
    _check_proj(o.find_projections(pts), d["proj"], v, f, diag)


@pytest.mark.gpu
def test_library_matches_reference_golden(gold, fwn_lib):
    import meshlib_gb300 as M
    d, (v, f, dims, xf, pts, sv, sf) = gold
    o = O.Oracle(v, f)
    diag = mg.diag(v)
    for precise in (False, True):
        g = M.FastWindingNumber(v, f, precise=precise)
        _check_sdf(g.calcFromGridWithDistances(dims, xf), d["sdf_grid"], o, dims, xf, diag)
        assert np.abs(g.calcFromGrid(dims, xf) - d["fwn_grid"]).max() <= WN_TOL
        assert np.abs(g.calcFromVector(pts, skipFace=11) - d["fwn_pts"]).max() <= WN_TOL
        _check_proj(M.PointsToMeshProjector.from_mesh(g).findProjections(pts), d["proj"], v, f, diag)
        gs = M.FastWindingNumber(sv, sf, precise=precise)
        _, wn = gs.calcSelfIntersections(with_wn=True)
        _, wn64 = O.Oracle(sv, sf).self_intersections(prec=1)
        _check_bits(wn, d["selfint_wn"], wn64)
