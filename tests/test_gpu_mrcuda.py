"""The library and the oracle against the reference's own GPU kernels (MRCuda), on the same GPU.

The reference kernels (MRCuda/MRCudaFastWindingNumber.cu) are built from the reference sources into
oracle/_ref/ and fed the reference's CPU-built tree and FP32 dipoles, as the reference's host class
does.  They compute in FP32 with -use_fast_math (fast atan2, FP32 leaf projection), so:
  * distances: |d - d_mrcuda| <= 1e-5 * bbox diagonal (the contract's tolerance);
  * inside/outside signs and self-intersection bits: exact, except where the FP64 oracle's winding
    number lies within TAU of the threshold (counted, not failed);
  * winding numbers: |w - w_mrcuda| <= MRCUDA_WN_TOL (fast-math atan2 and division differ from
    atan2f and IEEE division by a few ulps per term).
The same checks pin the CPU oracle itself to the reference's code run here.
"""
import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

TAU = 1e-3
MRCUDA_WN_TOL = 2e-4


def _mrcuda():
    from oracle import mrcuda
    if not mrcuda.kernels_present():
        pytest.skip("reference kernels not built here (oracle/ref/build_ref.py needs the reference sources)")
    return mrcuda


@pytest.fixture(scope="module")
def fwncls(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300.FastWindingNumber


def _ref(v, f):
    mrcuda = _mrcuda()
    o = O.Oracle(v, f)
    return o, mrcuda.RefKernels(v, f, o.nodes(), o.dipoles(0))


def _sign_counts(d, d_ref, wn_fp64, thr=0.5):
    both = np.isfinite(d) & np.isfinite(d_ref)
    mism = both & (np.signbit(d) != np.signbit(d_ref))
    near = np.abs(wn_fp64 - thr) < TAU
    return int((mism & ~near).sum()), int((mism & near).sum())


@pytest.mark.parametrize("precise", [False, True])
def test_signed_distance_torus_64_vs_mrcuda(fwncls, precise):
    """The CPU-runnable configuration: noisy torus, 16,384 triangles, 64^3 over the bbox + 10 %."""
    v, f = mg.noisy_torus(seed=0)
    assert len(f) == 16384
    dims, xf = mg.grid_for(v, 64)
    o, rk = _ref(v, f)
    d_ref = rk.signed_distance(dims, xf).cpu().numpy()
    d = fwncls(v, f, precise=precise).calcFromGridWithDistances(dims, xf)
    diag = mg.diag(v)
    assert np.isfinite(d_ref).all() and np.isfinite(d).all()
    err = np.abs(np.abs(d) - np.abs(d_ref))
    assert err.max() <= 1e-5 * diag, f"max |d - d_mrcuda| {err.max()} > {1e-5 * diag}"
    pts = O.grid_points(dims, xf)
    sel = np.flatnonzero(np.signbit(d) != np.signbit(d_ref))
    wn64 = np.full(len(d), 0.0)
    if len(sel):
        wn64[sel] = o.exact_wn(pts[sel])
    bad, near = _sign_counts(d, d_ref, wn64)
    assert bad == 0, f"{bad} sign mismatches vs MRCuda away from the threshold ({near} near it)"


def test_oracle_pinned_to_mrcuda_signed_distance():
    """The CPU oracle (FP32 reference arithmetic) against the reference's GPU kernel."""
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 24)
    o, rk = _ref(v, f)
    d_ref = rk.signed_distance(dims, xf).cpu().numpy()
    d_orc = o.from_grid_with_distances(dims, xf, prec=0)
    diag = mg.diag(v)
    assert np.abs(np.abs(d_orc) - np.abs(d_ref)).max() <= 1e-5 * diag
    sel = np.flatnonzero(np.signbit(d_orc) != np.signbit(d_ref))
    wn64 = np.zeros(len(d_orc))
    if len(sel):
        wn64[sel] = o.exact_wn(O.grid_points(dims, xf)[sel])
    bad, _ = _sign_counts(d_orc, d_ref, wn64)
    assert bad == 0


def test_banded_signed_distance_vs_mrcuda(fwncls):
    """The reference's banded request (NaN outside [minDistSq, maxDistSq)) on a 5k-triangle sphere."""
    from meshlib_gb300 import DistanceToMeshOptions
    v, f = mg.noisy_icosphere(seed=3, level=4)
    dims, xf = mg.grid_for(v, 48)
    band = 0.05 * mg.diag(v)
    o, rk = _ref(v, f)
    d_ref = rk.signed_distance(dims, xf, maxDistSq=band * band).cpu().numpy()
    d = fwncls(v, f).calcFromGridWithDistances(dims, xf, DistanceToMeshOptions(maxDistSq=band * band))
    fin, fin_ref = np.isfinite(d), np.isfinite(d_ref)
    # a voxel whose distance is within a rounding step of the band edge may fall on either side
    edge = np.abs(np.where(fin, np.abs(d), np.where(fin_ref, np.abs(d_ref), 0)) - band) <= 1e-5 * mg.diag(v)
    assert ((fin != fin_ref) & ~edge).sum() == 0
    both = fin & fin_ref
    assert np.abs(np.abs(d[both]) - np.abs(d_ref[both])).max() <= 1e-5 * mg.diag(v)


def test_winding_numbers_vs_mrcuda(fwncls):
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 32)
    o, rk = _ref(v, f)
    w_ref = rk.from_grid(dims, xf).cpu().numpy()
    w = fwncls(v, f, precise=False).calcFromGrid(dims, xf)
    assert np.abs(w - w_ref).max() <= MRCUDA_WN_TOL
    # the oracle (FP32, reference arithmetic) too
    w_orc = o.from_grid(dims, xf, prec=0)
    assert np.abs(w_orc - w_ref).max() <= MRCUDA_WN_TOL
    # points with a skipped face
    rng = np.random.default_rng(7)
    pts = (rng.random((4096, 3)) * 2.6 - 1.3).astype(np.float32)
    pts[:, 2] *= 0.4
    assert np.abs(fwncls(v, f, precise=False).calcFromVector(pts, skipFace=11) - rk.from_vector(pts, skip_face=11).cpu().numpy()).max() <= MRCUDA_WN_TOL


def test_self_intersections_vs_mrcuda(fwncls):
    """Face bits (wn < 0 or wn > 1 at the centroid, that face skipped) on overlapping spheres."""
    v, f = mg.overlapping_spheres(seed=0, level=5)
    o, rk = _ref(v, f)
    wn_ref = rk.from_mesh().cpu().numpy()
    bits_ref = (wn_ref < 0) | (wn_ref > 1)
    bits = fwncls(v, f, precise=False).calcSelfIntersections()
    assert bits.shape == bits_ref.shape
    diff = np.flatnonzero(bits != bits_ref)
    if len(diff):
        _, wn64 = o.self_intersections(prec=1)
        near = (np.abs(wn64[diff]) < TAU) | (np.abs(wn64[diff] - 1) < TAU)
        assert near.all(), f"{int((~near).sum())} face bits differ from MRCuda away from 0 and 1"
    assert bits_ref.sum() > 0
