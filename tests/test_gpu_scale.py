"""Parity at the benchmark's own sizes: the 1,310,720-triangle noisy icosphere (256^3 grid in full
against the reference's own GPU kernel; 512^3 grid, 4 M shell points and a 2.6 M-face overlapping
mesh sampled against the FP64 oracle) and the 64-mesh batch of uneven meshes and grids.

Bars (as in the small-case parity tests):
  * distances: |d - d_ref| <= 1e-5 x bounding-box diagonal;
  * inside/outside signs and self-intersection bits: exact, except where the FP64 oracle's winding
    number lies within TAU of the threshold (those are counted, not failed);
  * winding numbers: within WN_TOL of the FP64 oracle.
The whole-grid results are computed on the GPU; the oracle evaluates a seeded random sample of the
voxels, points or faces (the CPU cannot evaluate a 512^3 grid on a 1.3 M-triangle mesh in a test).
Reference: MRMesh/MRFastWindingNumber.cpp:28-94 (the CPU path the oracle restates),
MRCuda/MRCudaFastWindingNumber.cu:135-243 (the reference kernels)."""
import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

TAU = 1e-3
WN_TOL = 5e-5
SAMPLE = 100_000


@pytest.fixture(scope="module")
def c2(fwn_lib):
    """The C2 mesh, its FP64 oracle and a library handle."""
    import meshlib_gb300 as M
    v, f = mg.noisy_icosphere(seed=0, level=8)
    assert len(f) == 1_310_720
    return v, f, O.Oracle(v, f), M.FastWindingNumber(v, f)


def _check_signed(d, d_ref, wn_ref, diag, what):
    """d: ours; d_ref: oracle (FP64) or reference distances; wn_ref: FP64 winding numbers there."""
    fin, fin_ref = np.isfinite(d), np.isfinite(d_ref)
    assert np.array_equal(fin, fin_ref), f"{what}: NaN pattern differs at {int((fin != fin_ref).sum())} places"
    err = np.abs(np.abs(d[fin]) - np.abs(d_ref[fin]))
    assert err.max() <= 1e-5 * diag, f"{what}: max |d - d_ref| {err.max():.3e} > {1e-5 * diag:.3e}"
    mism = (np.signbit(d) != np.signbit(d_ref)) & fin
    near = np.abs(wn_ref - 0.5) < TAU
    bad = int((mism & ~near).sum())
    assert bad == 0, f"{what}: {bad} sign mismatches away from the threshold ({int((mism & near).sum())} within tau)"
    return float(err.max()), float(np.sqrt(np.mean(err.astype(np.float64) ** 2)))


def test_c2_256_signed_distance_vs_mrcuda(c2):
    """The whole 256^3 grid against the reference's own signedDistanceKernel on the same GPU."""
    from oracle import mrcuda
    if not mrcuda.kernels_present():
        pytest.skip("reference kernels not built here (oracle/ref/build_ref.py needs the reference sources)")
    import torch
    v, f, o, g = c2
    dims, xf = mg.grid_for(v, 256)
    rk = mrcuda.RefKernels(v, f, o.nodes(), o.dipoles(0))
    d_ref = rk.signed_distance(dims, xf).cpu().numpy()
    out = torch.empty(int(np.prod(dims)), device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    d = out.cpu().numpy()
    del out, rk
    diag = mg.diag(v)
    assert np.isfinite(d).all() and np.isfinite(d_ref).all()
    err = np.abs(np.abs(d) - np.abs(d_ref))
    assert err.max() <= 1e-5 * diag, f"max |d - d_mrcuda| {err.max():.3e}"
    sel = np.flatnonzero(np.signbit(d) != np.signbit(d_ref))
    if len(sel):  # decide every disagreement with the FP64 oracle's winding number
        _, wn = o.grid_voxels(dims, xf, sel, prec=1)
        bad = int((np.abs(wn - 0.5) >= TAU).sum())
        assert bad == 0, f"{bad} of {len(sel)} sign disagreements with the reference kernel are away from the threshold"


def test_c2_512_signed_distance_sampled_vs_fp64(c2):
    """calcFromGridWithDistances on the whole 512^3 grid; 100k seeded voxels against the FP64 oracle,
    plus calcFromGrid's winding numbers at the same voxels."""
    import torch
    v, f, o, g = c2
    dims, xf = mg.grid_for(v, 512)
    n = int(np.prod(dims))
    out = torch.empty(n, device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    rng = np.random.default_rng(512)
    ids = np.sort(rng.choice(n, SAMPLE, replace=False)).astype(np.int64)
    # half of the sample near the surface, where signs and near-plane arithmetic are decided
    near = torch.nonzero(out.abs() < 0.02 * mg.diag(v)).flatten()
    pick = near[torch.from_numpy(rng.integers(0, len(near), SAMPLE // 2)).cuda()].cpu().numpy().astype(np.int64)
    ids = np.unique(np.concatenate([ids[: SAMPLE // 2], pick]))
    d = out[torch.from_numpy(ids).cuda()].cpu().numpy()
    d_ref, wn_ref = o.grid_voxels(dims, xf, ids, prec=1)
    _check_signed(d, d_ref, wn_ref, mg.diag(v), "512^3 signed distance")
    # winding numbers of the same voxels (calcFromGrid)
    g.calcFromGrid_dev(dims, xf, out.data_ptr(), stream=0)
    torch.cuda.synchronize()
    w = out[torch.from_numpy(ids).cuda()].cpu().numpy()
    assert np.abs(w - wn_ref).max() <= WN_TOL


def test_c3_shell_points_sampled_vs_fp64(c2):
    """4 M points within 1e-3 of the surface: calcFromVector and the signed distance at points on all
    of them, 100k seeded ones against the FP64 oracle."""
    import torch
    v, f, o, g = c2
    pts = mg.shell_points(v, f, 4_000_000, width=1e-3, seed=0)
    dp = torch.from_numpy(pts).cuda()
    w = torch.empty(len(pts), device="cuda")
    d = torch.empty(len(pts), device="cuda")
    g.calcFromVector_dev(dp.data_ptr(), len(pts), w.data_ptr(), stream=0)
    g.calcWithDistances_dev(dp.data_ptr(), len(pts), d.data_ptr(), stream=0)
    torch.cuda.synchronize()
    idx = np.random.default_rng(3).choice(len(pts), SAMPLE, replace=False)
    sub = pts[idx]
    w_ref = o.from_vector(sub, prec=1)
    assert np.abs(w.cpu().numpy()[idx] - w_ref).max() <= WN_TOL
    d_ref = o.vector_with_distances(sub, prec=1)
    _check_signed(d.cpu().numpy()[idx], d_ref, w_ref, mg.diag(v), "shell points")


def test_c2_sized_self_intersections_sampled_vs_fp64(fwn_lib):
    """calcSelfIntersections on two overlapping level-8 spheres (2.6 M faces, about a third flagged);
    100k seeded faces' bits and centroid winding numbers against the FP64 oracle."""
    import meshlib_gb300 as M
    v, f = mg.overlapping_spheres(seed=0, level=8, offset=0.5)
    g = M.FastWindingNumber(v, f)
    bits, wn = g.calcSelfIntersections(with_wn=True)
    faces = np.random.default_rng(8).choice(len(f), SAMPLE, replace=False).astype(np.int32)
    o = O.Oracle(v, f)
    b_ref, w_ref = o.self_intersections_at(faces, prec=1)
    assert 0.1 < bits.mean() < 0.9
    assert np.abs(wn[faces] - w_ref).max() <= WN_TOL
    near = (np.abs(w_ref) < TAU) | (np.abs(w_ref - 1) < TAU)
    assert int(((bits[faces] != b_ref) & ~near).sum()) == 0


def test_c4_batch_sampled_vs_fp64(fwn_lib):
    """The 64-mesh batch (triangles log-uniform in [5k, 500k], grid sides log-uniform in [32, 192])
    in one persistent launch; 2,000 seeded voxels of every grid against the FP64 oracle."""
    import torch

    import meshlib_gb300 as M
    meshes = mg.batch_meshes(64, seed=0)
    items, outs = [], []
    for (bv, bf, bdims, bxf) in meshes:
        h = M.FastWindingNumber(bv, bf)
        o = torch.empty(int(np.prod(bdims)), device="cuda")
        items.append((h, bdims, bxf, None, o.data_ptr()))
        outs.append(o)
    b = M.Batch(items)
    b.run_dev()
    torch.cuda.synchronize()
    rng = np.random.default_rng(64)
    for k, ((bv, bf, bdims, bxf), o) in enumerate(zip(meshes, outs)):
        n = int(np.prod(bdims))
        ids = np.sort(rng.choice(n, min(n, 2000), replace=False)).astype(np.int64)
        d = o[torch.from_numpy(ids).cuda()].cpu().numpy()
        d_ref, wn_ref = O.Oracle(bv, bf).grid_voxels(bdims, bxf, ids, prec=1)
        _check_signed(d, d_ref, wn_ref, mg.diag(bv), f"batch item {k}")
    b.close()
