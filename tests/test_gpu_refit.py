"""Refit after moved vertices (MR::AABBTree::refit + dipoles) on the GPU vs the oracle's restatement.

Tolerances: the refit tree and dipoles are bit-exact (same float operations as the reference);
distances after a refit equal a rebuild's within 1e-5 * diagonal (the search is exact whatever the
tree); signed distances and winding numbers follow the oracle run on the refit tree, as in
tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

import oracle as O
from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

TAU = 1e-3


@pytest.fixture(scope="module")
def M(fwn_lib):
    import meshlib_gb300
    return meshlib_gb300


def _deform(v, seed, frac=1.0, amp=0.04):
    rng = np.random.default_rng(seed)
    moved = rng.random(len(v)) < frac
    v2 = v.copy()
    # smooth displacement (a wave) so the surface stays a surface
    disp = amp * np.stack([np.sin(3 * v[:, 1]), np.cos(2 * v[:, 2]), np.sin(4 * v[:, 0])], 1)
    v2[moved] += disp[moved].astype(np.float32)
    return v2, moved


@pytest.mark.parametrize("frac", [1.0, 0.2])
def test_refit_tree_bit_exact(M, frac):
    v, f = mg.noisy_torus(seed=1)
    g = M.FastWindingNumber(v, f)
    o = O.Oracle(v, f)
    v2, moved = _deform(v, 3, frac)
    changed = None if frac == 1.0 else moved
    g.refit(v2, changed)
    o.refit(v2, changed)
    nodes, dip = g.tree()
    assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8))
    assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32))


def test_refit_queries_follow_the_moved_mesh(M):
    v, f = mg.noisy_icosphere(seed=2, level=5)
    g = M.FastWindingNumber(v, f)
    o = O.Oracle(v, f)
    v2, moved = _deform(v, 5, 0.5, amp=0.08)
    g.refit(v2, moved)
    o.refit(v2, moved)
    dims, xf = mg.grid_for(v2, 24)
    d = g.calcFromGridWithDistances(dims, xf)
    ref, wref = o.from_grid_with_distances(dims, xf, prec=1, want_fwn=True)
    diag = mg.diag(v2)
    assert np.abs(np.abs(d) - np.abs(ref)).max() <= 1e-5 * diag
    mism = np.signbit(d) != np.signbit(ref)
    assert (mism & (np.abs(wref - 0.5) >= TAU)).sum() == 0
    # the same distances as a tree built from scratch on the moved mesh
    fresh = M.FastWindingNumber(v2, f)
    d2 = fresh.calcFromGridWithDistances(dims, xf)
    assert np.abs(np.abs(d) - np.abs(d2)).max() <= 1e-5 * diag
    # closest points too
    rng = np.random.default_rng(9)
    pts = rng.uniform(-1.5, 1.5, (3000, 3)).astype(np.float32)
    proj = M.PointsToMeshProjector.from_mesh(g).findProjections(pts)
    pref = o.find_projections(pts)
    assert np.abs(np.sqrt(proj["distSq"].astype(np.float64)) - np.sqrt(pref["distSq"].astype(np.float64))).max() <= 1e-5 * diag


def test_refit_dev_and_repeat(M):
    import torch
    v, f = mg.noisy_torus(seed=4)
    g = M.FastWindingNumber(v, f)
    o = O.Oracle(v, f)
    for k in range(3):  # repeated refits keep matching the oracle's
        v2, _ = _deform(v, 10 + k, 1.0, amp=0.02 * (k + 1))
        dv = torch.from_numpy(v2.reshape(-1)).cuda()
        torch.cuda.synchronize()  # the upload is on torch's stream; the refit runs on the handle's
        g.refit_dev(dv.data_ptr())
        o.refit(v2)
        nodes, dip = g.tree()
        assert np.array_equal(nodes.view(np.uint8), o.nodes().view(np.uint8))
        assert np.array_equal(dip.view(np.uint32), o.dipoles(0).view(np.uint32))
    with pytest.raises(M.FwnError):  # no vertex array
        M._check(M.lib().gbfwn_refit(g.handle, None, None))
