"""Batched persistent launch: every grid of an uneven batch equals the single-mesh result (bit for
bit: each voxel makes the same decisions and sums its terms in the same order whatever warp tile it
shares), for every tile-shape / block-size variant, with the one-voxel and the paired walk, and through
the CUDA-graph replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_single_calls(fwn_lib, tmp_path, monkeypatch):
    import torch

    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg
    monkeypatch.setenv("MESHLIB_GB300_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    specs = [(mg.noisy_torus(seed=1, nu=40, nv=20), 23), (mg.noisy_icosphere(seed=2, level=4), 37),
             (mg.noisy_torus(seed=3), 16), (mg.noisy_icosphere(seed=4, level=3), 50), (mg.figure8_torus(), 9)]
    items, refs, outs = [], [], []
    s = torch.cuda.Stream()
    for k, ((v, f), n) in enumerate(specs):
        g = M.FastWindingNumber(v, f)
        dims, xf = mg.grid_for(v, n)
        dims = (n, n + k, max(3, n - 2 * k))  # uneven, non-cubic
        if k == 2:  # a tilted grid: the paired variants project the upper voxel on its own
            c, s_ = np.float32(np.cos(0.3)), np.float32(np.sin(0.3))
            xf = np.asarray(xf, np.float32).copy()
            xf[:9] = (xf[:9].reshape(3, 3) @ np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]], np.float32)).reshape(-1)
        opts = M.DistanceToMeshOptions(maxDistSq=0.05) if k == 1 else None
        ref = torch.empty(int(np.prod(dims)), device="cuda")
        g.calcFromGridWithDistances_dev(dims, xf, ref.data_ptr(), options=opts, stream=s.cuda_stream)
        out = torch.full_like(ref, 7.0)
        items.append((g, dims, xf, opts, out.data_ptr()))
        refs.append(ref)
        outs.append(out)
    b = M.Batch(items)
    s.synchronize()
    for c in range(len(M.Batch.configs())):
        for o in outs:
            o.fill_(7.0)
        b.set_config(c)
        b.run_dev(stream=s.cuda_stream)
        s.synchronize()
        for r, o in zip(refs, outs):
            assert torch.equal(torch.isnan(r), torch.isnan(o))
            fin = ~torch.isnan(r)
            assert torch.equal(r[fin], o[fin]), c
    rec = b.autotune()
    assert rec["cached"] is False and len(rec["times_ms"]) == len(M.Batch.configs()) == 12
    assert M.Batch(items).autotune()["cached"] is True
    for o in outs:
        o.fill_(7.0)
    b.graph_launch(stream=s.cuda_stream)
    b.graph_launch(stream=s.cuda_stream)
    s.synchronize()
    for r, o in zip(refs, outs):
        fin = ~torch.isnan(r)
        assert torch.equal(r[fin], o[fin])


def test_mesh_of_live_batch_cannot_be_destroyed(fwn_lib):
    """A batch points into its meshes' trees: destroying one of them while the batch lives is refused
    (the handle stays usable), and succeeds once the batch is gone."""
    import torch

    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_icosphere(seed=5, level=3)
    g = M.FastWindingNumber(v, f)
    dims, xf = mg.grid_for(v, 12)
    out = torch.empty(int(np.prod(dims)), device="cuda")
    out2 = torch.empty_like(out)
    b = M.Batch([(g, dims, xf, None, out.data_ptr()), (g, dims, xf, None, out2.data_ptr())])
    with pytest.raises(M.FwnError) as ei:
        g.close()
    assert ei.value.status == M.INVALID and "batch" in str(ei.value)
    b.run_dev()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), g.calcFromGridWithDistances(dims, xf))
    assert torch.equal(out, out2)
    b.close()
    g.close()
    assert not g.handle.value


def test_batch_with_a_lower_distance_bound(fwn_lib):
    """An item with minDistSq > 0: a walk stops at the first distance <= minDistSq it meets (the
    reference's early stop), so below that bound a value depends on the walk's order and only the
    bound is guaranteed; every other voxel, and the sign of every voxel, equals the single calls in
    every variant (the paired ones run as their one-voxel counterparts)."""
    import torch

    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg
    items, refs, outs, lows = [], [], [], []
    for k, (v, f) in enumerate((mg.noisy_icosphere(seed=6, level=4), mg.noisy_torus(seed=7))):
        g = M.FastWindingNumber(v, f)
        dims, xf = mg.grid_for(v, 40)
        opts = M.DistanceToMeshOptions(minDistSq=0.001, maxDistSq=0.05, nullOutsideMinMax=False) if k == 0 else None
        lows.append(0.001 if k == 0 else 0.0)
        ref = torch.empty(int(np.prod(dims)), device="cuda")
        g.calcFromGridWithDistances_dev(dims, xf, ref.data_ptr(), options=opts, stream=0)
        out = torch.full_like(ref, 7.0)
        items.append((g, dims, xf, opts, out.data_ptr()))
        refs.append(ref)
        outs.append(out)
    b = M.Batch(items)
    torch.cuda.synchronize()
    for c in range(len(M.Batch.configs())):
        for o in outs:
            o.fill_(7.0)
        b.set_config(c)
        b.run_dev(stream=0)
        torch.cuda.synchronize()
        for r, o, low in zip(refs, outs, lows):
            assert torch.equal(torch.isnan(r), torch.isnan(o))
            fin = ~torch.isnan(r)
            assert torch.equal(torch.signbit(r[fin]), torch.signbit(o[fin])), c
            above = fin & (r * r >= low)
            assert torch.equal(r[above], o[above]), c
            below = fin & (r * r < low)
            assert bool((o[below] * o[below] <= low).all()), c
