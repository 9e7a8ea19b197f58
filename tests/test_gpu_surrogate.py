"""Surrogate network: tensor-core forward/backward against the FP64 CPU oracle of the same network
(oracle/mlp_oracle.py, same bf16 rounding points), and the banded signed distance with learned
brick culling against the plain banded result.

Tolerances: gradients, per parameter tensor, relative L2 error <= 2e-2 (FP32 accumulation and
single-ulp bf16 rounding differences against FP64); predictions within 2e-3 of the oracle; the banded
grids must be identical (the culling may only skip bricks whose voxels are all NaN)."""
import ctypes
import math

import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def _meta(clamp=0.5):
    m = np.zeros(48, np.float32)  # SURROGATE_META floats
    m[3] = 1.0
    m[4:36] = [np.float32(math.pi * 2 ** (k / 5)) for k in range(32)]
    m[36] = clamp
    return m


def _params(seed=0):
    rng = np.random.default_rng(seed)
    P = {}
    for name, shp in MO.SIZES:
        fan_in = shp[1] if len(shp) == 2 else 128
        lim = math.sqrt(3.0 / fan_in) * (1.0 if name == "W1" else 1.4142)
        P[name] = rng.uniform(-lim, lim, shp) if name.startswith("W") else rng.uniform(-0.1, 0.1, shp)
    P["w5"] = rng.uniform(-0.05, 0.05, 128)
    return MO.pack(P).astype(np.float32)


def test_gradients_match_cpu_oracle(fwn_lib):
    import torch

    import meshlib_gb300 as M
    params, meta = _params(1), _meta()
    s = M.Surrogate.create(params, meta)
    rng = np.random.default_rng(3)
    n = 4000  # not a multiple of 128: padded rows must not contribute
    pts = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    tgt = (np.linalg.norm(pts, axis=1) - 0.6).astype(np.float32)
    dp, dt = torch.from_numpy(pts).cuda(), torch.from_numpy(tgt).cuda()
    g, loss = s.gradients_dev(dp.data_ptr(), dt.data_ptr(), n)
    rl, rg = MO.loss_and_grads(params.astype(np.float64), meta, pts, tgt)
    assert abs(loss - rl) <= 1e-3 * abs(rl)
    o = 0
    for name, shp in MO.SIZES:
        k = int(np.prod(shp))
        a, b = g[o:o + k].astype(np.float64), rg[o:o + k]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err <= 2e-2, (name, err)
        o += k


def test_inference_matches_cpu_oracle(fwn_lib):
    import torch

    import meshlib_gb300 as M
    params, meta = _params(2), _meta()
    s = M.Surrogate.create(params, meta)
    pts = np.random.default_rng(4).uniform(-1, 1, (1000, 3)).astype(np.float32)
    out = torch.empty(1000, device="cuda")
    s.eval_dev(torch.from_numpy(pts).cuda().data_ptr(), 1000, out.data_ptr())
    torch.cuda.synchronize()
    ref = MO.predict(params.astype(np.float64), meta, pts)
    assert np.abs(out.cpu().numpy() - ref).max() <= 2e-3 * max(1.0, np.abs(ref).max())


@pytest.fixture(scope="module")
def banded_case(fwn_lib):
    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_torus(seed=3)
    dims, xf = mg.grid_for(v, 72)
    band = 0.04 * mg.diag(v)
    g = M.FastWindingNumber(v, f)
    sur = M.Surrogate.train(g, dims, xf, band, samples=262144, validation=131072, steps=800, batch=8192, seed=5)
    return g, sur, dims, xf, band


def test_surrogate_training_converges(banded_case):
    g, sur, dims, xf, band = banded_case
    st = sur.stats
    assert st["steps"] == 800
    assert st["validationMaxError"] < 2.0 * band, st
    # the culling margin covers the worst overstatement of |d| near the band, which cannot exceed
    # the worst two-sided error
    assert st["margin"] >= st["validationOverestimate"]
    assert st["validationOverestimate"] <= st["validationMaxError"]
    assert st["limit"] > band


def test_banded_culling_equals_plain_banded(banded_case):
    import torch

    import meshlib_gb300 as M
    g, sur, dims, xf, band = banded_case
    n = int(np.prod(dims))
    opts = M.DistanceToMeshOptions(maxDistSq=band * band)
    plain = torch.empty(n, device="cuda")
    exact = torch.empty(n, device="cuda")
    learned = torch.empty(n, device="cuda")
    s = torch.cuda.Stream()
    g.calcFromGridWithDistances_dev(dims, xf, plain.data_ptr(), options=opts, stream=s.cuda_stream)
    st_exact = g.calcFromGridWithDistancesBanded_dev(dims, xf, exact.data_ptr(), opts, None, stream=s.cuda_stream)
    st_learn = g.calcFromGridWithDistancesBanded_dev(dims, xf, learned.data_ptr(), opts, sur, stream=s.cuda_stream)
    s.synchronize()
    p, e, l = plain.cpu().numpy(), exact.cpu().numpy(), learned.cpu().numpy()
    assert np.isfinite(p).sum() > 1000
    for other in (e, l):
        assert np.array_equal(np.isnan(other), np.isnan(p))
        fin = np.isfinite(p)
        assert np.array_equal(other[fin], p[fin])
    assert st_exact["keptBricks"] < st_exact["bricks"]
    assert st_learn["keptBricks"] < st_learn["bricks"]


def test_parameters_roundtrip(banded_case):
    import torch

    import meshlib_gb300 as M
    g, sur, dims, xf, band = banded_case
    params, meta = sur.parameters()
    assert meta[38] == pytest.approx(band)
    clone = M.Surrogate.create(params, meta)
    pts = torch.rand(4096, 3, device="cuda") * 2 - 1
    a = torch.empty(4096, device="cuda")
    b = torch.empty(4096, device="cuda")
    sur.eval_dev(pts.data_ptr(), 4096, a.data_ptr())
    clone.eval_dev(pts.data_ptr(), 4096, b.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_learned_culling_gain_on_c5(fwn_lib):
    """What the trained network gains on the learned-band-culling configuration (1.31 M-triangle noisy
    icosphere, band 0.01 x diagonal, 512^3): against the method without it -- the reference's banded
    request evaluated at every voxel -- the same grid, far fewer voxels through the exact traversal and
    less time; against the no-learning control (bricks culled with exact brick-centre distances) a
    cheaper culling pass.  Times are CUDA-event medians of several runs after a warm-up."""
    import torch

    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_icosphere(seed=0, level=8)
    dims, xf = mg.grid_for(v, 512)
    n = int(np.prod(dims))
    band = 0.01 * mg.diag(v)
    g = M.FastWindingNumber(v, f)
    sur = M.Surrogate.train(g, dims, xf, band, seed=1)
    opts = M.DistanceToMeshOptions(maxDistSq=band * band)
    plain = torch.empty(n, device="cuda")
    learned = torch.empty(n, device="cuda")
    s = torch.cuda.Stream()

    def timed(fn, k=7):
        fn()
        s.synchronize()
        ts = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            fn()
            b.record(s)
            s.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    st = {}
    st_exact = {}
    plain_ms = timed(lambda: g.calcFromGridWithDistances_dev(dims, xf, plain.data_ptr(), options=opts, stream=s.cuda_stream))
    learned_ms = timed(lambda: st.update(g.calcFromGridWithDistancesBanded_dev(dims, xf, learned.data_ptr(), opts, sur,
                                                                              stream=s.cuda_stream)))
    timed(lambda: st_exact.update(g.calcFromGridWithDistancesBanded_dev(dims, xf, learned.data_ptr(), opts, None,
                                                                        stream=s.cuda_stream)), 3)
    timed(lambda: st.update(g.calcFromGridWithDistancesBanded_dev(dims, xf, learned.data_ptr(), opts, sur,
                                                                  stream=s.cuda_stream)), 3)
    assert torch.equal(torch.isnan(plain), torch.isnan(learned))
    fin = ~torch.isnan(plain)
    assert torch.equal(plain[fin], learned[fin])
    exact_fraction = st["keptBricks"] * 512 / n
    assert exact_fraction < 0.25, st  # plain banded sends every voxel through the traversal
    assert learned_ms < plain_ms, (learned_ms, plain_ms)
    assert st["cullMs"] < st_exact["cullMs"], (st, st_exact)
