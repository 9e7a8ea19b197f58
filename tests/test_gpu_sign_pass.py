"""makeSignedByWindingNumber (MRVoxels/MRVDBConversions.cpp:491-571) on a dense device grid: values
whose voxel's winding number exceeds the threshold are negated -- bit for bit the winding-number grid
of calcFromGrid applied on the host, and the sign of calcFromGridWithDistances for |d| input."""
import numpy as np
import pytest

from meshlib_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def test_sign_pass_matches_winding_grid(fwn_lib):
    import torch

    import meshlib_gb300 as M
    v, f = mg.noisy_torus(seed=5)
    g = M.FastWindingNumber(v, f)
    dims, xf = mg.grid_for(v, 40)
    n = int(np.prod(dims))
    rng = np.random.default_rng(3)
    vals = rng.uniform(0.1, 1.0, n).astype(np.float32)
    d = torch.from_numpy(vals.copy()).cuda()
    for beta, thr in ((2.0, 0.5), (2.0, 0.3), (1.5, 0.7)):
        d.copy_(torch.from_numpy(vals))
        g.makeSignedByWindingNumber_dev(dims, xf, d.data_ptr(), beta=beta, threshold=thr, stream=0)
        torch.cuda.synchronize()
        wn = g.calcFromGrid(dims, xf, beta=beta)
        assert np.array_equal(d.cpu().numpy(), np.where(wn > thr, -vals, vals))
    # |signed distance| signed by the pass == the signed distance (same winding numbers, threshold 0.5)
    sd = g.calcFromGridWithDistances(dims, xf)
    a = torch.from_numpy(np.abs(sd)).cuda()
    g.makeSignedByWindingNumber_dev(dims, xf, a.data_ptr(), stream=0)
    torch.cuda.synchronize()
    assert np.array_equal(a.cpu().numpy(), sd)


def test_sign_pass_vs_fp64_oracle(fwn_lib):
    """The negated voxels are exactly those whose FP64 oracle winding number exceeds the threshold,
    except within TAU of it (MRVoxels/MRVDBConversions.cpp:516-530 over the winding-number grid of
    MRMesh/MRFastWindingNumber.cpp:54-67)."""
    import torch

    import meshlib_gb300 as M
    import oracle as O
    TAU = 1e-3
    v, f = mg.noisy_icosphere(seed=7, level=5)
    g = M.FastWindingNumber(v, f)
    o = O.Oracle(v, f)
    dims, xf = mg.grid_for(v, 36)
    dims = (36, 31, 27)  # ragged
    n = int(np.prod(dims))
    vals = np.random.default_rng(5).uniform(0.1, 1.0, n).astype(np.float32)
    for beta, thr in ((2.0, 0.5), (1.5, 0.25)):
        d = torch.from_numpy(vals.copy()).cuda()
        g.makeSignedByWindingNumber_dev(dims, xf, d.data_ptr(), beta=beta, threshold=thr, stream=0)
        torch.cuda.synchronize()
        res = d.cpu().numpy()
        assert np.array_equal(np.abs(res), vals)
        wn = o.from_grid(dims, xf, beta=beta, prec=1)
        neg_expected = wn > thr
        near = np.abs(wn - thr) < TAU
        assert int(((res < 0) != neg_expected)[~near].sum()) == 0
        assert neg_expected.any() and (~neg_expected).any()
