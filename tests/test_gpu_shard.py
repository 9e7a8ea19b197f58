"""Slab entry points on the GPU: the z-slabs of every rank of a sharded run, computed separately and
stacked, equal the whole-grid call bit for bit (signed distance and winding number)."""
import numpy as np
import pytest

from meshlib_gb300 import meshgen as mg
from meshlib_gb300 import shard

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3, 7])
def test_slabs_stack_to_the_whole_grid(fwn_lib, world):
    import torch

    import meshlib_gb300 as M
    v, f = mg.noisy_icosphere(seed=2, level=5)
    dims, xf = mg.grid_for(v, 40)
    dims = (dims[0], dims[1], 37)  # ragged depth
    g = M.FastWindingNumber(v, f)
    n = int(np.prod(dims))
    whole = torch.empty(n, device="cuda")
    g.calcFromGridWithDistances_dev(dims, xf, whole.data_ptr(), stream=0)
    parts = [shard.rank_signed_distance(g, dims, xf, r, world, stream=0) for r in range(world)]
    torch.cuda.synchronize()
    stacked = torch.cat([p[2] for p in parts])
    assert torch.equal(stacked.view(torch.int32), whole.view(torch.int32))
    # winding numbers too
    wn = torch.empty(n, device="cuda")
    g.calcFromGrid_dev(dims, xf, wn.data_ptr(), stream=0)
    sl = []
    for z0, z1 in shard.zslabs(dims[2], world):
        t = torch.empty((z1 - z0) * dims[0] * dims[1], device="cuda")
        if z1 > z0:
            g.calcFromGridSlab_dev(dims, xf, z0, z1, t.data_ptr(), stream=0)
        sl.append(t)
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(sl).view(torch.int32), wn.view(torch.int32))
    with pytest.raises(M.FwnError):
        g.calcFromGridSlab_dev(dims, xf, 5, 5, wn.data_ptr())
