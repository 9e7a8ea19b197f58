"""The allocation-free signed-distance entry point (gbfwn_from_grid_with_distances_noalloc), called
through the C ABI, must give what the regular device entry point gives on the same mesh and grid.

It exists for callers that may not allocate device memory when they need a grid (a host that owns
the memory budget, a latency-bound loop that cannot take cudaFree's synchronisation).  Its scratch
is a fixed device array shared by all calls and kept between them, so the test makes two calls in
a row: the second must not see anything left over by the first.  This file is collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIST_TOL = 1e-5  # x bounding-box diagonal, the distance tolerance of the parity tests


def test_no_alloc_matches_device_entry_twice(fwn_lib):
    import torch

    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg

    v, f = mg.noisy_torus(seed=2)
    g = M.FastWindingNumber(v, f)
    dims = (37, 29, 23)  # ragged: not a multiple of the 4x4x2 warp tile
    _, xf = mg.grid_for(v, 37)
    n = int(np.prod(dims))
    s = torch.cuda.Stream()
    ref = torch.full((n,), 7.0, device="cuda")
    outs = [torch.full((n,), 7.0, device="cuda") for _ in range(2)]
    band = M.DistanceToMeshOptions(maxDistSq=0.04)  # some voxels NaN, some finite
    torch.cuda.synchronize()
    for opts in (None, band):
        g.calcFromGridWithDistances_dev(dims, xf, ref.data_ptr(), options=opts, stream=s.cuda_stream)
        for o in outs:
            o.fill_(7.0)
        torch.cuda.synchronize()
        L = M.lib()
        d = np.asarray(dims, np.int32)
        x12 = np.ascontiguousarray(xf, np.float32)
        copts = (opts or M.DistanceToMeshOptions())._c()
        # every device allocation the library makes on this thread fails while the hook is armed, so
        # an allocation slipped into this path would turn the status into GBFWN_OUT_OF_MEMORY
        L.gbfwn_debug_fail_next_allocs(1 << 30)
        try:
            for o in outs:  # two calls in a row through the C ABI
                st = L.gbfwn_from_grid_with_distances_noalloc(g.handle, d.ctypes.data, x12.ctypes.data,
                                                             ctypes.byref(copts), ctypes.c_void_p(o.data_ptr()),
                                                             ctypes.c_void_p(s.cuda_stream))
                assert st == M.OK, L.gbfwn_last_error()
        finally:
            L.gbfwn_debug_fail_next_allocs(0)
        s.synchronize()
        r = ref.cpu().numpy()
        tol = DIST_TOL * mg.diag(v)
        for o in outs:
            a = o.cpu().numpy()
            assert np.array_equal(np.isnan(a), np.isnan(r))
            fin = np.isfinite(r)
            assert np.abs(a[fin] - r[fin]).max() <= tol
            assert np.array_equal(np.sign(a[fin]), np.sign(r[fin]))


def test_no_alloc_rejects_oversized_grid(fwn_lib):
    import meshlib_gb300 as M
    from meshlib_gb300 import meshgen as mg

    v, f = mg.noisy_torus(seed=2, nu=16, nv=8)
    g = M.FastWindingNumber(v, f)
    import torch
    out = torch.empty(4, device="cuda")
    identity = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float32)
    with pytest.raises(M.FwnError) as ei:  # rejected on the host before any device work
        g.calcFromGridWithDistances_noalloc((1 << 20, 1 << 20, 1 << 10), identity, out.data_ptr())
    assert ei.value.status == M.INVALID
    assert "too large" in str(ei.value)
