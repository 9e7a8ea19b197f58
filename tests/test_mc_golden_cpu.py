"""The mesher oracle (oracle/mc_oracle.cpp) against MeshLib's own mesher, bit for bit.

tests/golden/mc_reference.npz holds the outputs of the reference's MRVoxels/MRMarchingCubes.cpp,
compiled from its own sources (oracle/ref/build_cpu_ref.py) and run on seeded volumes by
tests/golden/make_mc_golden.py: the reference's own test input, distance and density volumes,
z-blocks of several sizes, MarchingCubesByParts with even and uneven parts, NaN voxels, ragged and
degenerate sizes, a volume with every crossing cube configuration, and the reference's error cases
(a part of one layer, the vertex limit).  Where the reference library is present on this machine
the fixture is also re-derived from it."""
import os

import numpy as np
import pytest

import oracle as O
import oracle.mcref as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mc_reference.npz")
_G = np.load(GOLDEN)
CASES = [str(c) for c in _G["cases"]]


def case(name):
    p = _G[f"{name}/params"]
    parts = _G[f"{name}/parts"]
    kw = dict(origin=tuple(p[0:3]), voxel_size=tuple(p[3:6]), iso=float(p[6]), less_inside=bool(p[7]),
              part_starts=parts if len(parts) else None, max_vertices=int(p[8]))
    ref = (_G[f"{name}/points"], _G[f"{name}/tris"], _G[f"{name}/faceMap"])
    return _G[f"{name}/vol"], kw, int(p[9]), ref, str(_G[f"{name}/error"])


def _same(out, ref):
    assert out[0].shape == ref[0].shape and out[1].shape == ref[1].shape
    assert np.array_equal(out[0].view(np.uint32), ref[0].view(np.uint32))  # every float, bit for bit
    assert np.array_equal(out[1], ref[1])
    assert np.array_equal(out[2], ref[2])


def test_fixture_covers_the_cases():
    assert len(CASES) >= 20
    vol, kw, _, ref, _ = case("every_configuration")
    z, y, x = np.unravel_index(ref[2], vol.shape)
    cfg = np.zeros(len(z), np.int64)
    for i, bit in enumerate([0, 1, 3, 2, 4, 5, 7, 6]):
        cfg |= (vol[z + (i >> 2), y + ((i >> 1) & 1), x + (i & 1)] < 0).astype(np.int64) << bit
    assert len(np.unique(cfg)) == 254  # all but the empty and the full cube
    assert len(case("reference_test_sphere")[3][1]) > 0  # the reference test's own expectation
    assert any(case(c)[4] for c in CASES) and any(len(case(c)[3][0]) and not len(case(c)[3][1]) for c in CASES)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_mesher(name):
    vol, kw, _, ref, err = case(name)
    if err:
        with pytest.raises(O.McError, match=err.rstrip(".")):
            O.marching_cubes(vol, **kw)
    else:
        _same(O.marching_cubes(vol, **kw), ref)


@pytest.mark.skipif(not R.available(), reason="the reference mesher is built only where a copy of the reference is")
@pytest.mark.parametrize("name", CASES)
def test_fixture_rederived_from_reference(name):
    vol, kw, lpb, ref, err = case(name)
    if err:
        with pytest.raises(R.McRefError, match=err.rstrip(".")):
            R.marching_cubes(vol, layers_per_block=lpb, **kw)
    else:
        _same(R.marching_cubes(vol, layers_per_block=lpb, **kw), ref)
