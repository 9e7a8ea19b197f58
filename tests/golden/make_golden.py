"""Generates tests/golden/mrcuda_small.npz: outputs of the reference's own GPU kernels
(MRCuda/MRCudaFastWindingNumber.cu and MRCuda/MRCudaPointsToMeshProjector.cu, built from the
reference sources by oracle/ref/build_ref.py and launched by oracle/mrcuda.py) on small seeded inputs.

Run on a GPU machine where oracle/_ref holds the built reference kernels:
    python tests/golden/make_golden.py [output path, default tests/golden/mrcuda_small.npz]
The inputs are regenerated by the tests from the same seeded generators (meshlib_gb300/meshgen.py);
the file stores SHA-256 digests of the input arrays so a test can tell if a generator changed.

Contents (all float32 unless noted):
  sdf_grid    signedDistanceKernel on the 16,384-triangle noisy torus (seed 0), grid_for(v, 32)
  fwn_grid    fastWindingNumberFromGridKernel, same mesh and grid, beta 2
  pts         2,048 seeded points around the torus; fwn_pts = fastWindingNumberFromVectorKernel at
              them with face 11 skipped
  selfint_wn  fastWindingNumberFromMeshKernel on two overlapping level-3 spheres (self-intersection
              winding numbers; the face is flagged when wn < 0 or wn > 1)
  proj        the projector kernel's 32-byte MeshProjectionResult records for pts (uint8)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "mrcuda_small.npz")


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def inputs():
    """The seeded inputs of every fixture (shared with the tests)."""
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 32)
    rng = np.random.default_rng(2024)
    lo, hi = v.min(0), v.max(0)
    pts = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo), (2048, 3)).astype(np.float32)
    sv, sf = mg.overlapping_spheres(seed=0, level=3)
    return v, f, dims, xf, pts, sv, sf


def main(out: str = OUT):
    import oracle as O
    from oracle import mrcuda
    if not mrcuda.kernels_present():
        raise SystemExit("reference kernels not built (oracle/ref/build_ref.py)")
    v, f, dims, xf, pts, sv, sf = inputs()
    o = O.Oracle(v, f)
    rk = mrcuda.RefKernels(v, f, o.nodes(), o.dipoles(0))
    sdf = rk.signed_distance(dims, xf).cpu().numpy()
    fwn = rk.from_grid(dims, xf).cpu().numpy()
    fwn_pts = rk.from_vector(pts, skip_face=11).cpu().numpy()
    proj = rk.project(pts).cpu().numpy()
    os_ = O.Oracle(sv, sf)
    rks = mrcuda.RefKernels(sv, sf, os_.nodes(), os_.dipoles(0))
    selfint = rks.from_mesh().cpu().numpy()
    np.savez_compressed(out, sdf_grid=sdf, fwn_grid=fwn, pts=pts, fwn_pts=fwn_pts, selfint_wn=selfint, proj=proj,
                        dims=np.asarray(dims, np.int32), xf=np.asarray(xf, np.float32),
                        digest_torus=np.array(digest(v, f)), digest_spheres=np.array(digest(sv, sf)))
    print(f"wrote {out} ({os.path.getsize(out)} bytes)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else OUT)
