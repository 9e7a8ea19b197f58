"""Generates tests/golden/fwn_cpu_reference.npz: outputs of MeshLib's own CPU winding-number /
signed-distance path (MRMesh/MRFastWindingNumber.cpp with its tree, dipoles and projection, compiled
from the reference sources by oracle/ref/build_cpu_ref.py and called through oracle/fwnref.py) on
seeded inputs that the tests regenerate.

Run on an x86-64 machine with a copy of the reference:
    python tests/golden/make_fwn_cpu_golden.py [output path, default tests/golden/fwn_cpu_reference.npz]

Contents (float32 unless noted; digests are SHA-256 of the arrays' bytes):
  torus_*       the 16,384-triangle noisy torus (seed 0) on grid_for(v, 32):
                nodes_digest / dipoles_digest  the reference tree (32-byte nodes) and dipoles (8 floats)
                sdf       calcFromGridWithDistances, default options
                sdf_band  the same with maxDistSq = (0.05 diag)^2, minDistSq = (0.01 diag)^2 (NaN outside)
                fwn       calcFromGrid, beta 2
                fwn_pts   calcFromVector at 2,048 seeded points with face 11 skipped
                proj_dsq / proj_face / proj_point   findProjection at the same points
  spheres_selfint   calcSelfIntersections bits (uint8) of two overlapping level-3 spheres
  ico_*         the 1,310,720-triangle noisy icosphere (seed 0, level 8) on grid_for(v, 512):
                nodes_digest / dipoles_digest, ids (int64: 2,048 seeded voxels, half of them within
                0.02 diag of the surface), sdf (calcWithDistances at those voxels, as
                calcFromGridWithDistances evaluates them), pts (1,024 points within 1e-3 diag of the
                surface), fwn_pts, proj_dsq
  digest_*      of the generated meshes and points, so a test can tell if a generator changed
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "fwn_cpu_reference.npz")


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def torus_inputs():
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_torus(seed=0)
    dims, xf = mg.grid_for(v, 32)
    rng = np.random.default_rng(2024)
    lo, hi = v.min(0), v.max(0)
    pts = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo), (2048, 3)).astype(np.float32)
    return v, f, dims, xf, pts


def spheres_inputs():
    from meshlib_gb300 import meshgen as mg
    return mg.overlapping_spheres(seed=0, level=3)


def ico_inputs():
    from meshlib_gb300 import meshgen as mg
    v, f = mg.noisy_icosphere(seed=0, level=8)
    dims, xf = mg.grid_for(v, 512)
    return v, f, dims, xf


def ico_samples(v, f, dims, abs_dist):
    """2,048 voxel ids (1,024 uniform, 1,024 within 0.02 diag of the surface, chosen from a seeded pool
    by `abs_dist(ids)`) and 1,024 points within 1e-3 diag of the surface."""
    from meshlib_gb300 import meshgen as mg
    rng = np.random.default_rng(77)
    n = int(np.prod(dims))
    uniform = rng.integers(0, n, 1024)
    pool = rng.integers(0, n, 200_000)
    near = pool[abs_dist(pool) < 0.02 * mg.diag(v)][:1024]
    pts = mg.shell_points(v, f, 1024, 1e-3 * mg.diag(v), seed=5)
    return np.concatenate([uniform, near]).astype(np.int64), pts


def main(out: str = OUT):
    import oracle as O
    import oracle.fwnref as FR
    from oracle.ref import build_cpu_ref
    from meshlib_gb300 import meshgen as mg
    if not build_cpu_ref.build(targets=("libfwnref.so",)):
        raise SystemExit("the reference library could not be built here (no copy of the reference)")
    res = {}
    v, f, dims, xf, pts = torus_inputs()
    R = FR.Reference(v, f)
    diag = mg.diag(v)
    res["torus_nodes_digest"] = np.array(digest(R.nodes()))
    res["torus_dipoles_digest"] = np.array(digest(R.dipoles()))
    res["torus_sdf"] = R.from_grid_with_distances(dims, xf)
    res["torus_sdf_band"] = R.from_grid_with_distances(dims, xf, minDistSq=(0.01 * diag) ** 2, maxDistSq=(0.05 * diag) ** 2)
    res["torus_fwn"] = R.from_grid(dims, xf)
    res["torus_fwn_pts"] = R.from_vector(pts, skip_face=11)
    dsq, face, point, _, _ = R.project(pts)
    res["torus_proj_dsq"], res["torus_proj_face"], res["torus_proj_point"] = dsq, face, point
    res["digest_torus"] = np.array(digest(v, f, pts))
    sv, sf = spheres_inputs()
    res["spheres_selfint"] = FR.Reference(sv, sf).self_intersections().astype(np.uint8)
    res["digest_spheres"] = np.array(digest(sv, sf))
    vi, fi, di, xi = ico_inputs()
    Ri = FR.Reference(vi, fi)
    # near-surface voxels are picked with the oracle's FP32 distances (bit-identical to the reference's)
    oi = O.Oracle(vi, fi)
    ids, ipts = ico_samples(vi, fi, di, lambda p: np.abs(oi.grid_voxels(di, xi, p, prec=0)[0]))
    res["ico_nodes_digest"] = np.array(digest(Ri.nodes()))
    res["ico_dipoles_digest"] = np.array(digest(Ri.dipoles()))
    res["ico_ids"] = ids
    res["ico_sdf"] = Ri.grid_voxels(di, xi, ids)
    res["ico_pts"] = ipts
    res["ico_fwn_pts"] = Ri.from_vector(ipts)
    res["ico_proj_dsq"] = Ri.project(ipts)[0]
    res["digest_ico"] = np.array(digest(vi, fi))
    np.savez_compressed(out, **res)
    print(f"wrote {out} ({os.path.getsize(out)} bytes)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else OUT)
