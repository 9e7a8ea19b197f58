"""Seeded synthetic meshes, grids and query sets for the winding-number workloads.

The reference project's own fixtures (``test_data/``) are not available, so every
workload is generated here from a seed.  Conventions:

* noisy torus: major radius R, minor radius r, ``nu x nv`` quads split into two
  triangles each; every vertex moves along its torus normal by
  ``amp * sum_{k=1..4} sin(k*u + phi_k) * sin(k*v + psi_k)`` with phases drawn
  uniformly from [0, 2*pi) by the seed;
* noisy icosphere: a regular icosahedron subdivided ``level`` times by edge
  midpoints projected on the unit sphere (20*4**level triangles), then every
  vertex scaled radially by ``1 + amp * fbm(p)``, where ``fbm`` is seeded 3D
  value noise (lattice values uniform in [-1, 1], smoothstep trilinear
  interpolation), ``octaves`` octaves, base frequency 2, lacunarity 2, gain 0.5,
  normalised by the sum of the octave gains;
* grid over the mesh bounding box padded by 10 % of its extent on every side,
  voxel centres at ``origin + (i + 0.5) * voxel`` -- the basis that
  ``meshToDistanceVolume`` hands to ``calcFromGridWithDistances``
  (MRVoxels/MRMeshToDistanceVolume.cpp:55).

All triangles are oriented outward (positive signed volume), so the winding
number is ~1 inside and ~0 outside.
"""
from __future__ import annotations

import math

import numpy as np


def _orient_outward(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    a, b, c = (verts[faces[:, k]].astype(np.float64) for k in range(3))
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    if vol < 0:
        faces = faces[:, [0, 2, 1]]
    return np.ascontiguousarray(faces, dtype=np.int32)


def noisy_torus(seed: int = 0, R: float = 1.0, r: float = 0.3, nu: int = 128, nv: int = 64, amp: float = 0.02):
    """Torus with 2*nu*nv triangles (16,384 at the defaults), displaced along its normals."""
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0, 2 * np.pi, 4)
    psi = rng.uniform(0, 2 * np.pi, 4)
    u = 2 * np.pi * np.arange(nu) / nu
    v = 2 * np.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    disp = np.zeros_like(U)
    for k in range(1, 5):
        disp += np.sin(k * U + phi[k - 1]) * np.sin(k * V + psi[k - 1])
    disp *= amp
    n = np.stack([np.cos(V) * np.cos(U), np.cos(V) * np.sin(U), np.sin(V)], -1)
    p = np.stack([(R + r * np.cos(V)) * np.cos(U), (R + r * np.cos(V)) * np.sin(U), r * np.sin(V)], -1)
    p = p + disp[..., None] * n
    verts = p.reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i1, j1 = (i + 1) % nu, (j + 1) % nv
    a = (i * nv + j).ravel()
    b = (i1 * nv + j).ravel()
    c = (i1 * nv + j1).ravel()
    d = (i * nv + j1).ravel()
    faces = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], 0)
    return verts, _orient_outward(verts, faces)


def figure8_torus(R: float = 1.0, r: float = 0.3, nu: int = 32, nv: int = 32):
    """Torus whose tube section is a figure-eight (x = -r cos a, z = r sin 2a): a closed surface that
    crosses itself along two circles, like the reference's makeTorusWithSelfIntersections test mesh."""
    a = 2 * np.pi * np.arange(nv) / nv
    b = 2 * np.pi * np.arange(nu) / nu
    A, B = np.meshgrid(a, b, indexing="ij")
    rad = R - r * np.cos(A)
    p = np.stack([rad * np.cos(B), rad * np.sin(B), r * np.sin(2 * A)], -1)
    verts = p.reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    i1, j1 = (i + 1) % nv, (j + 1) % nu
    a0 = (i * nu + j).ravel()
    b0 = (i * nu + j1).ravel()
    c0 = (i1 * nu + j1).ravel()
    d0 = (i1 * nu + j).ravel()
    faces = np.concatenate([np.stack([a0, b0, c0], 1), np.stack([a0, c0, d0], 1)], 0).astype(np.int32)
    return verts, faces


def icosphere(level: int):
    """Unit icosphere with 20*4**level triangles and 10*4**level+2 vertices (float64 positions)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        nvert = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        key = np.minimum(e[:, 0], e[:, 1]) * nvert + np.maximum(e[:, 0], e[:, 1])
        uk, inv = np.unique(key, return_inverse=True)
        ea, eb = uk // nvert, uk % nvert
        mid = v[ea] + v[eb]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + nvert  # midpoint ids of edges (01, 12, 20) per face
        m01, m12, m20 = m[0], m[1], m[2]
        v = np.concatenate([v, mid], 0)
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)], 0)
    return v, f


def _value_noise(p: np.ndarray, perm: np.ndarray, vals: np.ndarray) -> np.ndarray:
    i0 = np.floor(p).astype(np.int64)
    fr = p - i0
    w = fr * fr * (3 - 2 * fr)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                ix, iy, iz = (i0[:, 0] + dx) & 255, (i0[:, 1] + dy) & 255, (i0[:, 2] + dz) & 255
                h = perm[(perm[(perm[ix] + iy) & 255] + iz) & 255]
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += wx * wy * wz * vals[h]
    return out


def fbm(p: np.ndarray, seed: int, octaves: int = 6, lacunarity: float = 2.0, gain: float = 0.5, base_freq: float = 2.0):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    vals = rng.uniform(-1.0, 1.0, 256)
    acc = np.zeros(len(p))
    norm = 0.0
    freq, g = base_freq, 1.0
    for _ in range(octaves):
        acc += g * _value_noise(p * freq, perm, vals)
        norm += g
        freq *= lacunarity
        g *= gain
    return acc / norm


def noisy_icosphere(seed: int = 0, level: int = 8, amp: float = 0.05, octaves: int = 6):
    """Icosphere (1,310,720 triangles at level 8) with seeded radial value-noise displacement."""
    v, f = icosphere(level)
    v = v * (1.0 + amp * fbm(v, seed, octaves))[:, None]
    verts = v.astype(np.float32)
    return verts, _orient_outward(verts, f.astype(np.int32))


def fold_faces(verts: np.ndarray, faces: np.ndarray, frac: float = 0.01, depth: float = 0.1, seed: int = 0):
    """Pushes the vertices of a seeded ``frac`` of the faces inward along the radial direction by
    ``depth``.  On a sphere this digs narrow pits whose walls stay inside the solid and cross no
    other part of the surface, so no face becomes self-intersecting; ``overlapping_spheres`` gives a
    surface that does cross itself."""
    rng = np.random.default_rng(seed + 7919)
    nf = len(faces)
    chosen = rng.choice(nf, max(1, int(round(frac * nf))), replace=False)
    vs = np.unique(faces[chosen].ravel())
    out = verts.astype(np.float64).copy()
    rad = np.linalg.norm(out[vs], axis=1, keepdims=True)
    out[vs] *= np.maximum(rad - depth, 0.05 * rad) / rad
    return out.astype(np.float32), faces


def grid_for(verts: np.ndarray, n: int, pad: float = 0.1):
    """``(dims, xf)`` of an n^3 grid over the bounding box padded by ``pad`` of its extent per side.
    ``xf`` is the 12-float affine map (3x3 row-major A, then b) from voxel indices to voxel centres."""
    lo = verts.min(0).astype(np.float64)
    hi = verts.max(0).astype(np.float64)
    ext = hi - lo
    lo = lo - pad * ext
    hi = hi + pad * ext
    vox = (hi - lo) / n
    xf = np.zeros(12, np.float32)
    xf[0], xf[4], xf[8] = vox
    xf[9:12] = lo + 0.5 * vox
    return (n, n, n), xf


def diag(verts: np.ndarray) -> float:
    return float(np.linalg.norm(verts.max(0).astype(np.float64) - verts.min(0).astype(np.float64)))


def shell_points(verts: np.ndarray, faces: np.ndarray, n: int, width: float = 1e-3, seed: int = 0) -> np.ndarray:
    """n points near the surface: a uniformly chosen triangle, a uniform barycentric sample on it,
    then an offset along the triangle normal drawn from U(-width, width)."""
    rng = np.random.default_rng(seed + 104729)
    f = rng.integers(0, len(faces), n)
    a, b, c = (verts[faces[f, k]].astype(np.float64) for k in range(3))
    r1, r2 = rng.random(n), rng.random(n)
    s = np.sqrt(r1)
    p = (1 - s)[:, None] * a + (s * (1 - r2))[:, None] * b + (s * r2)[:, None] * c
    nrm = np.cross(b - a, c - a)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    p += rng.uniform(-width, width, n)[:, None] * nrm
    return p.astype(np.float32)


def batch_meshes(count: int = 64, seed: int = 0, tri_lo: int = 5000, tri_hi: int = 500000, side_lo: int = 32, side_hi: int = 192):
    """Uneven batch: triangle counts and grid sides log-uniform in the given ranges; even-indexed
    meshes are noisy tori, odd ones noisy icospheres (the icosphere level is the one whose
    triangle count is closest to the drawn count)."""
    rng = np.random.default_rng(seed + 31337)
    out = []
    for i in range(count):
        nt = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        side = int(round(math.exp(rng.uniform(math.log(side_lo), math.log(side_hi)))))
        s = int(rng.integers(0, 2**31 - 1))
        if i % 2 == 0:
            nv = max(8, int(round(math.sqrt(nt / 4))))
            nu = max(8, int(round(nt / (2 * nv))))
            v, f = noisy_torus(seed=s, nu=nu, nv=nv)
        else:
            lvl = int(np.clip(round(math.log(nt / 20) / math.log(4)), 1, 8))
            v, f = noisy_icosphere(seed=s, level=lvl)
        dims, xf = grid_for(v, side)
        out.append((v, f, dims, xf))
    return out


def overlapping_spheres(seed: int = 0, level: int = 7, offset: float = 0.5):
    """Two noisy icospheres, the second shifted by `offset` along x, as one triangle list: a
    self-intersecting surface whose faces inside the other sphere have centroid winding number
    about 1.5."""
    v1, f1 = noisy_icosphere(seed=seed, level=level)
    v2, f2 = noisy_icosphere(seed=seed + 1, level=level)
    v2 = v2 + np.array([offset, 0, 0], np.float32)
    return np.concatenate([v1, v2]), np.concatenate([f1, f2 + len(v1)]).astype(np.int32)
