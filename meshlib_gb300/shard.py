"""Multi-GPU sharding of the signed-distance path: one process per GPU, no collective on the data path.

Every voxel, point and face query is independent given the read-only mesh data, so the work splits
into independent units (the by-parts unit of MRMesh/MRFastWindingNumber.h:96-106 and
MRMesh/MRChunkIterator.h:44-47):

* one grid  -> contiguous z-slabs, one per rank (`zslabs`), each computed with the slab entry point
  (`FastWindingNumber.calcFromGridWithDistancesSlab_dev`), bit-identical to the whole-grid call;
* many meshes (the batched workload) -> whole meshes per rank, longest-processing-time-first by the
  estimated cost voxels x log2(triangles) (`lpt`), the same cost the batched launch orders by.

The mesh is replicated on every rank.  The only communication is the optional gather of finished
slabs to one rank (`gather_slabs`, point-to-point sends of host tensors), outside the compute.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np


def zslabs(nz: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous layer ranges [z0, z1) per rank covering [0, nz); the first nz % world ranks take one
    layer more.  Ranks beyond nz get an empty range (z0 == z1)."""
    if nz < 0 or world <= 0:
        raise ValueError("zslabs: nz >= 0 and world > 0")
    base, extra = divmod(nz, world)
    out, z = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((z, z + n))
        z += n
    return out


def batch_cost(triangles: int, voxels: int) -> float:
    """Estimated cost of one mesh + grid of the batched workload."""
    return float(voxels) * math.log2(max(int(triangles), 2))


def lpt(costs: Sequence[float], world: int) -> List[List[int]]:
    """Longest processing time first: items sorted by cost, each to the least loaded rank (ties to
    the lower rank).  Returns the item indices of every rank."""
    if world <= 0:
        raise ValueError("lpt: world > 0")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return parts


def rank_signed_distance(fwn, dims, xf, rank: int, world: int, options=None, stream=None):
    """This rank's slab of the signed-distance grid on its GPU: (z0, z1, device tensor of
    (z1 - z0) * nx * ny floats).  An empty slab returns an empty tensor without a launch."""
    import torch

    z0, z1 = zslabs(int(dims[2]), world)[rank]
    out = torch.empty((z1 - z0) * int(dims[0]) * int(dims[1]), dtype=torch.float32, device="cuda")
    if z1 > z0:
        fwn.calcFromGridWithDistancesSlab_dev(dims, xf, z0, z1, out.data_ptr(), options=options, stream=stream)
    return z0, z1, out


def gather_slabs(local: "np.ndarray", dims, rank: int, world: int, dst: int = 0, group=None):
    """Stacks every rank's slab (host float32 arrays, zslabs order) into the whole grid on rank dst;
    other ranks return None.  Uses point-to-point sends (works on gloo and nccl process groups)."""
    import torch
    import torch.distributed as dist

    nx, ny, nz = int(dims[0]), int(dims[1]), int(dims[2])
    slabs = zslabs(nz, world)
    z0, z1 = slabs[rank]
    local = np.ascontiguousarray(local, np.float32).reshape(-1)
    if local.size != (z1 - z0) * nx * ny:
        raise ValueError("gather_slabs: local slab has the wrong size")
    if rank != dst:
        if local.size:
            dist.send(torch.from_numpy(local), dst, group=group)
        return None
    full = np.empty(nx * ny * nz, np.float32)
    for r, (a, b) in enumerate(slabs):
        if b == a:
            continue
        if r == dst:
            full[a * nx * ny:b * nx * ny] = local
        else:
            buf = torch.empty((b - a) * nx * ny, dtype=torch.float32)
            dist.recv(buf, r, group=group)
            full[a * nx * ny:b * nx * ny] = buf.numpy()
    return full
