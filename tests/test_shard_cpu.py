"""Multi-GPU sharding logic on CPU: z-slab partition, LPT batch partition, and a world-size-2 gloo run
in which each rank computes its slab (here with the CPU oracle standing in for the GPU) and rank 0
gathers the whole grid, which must equal the single-process grid exactly."""
import os
import socket

import numpy as np
import pytest

from meshlib_gb300 import shard


def test_zslabs_cover_exactly():
    for nz in (0, 1, 5, 64, 513):
        for world in (1, 2, 3, 8):
            s = shard.zslabs(nz, world)
            assert len(s) == world and s[0][0] == 0 and s[-1][1] == nz
            assert all(a <= b for a, b in s) and all(s[i][1] == s[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in s]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.zslabs(4, 0)


def test_lpt_balances_the_batched_workload():
    rng = np.random.default_rng(0)
    tris = np.exp(rng.uniform(np.log(5000), np.log(500000), 64)).astype(int)
    sides = np.exp(rng.uniform(np.log(32), np.log(192), 64)).astype(int)
    costs = [shard.batch_cost(t, s ** 3) for t, s in zip(tris, sides)]
    for world in (2, 4, 8):
        parts = shard.lpt(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(64))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT guarantee: max load <= 4/3 of the optimum, and the optimum >= max(mean, largest item)
        bound = max(sum(costs) / world, max(costs))
        assert max(loads) <= 4 / 3 * bound + 1e-6


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_path):
    import torch.distributed as dist

    import oracle as O
    from meshlib_gb300 import meshgen as mg
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        v, f = mg.noisy_torus(seed=0, nu=32, nv=16)
        dims, xf = mg.grid_for(v, 12)
        z0, z1 = shard.zslabs(int(dims[2]), world)[rank]
        pts = O.grid_points(dims, xf).reshape(int(dims[2]), -1, 3)[z0:z1].reshape(-1, 3)
        local = O.Oracle(v, f).vector_with_distances(pts, threads=1).astype(np.float32)
        full = shard.gather_slabs(local, dims, rank, world)
        if rank == 0:
            np.save(result_path, full)
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_gather_equals_whole_grid(tmp_path):
    import torch.multiprocessing as mp

    import oracle as O
    from meshlib_gb300 import meshgen as mg
    world, port = 2, _free_port()
    out = str(tmp_path / "full.npy")
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    got = np.load(out)
    v, f = mg.noisy_torus(seed=0, nu=32, nv=16)
    dims, xf = mg.grid_for(v, 12)
    ref = O.Oracle(v, f).vector_with_distances(O.grid_points(dims, xf), threads=1).astype(np.float32)
    assert np.array_equal(got, ref)
