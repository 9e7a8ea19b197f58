"""Times MeshLib's own CPU signed-distance code (oracle/_ref/libfwnref.so, built from the reference
sources by oracle/ref/build_cpu_ref.py) against the oracle's FP32 port of it (oracle/fwn_oracle.cpp)
on one core, on the same voxels, and checks that both return the same floats.

TEST / BENCH INFRASTRUCTURE ONLY.  The benchmark's CPU baseline is the port (the reference's code
cannot be built on the GPU machine); this measures how the port's speed compares with the
reference code's on a host where both exist.  Workload: calcWithDistances at seeded random voxels of
the 512^3 grid of the 1,310,720-triangle noisy icosphere (as calcFromGridWithDistances evaluates
them, MRMesh/MRFastWindingNumber.cpp:86-93), default options.

    python oracle/ref/calibrate_port.py [voxels, default 20000] [repeats, default 3]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main(n: int = 20000, repeats: int = 3) -> dict:
    import oracle as O
    import oracle.fwnref as FR
    from meshlib_gb300 import meshgen as mg
    from oracle.ref import build_cpu_ref
    if not build_cpu_ref.build(targets=("libfwnref.so",)):
        raise SystemExit("the reference library could not be built here (no copy of the reference)")
    v, f = mg.noisy_icosphere(seed=0, level=8)
    dims, xf = mg.grid_for(v, 512)
    ids = np.random.default_rng(1).integers(0, int(np.prod(dims)), n)
    t0 = time.perf_counter()
    ref = FR.Reference(v, f)
    ref.nodes(), ref.dipoles()
    ref_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    port = O.Oracle(v, f)
    port.nodes()
    port_build = time.perf_counter() - t0
    tr, tp = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        a = ref.grid_voxels(dims, xf, ids)
        tr.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        b, _ = port.grid_voxels(dims, xf, ids, prec=0, threads=1)
        tp.append(time.perf_counter() - t0)
    same = bool(np.array_equal(a.view(np.uint32), b.astype(np.float32).view(np.uint32)))
    res = {"voxels": n, "reference_voxels_per_s": n / min(tr), "port_voxels_per_s": n / min(tp),
           "port_over_reference": min(tr) / min(tp), "bit_identical": same, "cores": 1,
           "reference_tree_build_s": ref_build, "port_tree_build_s": port_build}
    print(json.dumps(res))
    return res


if __name__ == "__main__":
    main(*(int(a) for a in sys.argv[1:]))
