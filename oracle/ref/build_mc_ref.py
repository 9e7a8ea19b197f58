"""Recipe: compile MeshLib's own CPU mesher (MRVoxels/MRMarchingCubes.cpp and the MRMesh units it
calls at run time) into oracle/_ref/libmcref.so, with g++ directly on the reference's sources.

TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie (REF, default
/root/reference) and writes only into oracle/_ref/.  The library pins the mesher oracle
(oracle/mc_oracle.cpp): tests/golden/make_mc_golden.py runs it on seeded volumes and commits the
outputs as tests/golden/mc_reference.npz.  No reference source is copied.  Inputs besides the
reference's sources:
  oracle/ref/stub       forward declarations of the parallel-hashmap names (un-vendored submodule)
  oracle/ref/stub_mc    a working parallel-hashmap stand-in over the standard unordered containers,
                        a serial stand-in for the oneTBB names the units use (tbb/), and
                        declarations standing in for OpenVDB's grid types (openvdb/), whose paths
                        are compiled but never run
  oracle/ref/mc_ref_shims.cpp   no-op timer; aborting stand-ins for the VDB grid, the half-edge
                        mesh builder and the point tree, which the driver never reaches
  oracle/ref/mc_ref_driver.cpp  the C entry points (mcref_run / _get / _free)
Reference units compiled (paths inside the MeshLib project):
  source/MRVoxels/MRMarchingCubes.cpp      the mesher (VolumeMesher, marchingCubesAsTriMesh,
                                           MarchingCubesByParts)
  source/MRMesh/MRSeparationPoint.cpp      per-block vertex storage and numbering
  source/MRMesh/MRBitSet.cpp, MRBitSetParallelFor.cpp, MRVolumeIndexer.cpp, MRParallelFor.cpp,
  MRTbbThreadMutex.cpp, MRSharedThreadSafeOwner.cpp   what those call
Flags: C++23 with std::expected (MeshLib's MR_USE_STD_EXPECTED build), -O2, no floating-point
contraction (the reference's x86-64 build has no FMA either), NDEBUG as in a release build.
Only an x86-64 host with a copy of the reference runs this; the golden file it feeds travels.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT, "libmcref.so")

REF_UNITS = ("MRVoxels/MRMarchingCubes.cpp", "MRMesh/MRSeparationPoint.cpp", "MRMesh/MRBitSet.cpp",
             "MRMesh/MRBitSetParallelFor.cpp", "MRMesh/MRVolumeIndexer.cpp", "MRMesh/MRParallelFor.cpp",
             "MRMesh/MRTbbThreadMutex.cpp", "MRMesh/MRSharedThreadSafeOwner.cpp")
OWN_UNITS = ("mc_ref_driver.cpp", "mc_ref_shims.cpp")


def build(ref: str | None = None, force: bool = False) -> str | None:
    """Builds oracle/_ref/libmcref.so; returns its path, or None where no reference copy is present."""
    ref = ref or os.environ.get("MESHLIB_REFERENCE", "/root/reference")
    src = os.path.join(ref, "source")
    gxx = shutil.which("g++")
    if not os.path.isdir(src) or gxx is None:
        return None
    units = [os.path.join(src, u) for u in REF_UNITS] + [os.path.join(HERE, u) for u in OWN_UNITS]
    missing = [u for u in units if not os.path.exists(u)]
    if missing:
        print(f"build_mc_ref: {missing[0]} not found; reference mesher not built", file=sys.stderr)
        return None
    stubs = [os.path.join(HERE, "stub_mc"), os.path.join(HERE, "stub")]
    newest = max(os.path.getmtime(u) for u in units)
    for d in stubs:
        for root, _, files in os.walk(d):
            newest = max([newest] + [os.path.getmtime(os.path.join(root, f)) for f in files])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    objdir = os.path.join(OUT, "mcref_obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ["-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-DNDEBUG", "-DMR_USE_STD_EXPECTED=1",
             "-include", "memory", "-w", "-I", src] + [f for d in stubs for f in ("-I", d)]

    def compile_one(u):
        o = os.path.join(objdir, os.path.basename(u)[:-4] + ".o")
        r = subprocess.run([gxx] + flags + ["-c", u, "-o", o], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"build_mc_ref: {u}\n{r.stderr[-3000:]}")
        return o

    with ThreadPoolExecutor(min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, units))
    r = subprocess.run([gxx, "-shared", "-Wl,--no-undefined", "-o", LIB] + objs + ["-lpthread"], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError("build_mc_ref: link failed\n" + r.stderr[-3000:])
    return LIB


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print(path or "reference not present; nothing built")
