"""Recipe: compile MeshLib's own CPU code for this path from the reference sources, with g++
directly on them, into two libraries under oracle/_ref/:

  libmcref.so   the mesher: MRVoxels/MRMarchingCubes.cpp and the MRMesh units it calls at run time
  libfwnref.so  the winding-number / signed-distance path: MRMesh/MRFastWindingNumber.cpp with the
                mesh, topology builder, AABB tree, dipoles and projection it uses

TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie (REF, default
/root/reference) and writes only into oracle/_ref/.  The libraries pin the oracle: the scripts in
tests/golden/ run them on seeded inputs and commit the outputs (mc_reference.npz,
fwn_cpu_reference.npz); the winding-number library also times the reference code against the
oracle's port on one core.  No reference source is copied.  Inputs besides the reference's sources:
  oracle/ref/stub       forward declarations of the parallel-hashmap names (un-vendored submodule)
  oracle/ref/stub_mc    a working parallel-hashmap stand-in over the standard unordered containers
                        (one sub-map), a serial stand-in for the oneTBB names the units use (tbb/),
                        and declarations standing in for OpenVDB's grid types (openvdb/), whose
                        paths are compiled but never run
  oracle/ref/*_shims.cpp  no-op timer; aborting stand-ins for functions the drivers never reach
                        whose units need libraries absent here (OpenVDB, Eigen, boost, spdlog)
  oracle/ref/*_driver.cpp the C entry points
Flags: C++23 with std::expected (MeshLib's MR_USE_STD_EXPECTED build), -O2, no floating-point
contraction (the reference's x86-64 build has no FMA either), NDEBUG as in a release build.
Every parallel loop runs serially (the TBB stand-in), so the libraries compute on one core.
Only an x86-64 host with a copy of the reference runs this; the golden files it feeds travel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")

TARGETS = {
    "libmcref.so": (
        ("MRVoxels/MRMarchingCubes.cpp", "MRMesh/MRSeparationPoint.cpp", "MRMesh/MRBitSet.cpp",
         "MRMesh/MRBitSetParallelFor.cpp", "MRMesh/MRVolumeIndexer.cpp", "MRMesh/MRParallelFor.cpp",
         "MRMesh/MRTbbThreadMutex.cpp", "MRMesh/MRSharedThreadSafeOwner.cpp"),
        ("mc_ref_driver.cpp", "mc_ref_shims.cpp")),
    "libfwnref.so": (
        tuple("MRMesh/MR" + u + ".cpp" for u in (
            "FastWindingNumber", "Dipole", "AABBTree", "AABBTreePoints", "MeshProject", "Mesh", "MeshTopology",
            "MeshBuilder", "MeshMath", "MeshTriPoint", "EdgePoint", "EdgeMetric", "EdgePaths", "EdgePathsBuilder",
            "ComputeBoundingBox", "BitSet", "BitSetParallelFor", "IdentifyVertices", "Order", "ParallelFor",
            "PartMappingAdapters", "ProgressReadWrite", "RegionBoundary", "SharedThreadSafeOwner", "TbbThreadMutex",
            "VertDuplication")),
        ("fwn_ref_driver.cpp", "fwn_ref_shims.cpp")),
}


def _newest(paths):
    t = 0.0
    for p in paths:
        if os.path.isdir(p):
            for root, _, files in os.walk(p):
                t = max([t] + [os.path.getmtime(os.path.join(root, f)) for f in files])
        else:
            t = max(t, os.path.getmtime(p))
    return t


def build(ref: str | None = None, force: bool = False, targets=None) -> dict | None:
    """Builds the libraries; returns {name: path}, or None where no reference copy is present."""
    ref = ref or os.environ.get("MESHLIB_REFERENCE", "/root/reference")
    src = os.path.join(ref, "source")
    gxx = shutil.which("g++")
    if not os.path.isdir(src) or gxx is None:
        return None
    stubs = [os.path.join(HERE, "stub_mc"), os.path.join(HERE, "stub")]
    flags = ["-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-DNDEBUG", "-DMR_USE_STD_EXPECTED=1",
             "-include", "memory", "-w", "-I", src] + [f for d in stubs for f in ("-I", d)]
    objdir = os.path.join(OUT, "cpuref_obj")
    os.makedirs(objdir, exist_ok=True)
    out = {}
    for name, (ref_units, own_units) in TARGETS.items():
        if targets and name not in targets:
            continue
        units = [os.path.join(src, u) for u in ref_units] + [os.path.join(HERE, u) for u in own_units]
        missing = [u for u in units if not os.path.exists(u)]
        if missing:
            print(f"build_cpu_ref: {missing[0]} not found; {name} not built", file=sys.stderr)
            continue
        lib = os.path.join(OUT, name)
        if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _newest(units + stubs + [__file__]):
            out[name] = lib
            continue

        def compile_one(u):
            o = os.path.join(objdir, os.path.basename(u)[:-4] + ".o")
            if not force and os.path.exists(o) and os.path.getmtime(o) >= _newest([u] + stubs):
                return o
            r = subprocess.run([gxx] + flags + ["-c", u, "-o", o], capture_output=True, text=True)
            if r.returncode:
                raise RuntimeError(f"build_cpu_ref: {u}\n{r.stderr[-3000:]}")
            return o

        with ThreadPoolExecutor(min(8, os.cpu_count() or 1)) as ex:
            objs = list(ex.map(compile_one, units))
        r = subprocess.run([gxx, "-shared", "-Wl,--no-undefined", "-o", lib] + objs + ["-lpthread"], capture_output=True,
                           text=True)
        if r.returncode:
            raise RuntimeError(f"build_cpu_ref: link of {name} failed\n" + r.stderr[-3000:])
        out[name] = lib
    return out


if __name__ == "__main__":
    built = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print(built if built is not None else "reference not present; nothing built")
