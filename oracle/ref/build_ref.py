"""Recipe: compile the reference's own GPU kernels (MRCuda/MRCudaFastWindingNumber.cu and
MRCuda/MRCudaPointsToMeshProjector.cu) for sm_103a.

TEST / BENCH INFRASTRUCTURE ONLY.  Reads the reference sources where they lie (REF, default
/root/reference) and writes only into oracle/_ref/:
  mrcuda_fwn.cubin   device code of the four reference kernels (signedDistanceKernel,
                     fastWindingNumberFrom{Grid,Vector,Mesh}Kernel) in the reference's release
                     configuration: -use_fast_math (cmake/Modules/CudaCompilerOptions.cmake) and
                     CMake's release flags -O3 -DNDEBUG (so the kernels' device asserts are off)
  mrcuda_fwn.ptx     the same as PTX, used when a machine drops the cubin
  mrcuda_proj.*      the points-to-mesh projection kernel (MRCuda/MRCudaPointsToMeshProjector.cu)
No reference source is copied; the only extra input is oracle/ref/stub (forward declarations of the
un-vendored parallel-hashmap names).  The host launchers of the reference (.cu:245-274) are not
used: oracle/mrcuda_runner.cpp launches the kernels through the driver API with the same grid shape
(32 threads per block).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")


UNITS = (("MRCudaFastWindingNumber.cu", "mrcuda_fwn"), ("MRCudaPointsToMeshProjector.cu", "mrcuda_proj"))


def build(ref: str | None = None) -> bool:
    ref = ref or os.environ.get("MESHLIB_REFERENCE", "/root/reference")
    if not os.path.isdir(ref):  # no copy of the reference on this machine: keep what oracle/_ref holds
        return False
    ok = True
    for unit, stem in UNITS:
        src = os.path.join(ref, "source", "MRCuda", unit)
        if not os.path.exists(src):
            print(f"build_ref: {src} not found; reference kernels not built", file=sys.stderr)
            return False
        os.makedirs(OUT, exist_ok=True)
        common = ["nvcc", "-O3", "-DNDEBUG", "-use_fast_math", "-std=c++20", "-I" + os.path.join(ref, "source"),
                  "-I" + os.path.join(ref, "source", "MRCuda"), "-I" + os.path.join(HERE, "stub"), src]
        for kind, arch, ext in (("-cubin", "arch=compute_103a,code=sm_103a", ".cubin"),
                                ("-ptx", "arch=compute_103a,code=compute_103a", ".ptx")):
            dst = os.path.join(OUT, stem + ext)
            if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
                continue
            r = subprocess.call(common[:1] + [kind, "-gencode", arch] + common[1:] + ["-o", dst])
            ok = ok and r == 0
    return ok


if __name__ == "__main__":
    sys.exit(0 if build(sys.argv[1] if len(sys.argv) > 1 else None) else 1)
