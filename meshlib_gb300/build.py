"""Builds the in-tree CUDA library ``meshlib_gb300/libgbfwn.so`` for sm_103a with nvcc.

Translation units are compiled in parallel, then linked with the static CUDA runtime, so the
library only needs the NVIDIA driver at run time.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbfwn.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden,-ffp-contract=off", "--expt-relaxed-constexpr"]
# build.cu must round every float operation separately (bit-identical boxes and dipoles)
PER_FILE = {"build.cu": ["-fmad=false"], "treebuild.cu": ["-fmad=false"]}
SOURCES = ["capi.cu", "build.cu", "treebuild.cu", "query.cu", "columns.cu", "mlp_gemm.cu", "mlp_net.cu", "mlp_train.cu", "surrogate.cu", "batch.cu", "sort.cu",
           "projector.cu", "mc.cu"]
# measurement support for bench.py (the FP32 FMA peak), kept out of the product library
BENCH_SOURCES = ["bench/fp32_peak.cu"]
BENCH_LIB = os.path.join(HERE, "libgbfwn_bench.so")


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _needs(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "gbfwn.h"))
    objs, bench_objs, jobs = [], [], []
    for src in SOURCES + BENCH_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace("/", "_") + ".o")
        (bench_objs if src in BENCH_SOURCES else objs).append(o)
        if force or _needs(o, [s] + headers + [__file__]):
            cmd = [nvcc()] + ARCH + COMMON + PER_FILE.get(src, []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-Xlinker", "--no-undefined"]
        run(cmd)
    if jobs or not os.path.exists(BENCH_LIB):
        run([nvcc()] + ARCH + ["-shared", "-o", BENCH_LIB] + bench_objs + ["-Xlinker", "--no-undefined"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
