"""Build the pbf103 shared library (CUDA for sm_103a) in-tree.

The library is the product: ``libpbf103.so`` beside this file, exporting the
C ABI of ``include/pbf103.h``.  Translation units compile in parallel with
nvcc; nothing here needs cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpbf103.so")

SOURCES = ["pbf_kernels.cu", "pbf_engine.cu", "pbf_capi.cu", "pbf_server.cu", "pbf_noalloc.cu", "pbf_particles.cu",
           "pbf_ssf.cu"]
# per-file flags: the screen-space passes round every product and sum on its
# own (no contraction into FMA), as their CPU restatement does
FILE_FLAGS = {"pbf_ssf.cu": ["-fmad=false"]}
HEADERS = ["pbf_internal.h", "pbf_engine.h", "pbf_sort.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    # -ftz=true as the reference's shipped build (cuda_pbf_with_ssf.vcxproj:125-127);
    # division and square root stay IEEE-rounded.  Positions and their
    # differences are never subnormal, so the integer pipeline is unaffected.
    return ["-O3", "-std=c++17", "-lineinfo", "-ftz=true", *ARCH, "-I", INCLUDE, "-I", CSRC,
            "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", *extra]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "pbf103.h")]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *hdrs, __file__]):
            cmd = [nvcc(), *_flags(extra_flags), *FILE_FLAGS.get(src, []), "-c", s, "-o", o]
            if verbose and src == "pbf_kernels.cu":
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out, file=sys.stderr)
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nvcc(), *ARCH, "-shared", *objs, "-o", tmp, "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
