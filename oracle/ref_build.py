"""Build the reference's own CUDA step for pinning the oracle — TEST INFRASTRUCTURE ONLY.

The reference (yodaplusplus/ssf_pbf_cuda) is an MSVC/CUDA 7 project.  Its
solver (src/pbf/**) compiles with nvcc 13 for sm_103a after four mechanical
changes, which this recipe applies to a scratch copy under oracle/_ref/src
(git-ignored, never committed):
  1. backslashes in #include paths become slashes (<cub\\cub.cuh> ...);
  2. src/common/common_core.h, which pulls in GLEW/GLFW/GL interop for the
     renderer, is replaced by a stub with only <cuda_runtime.h> and GLM;
  3. `auto& grid_size = ...getGridSize();` (binding a non-const reference to
     a temporary, accepted only by MSVC) becomes `auto grid_size = ...`
     in pbf_xsph.cu and pbf_vorticity_confinement.cu;
  4. GLM_FORCE_CUDA is not defined (GLM 0.9.7 rejects CUDA 13 with it).
Two more, active only in the "cub" variant (-DUSE_CUB, the reference's
stable cub::DeviceRadixSort::SortPairs path, pbf_neighbor_search.cpp:123-131),
which does not compile as shipped:
  5. the detectNeighbors overload that path calls (with the sorted hash and
     index arrays, pbf_neighbor_search.cpp:129-131) is missing from
     pbf_neighbor_search_util.h:67-73; a forwarding overload is appended
     (the kernel it would launch ignores those arrays: it is passed nullptr
     for them, pbf_neighbor_search_util.cu:868-869);
  6. the radix sort's temporary storage is sized as the commented-out lines
     pbf_neighbor_search.cpp:39-41 did, instead of the counting sort's scan
     storage (:44-46).
That path skips deletion (pbf_neighbor_search.cpp:146-159), so it is run only
on scenes that keep every particle inside the simulation area.
The copy is made where the reference is mounted (prepare; the location comes
from $PBF_REFERENCE_ROOT or --root, default /root/reference); the build runs
wherever nvcc is (a machine of another architecture builds its own binary from the copy).
Outputs go only to oracle/_ref/.  The reference's own build files are not used.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PBF_REFERENCE_ROOT", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
PBF_REL = os.path.join("cuda_pbf_with_ssf", "src", "pbf")
GLM_REL = os.path.join("external", "include", "glm")

STUB_CORE = """#pragma once
// stub of the renderer's common header: the solver needs only CUDA and GLM
#include <cuda_runtime.h>
#include <glm/glm.hpp>
"""

VARIANTS = {
    # IEEE division / square root (parity is asserted against this build)
    "ieee": [],
    # the shipped flags (cuda_pbf_with_ssf.vcxproj:125-127)
    "fast": ["-use_fast_math", "-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    # IEEE, with the stable radix-sort path (changes 5 and 6 above)
    "cub": ["-DUSE_CUB"],
}

# change 5: appended inside namespace pbf::cuda of pbf_neighbor_search_util.h
CUB_OVERLOAD = """
#ifdef USE_CUB
// test-side shim: the overload pbf_neighbor_search.cpp calls under USE_CUB
inline void detectNeighbors(uint32_t *neighbor_list, const dom_dim *position, const uint32_t *, const uint32_t *,
                            const uint32_t *cell_start, const uint32_t *cell_end, scalar_t cell_width,
                            dom_udim grid_size, scalar_t h, uint32_t num_particle, uint32_t max_pair_particle_num)
{
    detectNeighbors(neighbor_list, position, cell_start, cell_end, cell_width, grid_size, h, num_particle,
                    max_pair_particle_num);
}
#endif
"""
# change 6: the scan-storage sizing line of the neighbor_search constructor
SCAN_SIZING = "cuda::getPrefixSumStorageSize(temp_cub_storage_size, cell_num);"
CUB_SIZING = """
#ifdef USE_CUB
	cuda::getRadixSortStorageSize(temp_cub_storage_size, max_particle_num);
#else
	cuda::getPrefixSumStorageSize(temp_cub_storage_size, cell_num);
#endif
"""


def present() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, PBF_REL))


def prepare() -> bool:
    """Copy the solver sources (and GLM) into oracle/_ref/src with the
    mechanical changes.  Returns False when the reference is not mounted."""
    if not present():
        return False
    if os.path.isdir(SRC):
        shutil.rmtree(SRC)
    shutil.copytree(os.path.join(REF_ROOT, PBF_REL), os.path.join(SRC, "pbf"))
    shutil.copytree(os.path.join(REF_ROOT, GLM_REL), os.path.join(SRC, "include", "glm"))
    os.makedirs(os.path.join(SRC, "common"), exist_ok=True)
    with open(os.path.join(SRC, "common", "common_core.h"), "w") as f:
        f.write(STUB_CORE)
    inc = re.compile(r'(#\s*include\s*[<"])([^>"]*)([>"])')
    for dirpath, _, files in os.walk(os.path.join(SRC, "pbf")):
        for fn in files:
            p = os.path.join(dirpath, fn)
            if not fn.endswith((".cu", ".cpp", ".h", ".cuh", ".inl")):
                continue
            s = open(p, encoding="latin-1").read()
            s2 = inc.sub(lambda m: m.group(1) + m.group(2).replace("\\", "/") + m.group(3), s)
            s2 = s2.replace("auto& grid_size = ns->getGridSize();", "auto grid_size = ns->getGridSize();")
            s2 = s2.replace("auto& grid_size = ns.getGridSize();", "auto grid_size = ns.getGridSize();")
            if fn == "pbf_neighbor_search_util.h":
                tail = "}\t// end of cuda ns"
                assert s2.count(tail) == 1, "pbf_neighbor_search_util.h: namespace end not found"
                s2 = s2.replace(tail, CUB_OVERLOAD + tail)
            if fn == "pbf_neighbor_search.cpp":
                assert s2.count(SCAN_SIZING) == 1, "pbf_neighbor_search.cpp: scan sizing not found"
                s2 = s2.replace(SCAN_SIZING, CUB_SIZING)
            if s2 != s:
                open(p, "w", encoding="latin-1").write(s2)
    return True


def sources() -> list:
    out = []
    for dirpath, _, files in os.walk(os.path.join(SRC, "pbf")):
        if os.path.basename(dirpath) == "neighbor_search":  # unused older header only
            continue
        for fn in sorted(files):
            if fn.endswith((".cu", ".cpp")):
                out.append(os.path.join(dirpath, fn))
    return sorted(out)


def binary(variant: str) -> str:
    return os.path.join(OUT, f"pbf_ref_step_{variant}")


def build(variant: str = "ieee", jobs: int = 16) -> str:
    """Compile the copied sources + oracle/ref_driver.cu with nvcc -rdc."""
    if not os.path.isdir(SRC):
        raise FileNotFoundError("oracle/_ref/src missing: run prepare() where the reference is mounted")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    objdir = os.path.join(OUT, f"obj_{variant}")
    os.makedirs(objdir, exist_ok=True)
    flags = ["-O2", "-std=c++17", "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a",
             "-I", SRC, "-I", os.path.join(SRC, "include"), "-w", *VARIANTS[variant]]
    srcs = sources() + [os.path.join(HERE, "ref_driver.cu")]
    exe = binary(variant)
    if os.path.exists(exe) and os.path.getmtime(exe) > max(os.path.getmtime(s) for s in srcs + [__file__]):
        # built from these sources already (the binary runs only where it was built:
        # a machine of another architecture has none)
        return exe
    objs = []

    def cc(s):
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        r = subprocess.run([nvcc, *flags, "-x", "cu", "-c", s, "-o", o], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"nvcc failed on {s}:\n{r.stderr[-4000:]}")
        return o

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(cc, srcs))
    exe = binary(variant)
    r = subprocess.run([nvcc, "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", exe],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return exe


def build_if_present() -> None:
    """Called by the package build: copy (and compile) the reference only on the
    machine where it is mounted; elsewhere the copied sources, if any, are used
    by tests/golden/make_golden.py."""
    if present():
        prepare()


if __name__ == "__main__":
    if "--root" in sys.argv:
        REF_ROOT = sys.argv[sys.argv.index("--root") + 1]
    if "--prepare" in sys.argv or present():
        prepare()
    for v in ([a for a in sys.argv[1:] if a in VARIANTS] or ["ieee"]):
        print(build(v))
