"""Golden points of the reference's arrangement generators.

Builds oracle/ref_arrangement.cpp against the reference's own
src/pbf/util/pbf_arrangement.h (the copy oracle/ref_build.py prepares under
oracle/_ref/src, where the reference is mounted), runs it on CASES and
writes tests/golden/arrangements/points.npz:

    python tests/golden/make_arrangement_golden.py
"""
from __future__ import annotations

import os
import shutil
import struct
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402

# (kind, keyword arguments of oracle/arrangement.py) — spacings and extents of
# the reference's scenes (dam / sphere init, the sphere scene's jet) and
# edge cases: a degenerate axis, an empty range, negative coordinates
CASES = [
    ("volume", dict(origin=(2.25, 2.25, 2.25), end=(5.65, 5.65, 5.65), space=0.2)),
    ("volume", dict(origin=(0.05, 0.05, 0.05), end=(1.6, 1.6, 1.6), space=0.05)),
    ("volume", dict(origin=(-0.3, 0.1, -1.0), end=(0.3, 0.1, 1.0), space=0.07)),
    ("volume", dict(origin=(1.0, 1.0, 1.0), end=(0.5, 2.0, 2.0), space=0.1)),
    ("rectangle", dict(axis="x", axis_value=1.25, origin2=(3.5, 2.5), end2=(4.5, 3.5), space=0.05)),
    ("rectangle", dict(axis="y", axis_value=0.7, origin2=(0.1, -0.4), end2=(1.3, 0.35), space=0.05)),
    ("rectangle", dict(axis="z", axis_value=-2.0, origin2=(0.0, 0.0), end2=(0.45, 0.9), space=0.1)),
    ("line", dict(origin=(0.0, 0.0, 0.0), end=(1.0, 2.0, 3.0), space=0.05)),
    ("line", dict(origin=(0.5, -0.25, 2.0), end=(0.5, 1.75, 2.0), space=0.1)),
    ("cylinder", dict(axis="x", axis_value=3.0, origin2=(3.0, 3.0), radius=0.8, height=0.2, space=0.05)),
    ("cylinder", dict(axis="y", axis_value=0.5, origin2=(1.0, 2.0), radius=0.3, height=0.35, space=0.07)),
    ("cylinder", dict(axis="z", axis_value=-1.0, origin2=(0.0, 0.0), radius=1.5, height=0.1, space=0.1)),
]


def case_line(kind: str, kw: dict) -> str:
    f = lambda *a: " ".join(repr(float(t)) for t in a)  # noqa: E731
    if kind in ("volume", "line"):
        return f"{kind} {f(*kw['origin'], *kw['end'], kw['space'])}"
    if kind == "rectangle":
        return f"rectangle {kw['axis']} {f(kw['axis_value'], *kw['origin2'], *kw['end2'], kw['space'])}"
    return (f"cylinder {kw['axis']} "
            f"{f(kw['axis_value'], *kw['origin2'], kw['radius'], kw['height'], kw['space'])}")


def build() -> str:
    src = os.path.join(ref_build.SRC)
    if not os.path.isdir(src):
        if not ref_build.prepare():
            raise SystemExit("the reference is not mounted and oracle/_ref/src is missing")
    exe = os.path.join(ref_build.OUT, "ref_arrangement")
    cxx = shutil.which("g++") or "g++"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-I", src, "-I",
                    os.path.join(src, "include"), "-I", "/usr/local/cuda/include",
                    os.path.join(ROOT, "oracle", "ref_arrangement.cpp"), "-o", exe], check=True)
    return exe


def run(exe: str) -> list:
    text = "\n".join(case_line(k, kw) for k, kw in CASES) + "\n"
    out = subprocess.run([exe], input=text.encode(), capture_output=True, check=True).stdout
    pts, off = [], 0
    for _ in CASES:
        (n,) = struct.unpack_from("<I", out, off)
        off += 4
        pts.append(np.frombuffer(out, np.float32, 3 * n, off).reshape(n, 3).copy())
        off += 12 * n
    return pts


def main():
    pts = run(build())
    out = {}
    for k, ((kind, kw), p) in enumerate(zip(CASES, pts)):
        out[f"case{k}_kind"] = np.array(kind)
        out[f"case{k}_args"] = np.array(repr(kw))
        out[f"case{k}_points"] = p
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "arrangements", "points.npz"),
                        **out)
    for (kind, kw), p in zip(CASES, pts):
        print(kind, len(p))


if __name__ == "__main__":
    main()
