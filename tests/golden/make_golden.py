"""Generate golden fixtures from the reference's own CUDA step.

Run on a machine with a GPU after `python oracle/ref_build.py` has prepared
oracle/_ref/src (where the reference is mounted); the binary itself is built
on the machine that runs it (ref_build.build):

    python tests/golden/make_golden.py [out_dir]    (default: this directory)

Each fixture holds the seeded input, the parameters, and the reference's
outputs: num, sorted positions/velocities, sorted hash and index arrays,
cellStart/cellEnd and the neighbour list, per reference build:
  ieee  the shipped counting-sort path, IEEE division and square root;
  fast  the shipped fast-math flags (scenes without boundary contact);
  cub   the reference's stable radix-sort path (-DUSE_CUB), whose sorted
        index array is the permutation itself, bit for bit (scenes that
        delete nothing: that path has no deletion).
Fixtures whose name starts with "post_" run one_step's body with the
post-solve passes the shipped step leaves commented out (XSPH, vorticity
confinement; oracle/ref_driver.cu) and also hold the plain step's outputs
(ieee0_*) for the velocity increments.  The "capped" fixture runs the cub
build with no solver iteration at spacing h/2, where most particles reach
the 29-neighbour cap: its lists pin the cap's selection order.

Before a scene is handed to the reference, the CPU oracle checks that it
stays clear of three reference hazards: a particle with exactly 29 listed
neighbours in a scene that runs solver iterations (opt::memorizeKernelCUDA
then reads into the next warp group's slots, pbf_kernel_memorization.cu:121-132),
a delete cell id Gz*Gy*Gz-1 outside the table or occupied by a live particle
(pbf_neighbor_search.cpp:146), and long collision loops (the reference's loop
is unbounded, pbf_response_collision.cu:33).
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import ref_build  # noqa: E402
from ssf_pbf_cuda_gb300 import api, scenes  # noqa: E402

PARAM_ORDER = ["stable_density", "stable_distance", "particle_mass", "smoothing_length", "time_step",
               "relaxation", "xsph_parameter", "vc_parameter"]


def reflike(s=0.05, **kw):
    h = 1.4 * s
    p = api.default_params(smoothing_length=h, cell_width=h, stable_distance=s, particle_mass=1000 * s ** 3,
                           relaxation=1 / s ** 2, time_step=0.015)
    p.update(kw)
    return p


def golden_cases():
    s = 0.05
    cases = []
    # 1: the reference's dam-break parameters, planes boundary
    sc = scenes.dam_break(16, 16, 16, (2.0, 2.0, 2.0), scene_id=501, h=1.4 * s, spacing=s)
    cases.append(("dam_planes", sc, reflike(), "planes", 4))
    # 2: one iteration
    cases.append(("dam_planes_it1", sc, reflike(), "planes", 1))
    # 3: the no-boundary overload (fixed sphere c=(3,3,3) r=3), particles inside it
    sc2 = scenes.dam_break(16, 16, 16, (7.0, 7.0, 7.0), scene_id=502, h=1.4 * s, spacing=s,
                           origin=(2.4, 2.4, 2.4))
    sc2.v[:] = np.float32([0.3, -0.2, 0.1])
    cases.append(("sphere_builtin", sc2, reflike(), "builtin", 4))
    # 4: spheres + planes, random initial velocities
    sc3 = scenes.dam_break(16, 16, 8, (2.0, 2.0, 2.0), scene_id=503, h=1.4 * s, spacing=s, origin=(0.3, 0.3, 0.3))
    rng = scenes.rng_for(503)
    sc3.v = rng.normal(0, 0.5, size=sc3.x.shape).astype(np.float32)
    cases.append(("spheres_planes", sc3, reflike(), "spheres", 4))
    # 5: denser kernel support (h = 1.7 spacing, up to ~27 neighbours)
    p17 = reflike()
    p17.update(smoothing_length=1.7 * s, cell_width=1.7 * s)
    sc5 = scenes.dam_break(16, 16, 16, (2.0, 2.0, 2.0), scene_id=505, h=1.7 * s, spacing=s)
    cases.append(("dam_dense", sc5, p17, "planes", 4))
    # 6: sparse random particles, some deleted by the simulation area
    rng = scenes.rng_for(504)
    x = rng.uniform(0.2, 1.8, size=(2048, 3)).astype(np.float32)
    v = rng.normal(0, 2.0, size=x.shape).astype(np.float32)
    sc4 = scenes.Scene(x, v, (2.0, 2.0, 2.0), ((0.25, 0.25, 0.25), (1.8, 1.8, 1.8)), scenes.box_planes((2, 2, 2)))
    cases.append(("sparse_deletion", sc4, reflike(), "planes", 4))
    # 7-9: the post-solve passes (ref_driver post modes 1-3) on the block of
    # case 4 (random velocities: non-zero curl), with the reference dam's
    # XSPH c (pbf_dam_init_cond.cpp:20) and a vorticity epsilon large enough
    # that the confinement increment (h passed for 1/h shrinks it by h^8,
    # pbf_vorticity_confinement.cu:28) stands far above rounding
    pv = reflike(xsph_parameter=0.1, vc_parameter=VC_POST)
    cases.append(("post_xsph", sc3, dict(pv, xsph_mode=1), "spheres", 4, 1))
    cases.append(("post_vort_xsph", sc3, dict(pv, xsph_mode=1, vorticity_mode=1), "spheres", 4, 2))
    cases.append(("post_vort", sc3, dict(pv, vorticity_mode=1), "spheres", 4, 3))
    # 10: spacing h/2 (the benchmark configs' density), no solver iteration:
    # interior particles meet ~30 candidates within h and keep the first 29
    pc = reflike()
    pc.update(smoothing_length=2 * s, cell_width=2 * s)
    sc6 = scenes.dam_break(16, 16, 16, (2.0, 2.0, 2.0), scene_id=506, h=2 * s, spacing=s)
    cases.append(("capped", sc6, pc, "planes", 0))
    return cases


# vorticity epsilon of the post_* fixtures
VC_POST = 2.0e4


def boundary_arrays(sc, mode):
    z3, z4 = np.zeros((0, 3), np.float32), np.zeros((0, 4), np.float32)
    if mode == "planes":
        return z4, z4, sc.planes[0], sc.planes[1], 1
    if mode == "builtin":
        return z4, z4, z3, z3, 0
    if mode == "spheres":
        # two overlapping spheres that each hold most of the block, so the
        # projections are moderate (the reference routes outer spheres through
        # its inner-sphere routine, pbf_response_collision.cu:49)
        inner = np.array([[0.7, 0.7, 0.5, 0.52]], np.float32)
        outer = np.array([[0.66, 0.68, 0.48, 0.55]], np.float32)
        return inner, outer, sc.planes[0], sc.planes[1], 1
    raise ValueError(mode)


def oracle_run(sc, p, mode, iters, f64=False):
    inner, outer, pts, nrm, use_b = boundary_arrays(sc, mode)
    b = O.Boundary(inner=inner, outer=outer, plane_pts=pts, plane_nrm=nrm) if use_b else None
    return O.step(p, b, sc.area[0], sc.area[1], iters, sc.x, sc.v, f64=f64)


def check_hazards(sc, p, mode, iters):
    g = p["grid_size"]
    C = g[0] * g[1] * g[2]
    delete_id = g[2] * g[1] * g[2] - 1
    assert delete_id < C, "reference delete cell outside the table"
    r = oracle_run(sc, p, mode, iters)
    live_keys = r["keys"][r["keys"] < C]
    assert not np.any(live_keys == delete_id), "a live particle sits in the reference's delete cell"
    if iters > 0:  # the kernel-cache hazard runs only inside solver iterations
        assert r["nnb"].max(initial=0) <= 28, "a particle reaches the 29-neighbour cap"
    assert 0 <= r["collision_passes"] <= 4, f"collision passes {r['collision_passes']}"
    assert sc.n % 32 == 0
    return r


def write_input(path, sc, p, mode, iters, cap, post=0):
    inner, outer, pts, nrm, use_b = boundary_arrays(sc, mode)
    with open(path, "wb") as f:
        f.write(b"PBFI")
        f.write(struct.pack("<IIIiii", 2, sc.n, cap, iters, use_b, post))
        f.write(np.array([p[k] for k in PARAM_ORDER], np.float32).tobytes())
        for a in (p["body_force"], sc.domain_end, sc.area[0], sc.area[1]):
            f.write(np.asarray(a, np.float32).reshape(3).tobytes())
        f.write(struct.pack("<III", len(inner), len(outer), len(pts)))
        for a in (inner, outer, pts, nrm, sc.x, sc.v):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())


def read_output(path):
    b = open(path, "rb").read()
    assert b[:4] == b"PBFO"
    num, n_in, gx, gy, gz, mp = struct.unpack_from("<6I", b, 4)
    off = 28
    C = gx * gy * gz

    def take(dt, cnt):
        nonlocal off
        a = np.frombuffer(b, dt, cnt, off)
        off += a.nbytes
        return a.copy()

    out = {"num": num, "n_in": n_in, "grid": np.array([gx, gy, gz], np.uint32), "max_pair": mp}
    out["x"] = take(np.float32, 3 * num).reshape(-1, 3)
    out["v"] = take(np.float32, 3 * num).reshape(-1, 3)
    out["sorted_hash"] = take(np.uint32, n_in)
    out["sorted_index"] = take(np.uint32, n_in)
    out["cell_start"] = take(np.uint32, C)
    out["cell_end"] = take(np.uint32, C)
    out["neighbor_list"] = take(np.uint32, (num + 31) // 32 * 32 * mp)
    return out


def main(out_dir, only=None):
    os.makedirs(out_dir, exist_ok=True)
    exes = {v: ref_build.build(v) for v in ("ieee", "fast", "cub")}
    for case in golden_cases():
        name, sc, p, mode, iters = case[:5]
        post = case[5] if len(case) > 5 else 0
        if only and name not in only:
            continue
        p = dict(p)
        p["grid_size"] = list(api.calc_grid_size(2.0 * p["smoothing_length"], sc.domain_end))
        r = check_hazards(sc, p, mode, iters)
        cap = sc.n + 64
        # (output key, build, post mode)
        runs = [("ieee", "ieee", post)]
        if post:
            runs.append(("ieee0", "ieee", 0))  # the plain step: velocity increments of the post passes
        else:
            # the fast-math build only gets scenes with no boundary contact (one
            # collision pass in the oracle), where its approximate division cannot
            # change how the reference's unbounded collision loop ends
            if r["collision_passes"] == 1 and iters > 0:
                runs.append(("fast", "fast", 0))
            if r["num"] == sc.n:  # the radix-sort path has no deletion
                runs.append(("cub", "cub", 0))
        res = {}
        for key, build, pm in runs:
            inp = os.path.join(out_dir, f"{name}.{key}.in.bin")
            write_input(inp, sc, p, mode, iters, cap, pm)
            outp = os.path.join(out_dir, f"{name}.{key}.out.bin")
            subprocess.run([exes[build], inp, outp], check=True, timeout=120)
            res[key] = read_output(outp)
            os.remove(outp)
            os.remove(inp)
        inner, outer, pts, nrm, use_b = boundary_arrays(sc, mode)
        arrays = {"x_in": sc.x, "v_in": sc.v, "inner": inner, "outer": outer, "plane_pts": pts,
                  "plane_nrm": nrm, "use_boundary": np.int32(use_b), "iters": np.int32(iters),
                  "domain_end": np.float32(sc.domain_end), "area_min": np.float32(sc.area[0]),
                  "area_max": np.float32(sc.area[1]),
                  "params": np.array([p[k] for k in PARAM_ORDER], np.float32),
                  "body_force": np.float32(p["body_force"]), "post": np.int32(post),
                  # some particle's list is cut at the cap: the kept set then
                  # depends on the order inside a cell, which only the cub
                  # build fixes
                  "cap_binds": np.int32(int(r["nnb"].max(initial=0)) >= p["max_pair_particle_num"] - 1)}
        for v, r in res.items():
            for k, a in r.items():
                arrays[f"{v}_{k}"] = np.asarray(a)
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **arrays)
        print(name, "num", res["ieee"]["num"], "of", sc.n, "runs", [k for k, _, _ in runs])


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a[7:] for a in sys.argv[1:] if a.startswith("--only=")]
    main(args[0] if args else os.path.dirname(os.path.abspath(__file__)), only or None)
