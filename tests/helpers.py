"""Shared test helpers: run one scene through the CUDA path (C ABI) and the
CPU oracle, and compare them."""
from __future__ import annotations

import os

import numpy as np

from ssf_pbf_cuda_gb300 import api, scenes

# Positions: 1e-5 relative, with the denominator floored at 0.1 m (one h) so
# coordinates near 0 are compared to 1e-6 m absolute.
POS_RTOL = 1e-5
POS_FLOOR = 0.1


def pos_rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float((np.abs(a - b) / np.maximum(np.abs(b), POS_FLOOR)).max())


def vel_abs_tol(dt: float, x=None) -> float:
    # v = (x - x_old) / dt turns the allowed position error (1e-5 of |x|) into e / dt
    scale = max(POS_FLOOR, float(np.abs(np.asarray(x)).max(initial=0.0))) if x is not None else POS_FLOOR
    return POS_RTOL * scale / dt * 2.0


def resolved(params: dict, sc: scenes.Scene) -> dict:
    p = sc.params(params)
    p["grid_size"] = list(api.resolve_grid(p, sc.domain_end))
    p["cell_width"] = p["cell_width"] or p["smoothing_length"]
    return p


def reflike_params(s: float = 0.05) -> dict:
    """The reference's own dam-break parameters (pbf_dam_init_cond.cpp:13-23):
    h = 1.4 s, eps = 1/s^2, dt = 0.015, reference s_corr, XSPH/vorticity off."""
    h = 1.4 * s
    return api.default_params(smoothing_length=h, cell_width=h, stable_distance=s, particle_mass=1000 * s ** 3,
                              relaxation=1 / s ** 2, time_step=0.015)


def reflike_dam(n_side: int = 32, scene_id: int = 7) -> scenes.Scene:
    s = 0.05
    return scenes.dam_break(n_side, n_side, n_side, (4.0, 2.0, 2.0), scene_id=scene_id, h=1.4 * s, spacing=s)


def oracle_boundary(O, sc: scenes.Scene, mode: str):
    if mode == "planes":
        return O.Boundary(plane_pts=sc.planes[0], plane_nrm=sc.planes[1])
    if mode == "builtin":
        return None
    raise ValueError(mode)


def gpu_boundary(sc: scenes.Scene, mode: str):
    if mode == "planes":
        return api.Boundary(points_on_planes=sc.planes[0], normals_on_planes=sc.planes[1])
    return None


def run_oracle(O, sc, params, mode="planes", iters=4, f64=False, x=None, v=None):
    p = resolved(params, sc)
    return O.step(p, oracle_boundary(O, sc, mode), sc.area[0], sc.area[1], iters,
                  sc.x if x is None else x, sc.v if v is None else v, f64=f64)


def run_gpu(sc, params, mode="planes", iters=4, steps=1, graph=True, debug=True, capacity=None, x=None, v=None):
    p = resolved(params, sc)
    part = api.PbfParticle(p, capacity or max(sc.n, 1), sc.domain_end)
    part.set_graph_mode(graph)
    part.set_particles(sc.x if x is None else x, sc.v if v is None else v)
    b = gpu_boundary(sc, mode)
    for _ in range(steps):
        api.one_step(part, b, sc.area, iters)
    xo, vo = part.get_particles()
    out = {"x": xo, "v": vo, "num": part.num, "flags": part.flags(), "launches": part.launches}
    if debug:
        out.update(part.neighbor_debug())
    out["particle"] = part
    return out


def oracle_reference_layout(r: dict, max_pair: int, C: int) -> dict:
    """Oracle integer outputs in the reference's layouts (as the debug getter gives them)."""
    live = r["num"]
    keys, perm, off = r["keys"], r["perm"], r["offsets"]
    sorted_hash = keys[perm]
    cs = np.full(C, 0xFFFFFFFF, np.uint32)
    ce = np.full(C, 0xFFFFFFFF, np.uint32)
    ne = off[1:C + 1] > off[:C]
    cs[ne] = off[:C][ne]
    ce[ne] = off[1:C + 1][ne]
    nl = np.full((live + 31) // 32 * 32 * max_pair, 0xFFFFFFFF, np.uint32)
    cap = max_pair - 1
    for k in range(cap):
        p = np.nonzero(r["nnb"] > k)[0]
        idx = (k << 5) + (p & 31) + ((p >> 5) << 5) * max_pair
        nl[idx] = r["nbr"][p, k]
    return {"sorted_hash": sorted_hash, "perm": perm, "cell_start": cs, "cell_end": ce, "neighbor_list": nl}


def assert_integer_parity(g: dict, r: dict, params: dict):
    C = int(np.prod(params["grid_size"]))
    ref = oracle_reference_layout(r, params["max_pair_particle_num"], C)
    assert g["num"] == r["num"]
    assert g["n_in"] == len(r["perm"])
    for k in ("sorted_hash", "perm", "cell_start", "cell_end", "neighbor_list"):
        a, b = np.asarray(g[k]), np.asarray(ref[k])
        assert a.shape == b.shape, (k, a.shape, b.shape)
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, f"{k}: {bad.size} mismatches, first at {bad[:5]}: gpu {a[bad[:5]]} oracle {b[bad[:5]]}"


# ---------------------------------------------------------------- golden --
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_PARAM_ORDER = ["stable_density", "stable_distance", "particle_mass", "smoothing_length", "time_step",
                      "relaxation", "xsph_parameter", "vc_parameter"]


def golden_files():
    import glob
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def golden_case(path):
    """(scene, params, boundary mode arrays, iters, fixture) from a fixture file."""
    fx = dict(np.load(path))
    p = api.default_params()
    for k, val in zip(GOLDEN_PARAM_ORDER, fx["params"]):
        p[k] = float(val)
    p["body_force"] = [float(t) for t in fx["body_force"]]
    p["cell_width"] = p["smoothing_length"]
    p["grid_size"] = [int(t) for t in fx["ieee_grid"]]
    # post-solve passes the fixture's reference run made (oracle/ref_driver.cu):
    # 1 XSPH, 2 vorticity then XSPH, 3 vorticity; both in the reference's forms
    post = int(fx["post"]) if "post" in fx else 0
    if post in (1, 2):
        p["xsph_mode"] = api.L.PBF_XSPH_WALK
    if post in (2, 3):
        p["vorticity_mode"] = api.L.PBF_VORTICITY_REFERENCE
    sc = scenes.Scene(fx["x_in"], fx["v_in"], tuple(float(t) for t in fx["domain_end"]),
                      (tuple(float(t) for t in fx["area_min"]), tuple(float(t) for t in fx["area_max"])),
                      (fx["plane_pts"], fx["plane_nrm"]))
    return sc, p, int(fx["iters"]), fx


def golden_oracle_boundary(O, fx):
    if not int(fx["use_boundary"]):
        return None
    return O.Boundary(inner=fx["inner"], outer=fx["outer"], plane_pts=fx["plane_pts"], plane_nrm=fx["plane_nrm"])


def golden_gpu_boundary(fx):
    if not int(fx["use_boundary"]):
        return None
    return api.Boundary(inner_spheres=fx["inner"], outer_spheres=fx["outer"], points_on_planes=fx["plane_pts"],
                        normals_on_planes=fx["plane_nrm"])


def reference_of(fx, variant="ieee"):
    return {k[len(variant) + 1:]: fx[k] for k in fx if k.startswith(variant + "_")}


def golden_with(variant):
    """Fixture files holding outputs of a reference build ("cub") or run ("ieee0")."""
    return [f for f in golden_files() if f"{variant}_num" in np.load(f).files]


def compare_to_reference_exact(ours: dict, ref: dict) -> dict:
    """Against the reference's stable radix-sort build (cub): the sorted
    index array is the permutation, so every integer array is compared as
    is, the neighbour lists slot by slot in their order (live particles'
    entries; the reference fills only num * max_pair entries), and
    positions and velocities in sorted order.  Returns the error report and
    the number of mismatching integers per array."""
    num = int(ref["num"])
    assert ours["num"] == num, (ours["num"], num)
    rep = {}
    rep["perm"] = int(np.count_nonzero(np.asarray(ours["perm"])[:len(ref["sorted_index"])] != ref["sorted_index"]))
    rep["sorted_hash"] = int(np.count_nonzero(np.asarray(ours["sorted_hash"])[:num] != ref["sorted_hash"][:num]))
    cs_r, ce_r = ref["cell_start"], ref["cell_end"]
    ne = cs_r != 0xFFFFFFFF
    rep["cell_start"] = int(np.count_nonzero(np.asarray(ours["cell_start"]) != cs_r))
    rep["cell_end"] = int(np.count_nonzero(np.asarray(ours["cell_end"])[ne] != ce_r[ne]))
    mp = int(ref["max_pair"])
    p = np.arange(num)
    slots = ((np.arange(mp)[None, :] << 5) + ((p & 31) + ((p >> 5) << 5) * mp)[:, None]).reshape(-1)
    nl_o, nl_r = np.asarray(ours["neighbor_list"])[slots], ref["neighbor_list"][slots]
    rep["neighbor_list"] = int(np.count_nonzero(nl_o != nl_r))
    rep["listed"] = int(np.count_nonzero(nl_r != 0xFFFFFFFF))
    rep["pos_rel_err"] = pos_rel_err(ours["x"], ref["x"])
    rep["vel_abs_err"] = float(np.abs(np.asarray(ours["v"], np.float64) - ref["v"]).max(initial=0))
    return rep


def by_id(v, perm, num):
    """Rows of a sorted-order array placed by input index."""
    out = np.zeros((len(perm), 3))
    out[np.asarray(perm, np.int64)[:num]] = np.asarray(v, np.float64)[:num]
    return out


def post_increment_error(ours: dict, ours0: dict, ref: dict, ref0: dict) -> tuple:
    """Velocity increments of the post-solve passes (run with them minus run
    without), by particle id, ours against the reference's: (max error /
    max reference increment, max reference increment)."""
    num = int(ref["num"])
    d_ref = by_id(ref["v"], ref["sorted_index"], num) - by_id(ref0["v"], ref0["sorted_index"], num)
    d_our = by_id(ours["v"], ours["perm"], num) - by_id(ours0["v"], ours0["perm"], num)
    scale = float(np.abs(d_ref).max(initial=0.0))
    return float(np.abs(d_our - d_ref).max(initial=0.0)) / max(scale, 1e-30), scale


def compare_to_reference(ours: dict, ref: dict, C: int) -> dict:
    """Compare a step's outputs with the reference's.  The reference's sort is
    a counting sort with atomic ranks, so the order inside a cell is
    arbitrary: integers are compared on sort-invariant forms (sorted hashes,
    cell ranges, per-cell index sets, neighbour sets by particle id), and
    positions/velocities by particle id.  ``ours`` holds num, x, v (sorted),
    perm (sorted -> input), sorted_hash, cell_start, cell_end and
    neighbor_list (reference layout)."""
    rep = {}
    num = int(ref["num"])
    assert ours["num"] == num, (ours["num"], num)
    # sorted hashes of live particles; deleted ones carry C here, Gz*Gy*Gz-1 there
    assert np.array_equal(np.asarray(ours["sorted_hash"])[:num], ref["sorted_hash"][:num])
    cs_r, ce_r = ref["cell_start"], ref["cell_end"]
    ne = cs_r != 0xFFFFFFFF
    assert np.array_equal(ne, ours["cell_start"] != 0xFFFFFFFF)
    assert np.array_equal(ours["cell_start"][ne], cs_r[ne]) and np.array_equal(ours["cell_end"][ne], ce_r[ne])
    pr = ref["sorted_index"].astype(np.int64)
    po = np.asarray(ours["perm"]).astype(np.int64)
    # the same index set in every cell: order each cell's indices (the sorted
    # hashes are equal, so (hash, index) order compares cell by cell)
    sh = np.asarray(ref["sorted_hash"][:num], np.int64)
    assert np.array_equal(pr[:num][np.lexsort((pr[:num], sh))], po[:num][np.lexsort((po[:num], sh))])
    assert np.array_equal(np.sort(pr[num:]), np.sort(po[num:]))
    # positions / velocities by particle id
    xr = np.zeros((len(pr), 3)); xo = np.zeros((len(pr), 3))
    vr = np.zeros((len(pr), 3)); vo = np.zeros((len(pr), 3))
    xr[pr[:num]] = ref["x"]; xo[po[:num]] = ours["x"]
    vr[pr[:num]] = ref["v"]; vo[po[:num]] = ours["v"]
    rep["pos_rel_err"] = pos_rel_err(xo, xr)
    rep["vel_abs_err"] = float(np.abs(vo - vr).max(initial=0))
    # neighbour sets by particle id
    mp = int(ref["max_pair"])

    def sets(nl, perm):
        """Row id(p) holds the sorted ids of p's listed neighbours (-1 pads);
        a list ends at its first empty slot."""
        p = np.arange(num)
        slots = (np.arange(mp)[None, :] << 5) + ((p & 31) + ((p >> 5) << 5) * mp)[:, None]
        q = np.asarray(nl, np.int64)[slots]
        live = np.cumprod(q != 0xFFFFFFFF, axis=1).astype(bool)
        ids = np.where(live, perm[np.where(live, q, 0)], np.int64(-1))
        out = np.full((len(perm), mp), -1, np.int64)
        out[perm[:num]] = np.sort(ids, axis=1)
        return out

    so, sr = sets(np.asarray(ours["neighbor_list"]), po), sets(ref["neighbor_list"], pr)
    rep["neighbor_set_mismatches"] = int(np.count_nonzero((so != sr).any(axis=1)))
    return rep
