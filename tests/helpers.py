"""Shared test helpers: run one scene through the CUDA path (C ABI) and the
CPU oracle, and compare them."""
from __future__ import annotations

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
