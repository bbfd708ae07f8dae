"""Batched engine and continuous-batching server on the GPU.

Each scene's result in a batch must equal (bitwise) the same scene stepped
alone through the plain single-scene path, and match the oracle within the
parity tolerance."""
import numpy as np
import pytest

import ssf_pbf_cuda_gb300 as pbf
from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H

pytestmark = pytest.mark.gpu


def mixed_scenes():
    """Scenes of uneven sizes and different physics modes."""
    out = []
    s = 0.05
    out.append((H.reflike_dam(10, scene_id=31), H.reflike_params()))
    sc = scenes.dam_break(14, 9, 11, (2.0, 1.5, 1.5), scene_id=32)
    out.append((sc, api.config_params(scorr_k=1e-4)))
    sc = scenes.dam_break(7, 20, 6, (1.0, 2.0, 1.0), scene_id=33)
    out.append((sc, api.config_params(scorr_k=1e-4, vorticity_mode=pbf.PBF_VORTICITY_REFERENCE, xsph_mode=0)))
    sc = scenes.dam_break(16, 16, 16, (3.0, 2.0, 2.0), scene_id=34, h=1.4 * s, spacing=s)
    out.append((sc, H.reflike_params()))
    sc = scenes.dam_break(5, 5, 5, (1.0, 1.0, 1.0), scene_id=35)
    out.append((sc, api.config_params(tensile_mode=pbf.PBF_TENSILE_OFF, xsph_mode=1, vorticity_mode=0)))
    return out


def make_batch(items, extra_particles=0):
    n = sum(sc.n for sc, _ in items) + extra_particles
    cells = sum(int(np.prod(H.resolved(p, sc)["grid_size"])) + 1 for sc, p in items) + 100000
    b = api.Batch(len(items) + 4, n + 1000, cells, 30)
    ids = []
    for sc, p in items:
        ids.append(b.add_scene(H.resolved(p, sc), sc.n, sc.domain_end, H.gpu_boundary(sc, "planes"), sc.area,
                               sc.x, sc.v))
    return b, ids


def alone(sc, p, steps):
    return H.run_gpu(sc, p, "planes", 4, steps=steps, debug=False)


def test_alone_equals_in_mix_bitwise(gpu):
    items = mixed_scenes()
    b, ids = make_batch(items)
    for _ in range(2):
        b.step(4)
    for (sc, p), sid in zip(items, ids):
        x, v = b.get_scene(sid)
        a = alone(sc, p, 2)
        assert np.array_equal(x, a["x"]) and np.array_equal(v, a["v"])


def test_mixed_list_formats_alone_equals_in_mix(oracle, gpu):
    """A batch mixing a scene of more than 65,536 slots (u32 neighbour
    lists) with smaller ones (u16 lists), large enough for the large-step
    kernels, with the configured XSPH and vorticity list forms (each pass
    runs once per list format, the vorticity pass gathering (x, v) records):
    every scene equals itself stepped alone, bit for bit, and the big scene
    matches the FP64 oracle."""
    p = api.config_params(scorr_k=1e-4)
    items = [(scenes.dam_break(40, 40, 44, (4.0, 3.0, 3.0), scene_id=61), p)]
    items += [(scenes.dam_break(25, 25, 25, (2.0, 2.0, 2.0), scene_id=62 + k), p) for k in range(4)]
    assert items[0][0].n > 65536 and sum(sc.n for sc, _ in items) > 131072
    b, ids = make_batch(items)
    b.step(4)
    for (sc, pp), sid in zip(items, ids):
        x, v = b.get_scene(sid)
        a = alone(sc, pp, 1)
        assert np.array_equal(x, a["x"]) and np.array_equal(v, a["v"])
    sc = items[0][0]
    x, v = b.get_scene(ids[0])
    r = H.run_oracle(oracle, sc, p, "planes", 4, f64=True)
    assert H.pos_rel_err(x, r["x"]) <= H.POS_RTOL
    assert np.abs(v - r["v"]).max(initial=0) <= H.vel_abs_tol(p["time_step"], r["x"])


def test_batch_matches_oracle_per_scene(oracle, gpu):
    items = mixed_scenes()
    b, ids = make_batch(items)
    b.step(4)
    for (sc, p), sid in zip(items, ids):
        x, v = b.get_scene(sid)
        r = H.run_oracle(oracle, sc, p, "planes", 4, f64=True)
        assert H.pos_rel_err(x, r["x"]) <= H.POS_RTOL
        assert np.abs(v - r["v"]).max(initial=0) <= H.vel_abs_tol(p["time_step"], r["x"])


SCORR_FORMS = {
    "textbook_n4": dict(scorr_k=1e-4),
    "textbook_n3": dict(scorr_k=1e-4, scorr_n=3),
    "reference": dict(tensile_mode=pbf.PBF_TENSILE_REFERENCE),
    "off": dict(tensile_mode=pbf.PBF_TENSILE_OFF),
}


@pytest.mark.parametrize("form", sorted(SCORR_FORMS))
def test_small_and_large_step_paths_agree(oracle, gpu, form):
    """Steps of at most 131,072 particle slots are latency bound: they rank
    each bucket from the particle side, split each particle's neighbour walk
    and its iteration-0 lambda sum over four lanes (terms added in list
    order) and keep lambda in its own array.  Larger steps rank per cell,
    give a particle one lane and carry lambda in the positions' w lane.  The
    same scene stepped
    alone (small) and inside a 163,840-particle batch (large) gives
    bit-identical results for every s_corr form, and the large path matches
    the oracle.  The reference s_corr with these parameters (spacing 0.5h,
    eps 600) is unstable within one step, so its oracle parity is checked
    with the reference's dam parameters instead (test_gpu_parity)."""
    p = api.config_params(**SCORR_FORMS[form])
    items = [(scenes.dam_break(32, 32, 32, (4.0, 2.0, 2.0), scene_id=41 + k), p) for k in range(5)]
    b, ids = make_batch(items)
    for _ in range(2):
        b.step(4)
    sc = items[0][0]
    x, v = b.get_scene(ids[0])
    a = alone(sc, p, 2)
    assert np.array_equal(x, a["x"]) and np.array_equal(v, a["v"])
    b2, ids2 = make_batch(items[:1])
    b2.step(4)
    x1, v1 = b2.get_scene(ids2[0])
    b3, ids3 = make_batch(items)
    b3.step(4)
    xl, vl = b3.get_scene(ids3[0])
    assert np.array_equal(x1, xl) and np.array_equal(v1, vl)
    if form == "reference":
        return
    r = H.run_oracle(oracle, sc, p, "planes", 4, f64=True)
    assert H.pos_rel_err(xl, r["x"]) <= H.POS_RTOL
    assert np.abs(vl - r["v"]).max(initial=0) <= H.vel_abs_tol(p["time_step"], r["x"])


@pytest.mark.parametrize("tile", [64, 128, 256, 512])
def test_tile_sizes_give_identical_results(gpu, tile):
    items = mixed_scenes()[:3]
    b, ids = make_batch(items)
    b.set_tile(tile)
    b.step(4)
    for (sc, p), sid in zip(items, ids):
        x, _ = b.get_scene(sid)
        assert np.array_equal(x, alone(sc, p, 1)["x"])


def test_remove_and_reuse_slots(gpu):
    items = mixed_scenes()
    b, ids = make_batch(items)
    b.step(4)
    b.remove_scene(ids[1])
    b.remove_scene(ids[3])
    assert b.num_scenes == 3
    sc, p = items[1]
    nid = b.add_scene(H.resolved(p, sc), sc.n, sc.domain_end, H.gpu_boundary(sc, "planes"), sc.area, sc.x, sc.v)
    assert nid in (ids[1], ids[3])
    b.step(4)
    x, _ = b.get_scene(nid)
    assert np.array_equal(x, alone(sc, p, 1)["x"])
    x0, _ = b.get_scene(ids[0])
    assert np.array_equal(x0, alone(*items[0], 2)["x"])


def test_set_all_get_all_roundtrip(gpu):
    import torch
    items = mixed_scenes()
    b, ids = make_batch(items)
    assert b.scene_ids() == sorted(ids)
    counts, x, v = b.get_all()
    assert list(counts) == [sc.n for sc, _ in items]
    assert np.array_equal(x, np.concatenate([sc.x for sc, _ in items]))
    # device round trip with a perturbed state
    xd = torch.from_numpy(x + 0.001).cuda()
    vd = torch.from_numpy(v + 0.5).cuda()
    b.set_all(xd, vd, counts)
    c2, x2, v2 = b.get_all()
    assert np.array_equal(x2, x + np.float32(0.001)) and np.array_equal(v2, v + np.float32(0.5))


def test_get_all_async_equals_get_all(gpu):
    """pbf_batch_get_all_async packs the batch into device buffers with the
    packed offsets computed on the device from the live counts (no host
    round trip): the same counts and particles as pbf_batch_get_all, with a
    removed scene's slot left out and a scene whose area deletes a third of
    its particles in the first step."""
    import dataclasses
    import torch
    items = mixed_scenes()
    sc = scenes.dam_break(12, 12, 12, (1.5, 1.5, 1.5), scene_id=52)
    items.append((dataclasses.replace(sc, area=((-0.1, -0.1, -0.1), (1.6, 0.45, 1.6))),
                  api.config_params(scorr_k=1e-4)))
    b, ids = make_batch(items)
    b.remove_scene(ids[1])
    for _ in range(2):
        b.step(4)
    counts, x, v = b.get_all()
    assert counts[-1] < sc.n  # the last scene lost particles
    cap = sum(sc_.n for k, (sc_, _) in enumerate(items) if k != 1)
    cd = torch.zeros(len(counts), dtype=torch.int32, device="cuda")
    xd = torch.full((cap, 3), -1.0, dtype=torch.float32, device="cuda")
    vd = torch.full((cap, 3), -1.0, dtype=torch.float32, device="cuda")
    b.get_all_async(cd, xd, vd)
    torch.cuda.synchronize()
    tot = int(counts.sum())
    assert np.array_equal(cd.cpu().numpy().view(np.uint32), counts)
    assert np.array_equal(xd[:tot].cpu().numpy(), x) and np.array_equal(vd[:tot].cpu().numpy(), v)
    assert bool((xd[tot:] == -1.0).all())  # nothing written past the live particles


@pytest.mark.parametrize("graph", [True, False], ids=["graph", "no_graph"])
def test_step_packed_equals_set_all_then_step(gpu, graph):
    """pbf_batch_step_packed (the step reading its packed input where it lies,
    no unpack pass) gives bit for bit what pbf_batch_set_all from the same
    device buffers followed by pbf_batch_step gives: counts, positions,
    velocities and particle ids, over two steps from two different input
    buffers (the second without velocities), with a removed scene's slot and
    a scene whose area deletes particles; captured in a graph or launched
    kernel by kernel."""
    import dataclasses
    import torch
    items = mixed_scenes()
    sc = scenes.dam_break(12, 12, 12, (1.5, 1.5, 1.5), scene_id=53)
    items.append((dataclasses.replace(sc, area=((-0.1, -0.1, -0.1), (1.6, 0.45, 1.6))),
                  api.config_params(scorr_k=1e-4)))
    keep = [k for k in range(len(items)) if k != 1]
    counts = [items[k][0].n for k in keep]
    x = np.concatenate([items[k][0].x for k in keep]).astype(np.float32)
    v = np.concatenate([items[k][0].v for k in keep]).astype(np.float32)
    inputs = [(torch.from_numpy(x).cuda(), torch.from_numpy(v).cuda()),
              (torch.from_numpy(x + np.float32(0.002)).cuda(), None)]
    b1, ids1 = make_batch(items)
    b2, ids2 = make_batch(items)
    b1.remove_scene(ids1[1])
    b2.remove_scene(ids2[1])
    b2.set_graph_mode(graph)
    for xd, vd in inputs:
        b1.set_all(xd, vd, counts)
        b1.step(4)
        b2.step_packed(4, xd, vd, counts)
        c1, x1, v1 = b1.get_all()
        c2, x2, v2 = b2.get_all()
        assert np.array_equal(c1, c2) and c1[-1] < counts[-1]
        assert np.array_equal(x1, x2) and np.array_equal(v1, v2)
        for k in keep:
            assert np.array_equal(b1.particle_ids(ids1[k]), b2.particle_ids(ids2[k]))


def test_pinned_and_pageable_host_buffers_agree(gpu):
    """Packed host buffers in page-locked (pinned) and in pageable memory
    give the same bits, in both directions, around a step."""
    import torch
    items = mixed_scenes()
    counts = np.array([sc.n for sc, _ in items], np.uint32)
    x0 = np.concatenate([sc.x for sc, _ in items]) + np.float32(0.002)
    v0 = np.concatenate([sc.v for sc, _ in items]) + np.float32(0.25)
    xp = torch.from_numpy(x0.copy()).pin_memory()
    vp = torch.from_numpy(v0.copy()).pin_memory()
    out = []
    for pinned in (False, True):
        b, _ = make_batch(items)
        if pinned:
            b.set_all(xp.numpy(), vp.numpy(), counts)
        else:
            b.set_all(x0, v0, counts)
        b.step(4)
        if pinned:
            xo = torch.zeros_like(xp).pin_memory()
            vo = torch.zeros_like(vp).pin_memory()
            c, _, _ = b.get_all(xo.numpy(), vo.numpy())
            out.append((np.asarray(c), xo.numpy().copy(), vo.numpy().copy()))
        else:
            out.append(b.get_all())
    assert np.array_equal(out[0][0], out[1][0])
    n = int(np.sum(out[0][0]))
    assert np.array_equal(out[0][1][:n], out[1][1][:n]) and np.array_equal(out[0][2][:n], out[1][2][:n])


def test_autotune_preserves_state(gpu):
    items = mixed_scenes()
    b, ids = make_batch(items)
    tile = b.autotune(4)
    assert tile in (64, 128, 256, 512)
    b.step(4)
    for (sc, p), sid in zip(items, ids):
        x, _ = b.get_scene(sid)
        assert np.array_equal(x, alone(sc, p, 1)["x"])


def test_nonfinite_scene_is_isolated(gpu):
    items = mixed_scenes()[:3]
    sc, p = items[1]
    bad = scenes.Scene(sc.x.copy(), sc.v.copy(), sc.domain_end, sc.area, sc.planes)
    bad.x[5] = np.nan
    items[1] = (bad, p)
    b, ids = make_batch(items)
    b.step(4)
    assert b.flags(ids[1]) & pbf.PBF_FLAG_NONFINITE
    assert b.flags(ids[0]) == 0 and b.flags(ids[2]) == 0
    x0, _ = b.get_scene(ids[0])
    assert np.array_equal(x0, alone(*items[0], 1)["x"])


def test_graph_off_matches_graph_on(gpu):
    items = mixed_scenes()
    b1, ids1 = make_batch(items)
    b2, ids2 = make_batch(items)
    b2.set_graph_mode(False)
    for _ in range(3):
        b1.step(4)
        b2.step(4)
    for i1, i2 in zip(ids1, ids2):
        assert np.array_equal(b1.get_scene(i1)[0], b2.get_scene(i2)[0])


def test_profile_step_names_every_kernel(gpu):
    items = mixed_scenes()
    b, _ = make_batch(items)
    prof = b.profile_step(4)
    names = [n for n, _ in prof]
    # small tables are scanned by one block, larger ones in three phases
    scan = ["k_scan_single"] if names[1] == "k_scan_single" else ["k_scan_reduce", "k_scan_spine", "k_scan_down"]
    # small (latency-bound) steps rank per particle and split the neighbour
    # walk over lanes; larger ones rank per cell
    small = "k_rank_reorder" in names
    rank = "k_rank_reorder" if small else "k_rank_cells"
    walk = "k_neighbors_split" if small else "k_neighbors_lambda"
    head = ["k_predict_hash", *scan, "k_scatter", rank, "k_dense_sort", "k_gather", walk]
    assert names[:len(head)] == head
    assert names.count("k_dp") == 4 and names.count("k_lambda") == 3
    assert b.launches == len(prof)


# ------------------------------------------------------------------ server --

def server_requests(n=6):
    reqs = []
    for k in range(n):
        sc = scenes.dam_break(6 + k, 8, 7, (1.5, 1.5, 1.5), scene_id=200 + k)
        reqs.append((sc, api.config_params(scorr_k=1e-4), 2 + (k % 3)))
    return reqs


def submit_all(srv, reqs):
    rids = []
    for sc, p, hz in reqs:
        rids.append(srv.submit(H.resolved(p, sc), sc.domain_end, sc.area, sc.x, sc.v, horizon_steps=hz,
                               planes=sc.planes))
    return rids


def test_server_results_equal_alone(gpu):
    reqs = server_requests()
    big = sum(api.scene_bytes(H.resolved(p, sc), sc.n, sc.domain_end) for sc, p, _ in reqs)
    srv = api.Server(hbm_budget_bytes=big * 2, max_scenes=8, max_particles=20000, max_cells=200000, iters=4)
    rids = submit_all(srv, reqs)
    srv.run_until_idle()
    done = {c["request_id"]: c for c in srv.poll()}
    assert set(done) == set(rids)
    for (sc, p, hz), rid in zip(reqs, rids):
        x, v = srv.result(rid)
        a = alone(sc, p, hz)
        assert done[rid]["steps"] == hz
        assert np.array_equal(x, a["x"]) and np.array_equal(v, a["v"])
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["resident_scenes"] == 0


def test_server_budget_admission_queues(gpu):
    reqs = server_requests(6)
    per = [api.scene_bytes(H.resolved(p, sc), sc.n, sc.domain_end) for sc, p, _ in reqs]
    budget = max(per) * 2  # at most two resident at a time
    srv = api.Server(hbm_budget_bytes=budget, max_scenes=8, max_particles=20000, max_cells=200000, iters=4)
    rids = submit_all(srv, reqs)
    srv.run_until_idle()
    st = srv.stats()
    assert st["completed"] == 6 and st["peak_resident_bytes"] <= budget
    comps = srv.poll()
    assert all(c["admit_s"] >= c["arrival_s"] and c["complete_s"] >= c["admit_s"] for c in comps)
    for (sc, p, hz), rid in zip(reqs, rids):
        assert np.array_equal(srv.result(rid)[0], alone(sc, p, hz)["x"])


def test_server_rejects_over_budget(gpu):
    sc, p, hz = server_requests(1)[0]
    srv = api.Server(hbm_budget_bytes=1000, max_scenes=2, max_particles=5000, max_cells=100000)
    with pytest.raises(pbf.PbfError) as e:
        srv.submit(H.resolved(p, sc), sc.domain_end, sc.area, sc.x, sc.v, horizon_steps=hz, planes=sc.planes)
    assert e.value.status == 8


def test_server_threaded_loop_with_live_arrivals(gpu):
    import time
    reqs = server_requests(6)
    srv = api.Server(hbm_budget_bytes=1 << 32, max_scenes=8, max_particles=20000, max_cells=200000, iters=4)
    srv.start()
    rids = []
    for r in reqs:
        rids += submit_all(srv, [r])
        time.sleep(0.002)
    srv.stop(drain=True)
    done = {c["request_id"] for c in srv.poll()}
    assert done == set(rids)
    for (sc, p, hz), rid in zip(reqs, rids):
        assert np.array_equal(srv.result(rid)[0], alone(sc, p, hz)["x"])


def test_server_refuses_requests_larger_than_the_arena(gpu):
    """A request whose particles or cells exceed the empty arena can never be
    admitted: submit refuses it (PBF_ERROR_CAPACITY) instead of queueing it
    at the head forever, and requests behind it are served."""
    import threading
    reqs = server_requests(2)
    (sc, p, hz), (sc2, p2, hz2) = reqs
    srv = api.Server(hbm_budget_bytes=1 << 34, max_scenes=4, max_particles=sc.n - 1, max_cells=200000, iters=4)
    with pytest.raises(pbf.PbfError) as e:
        srv.submit(H.resolved(p, sc), sc.domain_end, sc.area, sc.x, sc.v, horizon_steps=hz, planes=sc.planes)
    assert e.value.status == 4
    cells = int(np.prod(H.resolved(p, sc)["grid_size"]))
    srv2 = api.Server(hbm_budget_bytes=1 << 34, max_scenes=4, max_particles=20000, max_cells=cells, iters=4)
    with pytest.raises(pbf.PbfError) as e:  # the scene needs cells + 1 (its deleted bucket)
        srv2.submit(H.resolved(p, sc), sc.domain_end, sc.area, sc.x, sc.v, horizon_steps=hz, planes=sc.planes)
    assert e.value.status == 4
    srv3 = api.Server(hbm_budget_bytes=1 << 34, max_scenes=4, max_particles=sc2.n, max_cells=200000, iters=4)
    srv3.start()
    if sc.n > sc2.n:
        with pytest.raises(pbf.PbfError):
            srv3.submit(H.resolved(p, sc), sc.domain_end, sc.area, sc.x, sc.v, horizon_steps=hz, planes=sc.planes)
    rid = srv3.submit(H.resolved(p2, sc2), sc2.domain_end, sc2.area, sc2.x, sc2.v, horizon_steps=hz2,
                      planes=sc2.planes)
    t = threading.Thread(target=srv3.stop, kwargs={"drain": True})
    t.start()
    t.join(timeout=120)
    assert not t.is_alive()
    assert {c["request_id"] for c in srv3.poll()} == {rid}
    assert np.array_equal(srv3.result(rid)[0], alone(sc2, p2, hz2)["x"])


@pytest.mark.parametrize("cells", [64, 128, 512])
def test_cell_tiles_give_identical_results(gpu, cells):
    """The per-cell stable rank of large steps (more than 131,072 particle
    slots) runs `cells` cells per CTA, a launch-shape choice of the
    autotuner: results equal the default 256 bit for bit."""
    p = api.config_params(scorr_k=1e-4)
    items = [(scenes.dam_break(32, 32, 32, (4.0, 2.0, 2.0), scene_id=71 + k), p) for k in range(5)]
    out = {}
    for c in (256, cells):
        b, ids = make_batch(items)
        b.set_cell_tile(c)
        assert b.launch_shape()["cell_tile"] == c
        b.step(4)
        out[c] = [b.get_scene(sid) for sid in ids]
    for (xa, va), (xb, vb) in zip(out[256], out[cells]):
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    with pytest.raises(pbf.PbfError):
        b.set_cell_tile(100)
