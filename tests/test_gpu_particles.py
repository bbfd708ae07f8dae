"""Particle-set operations on the GPU: ids that follow the sort, order
restore, the arrangement generators on the device and the device-side
emitter — against the oracle (oracle/oracle.py, oracle/arrangement.py)."""
import numpy as np
import pytest

from oracle import arrangement as A
from ssf_pbf_cuda_gb300 import _lib as L
from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H
from tests.test_arrangement import CASES, abi_arrangement

pytestmark = pytest.mark.gpu


def small_dam(scene_id=11):
    return scenes.dam_break(12, 10, 8, (1.5, 1.2, 1.0), scene_id=scene_id)


def stable_params(**kw):
    return api.config_params(scorr_k=1e-4, **kw)


def handle_for(sc, params, capacity=None):
    p = H.resolved(params, sc)
    part = api.PbfParticle(p, capacity or sc.n, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    return part, p


@pytest.mark.parametrize("k", range(len(CASES)))
def test_generate_matches_oracle(gpu, k):
    kind, kw, _ = CASES[k]
    pts = A.generate(kind, **kw)
    lead = np.array([[0.5, 0.5, 0.5], [0.6, 0.5, 0.5], [0.7, 0.5, 0.5]], np.float32)
    part = api.PbfParticle(api.default_params(), len(pts) + 8, (8.0, 8.0, 8.0))
    part.set_particles(lead)
    v0 = (0.25, -1.0, 2.8)
    n = part.generate(abi_arrangement(kind, kw), v0)
    assert n == len(pts)
    x, v = part.get_particles()
    assert part.num == 3 + n and part.flags() == 0
    assert np.array_equal(x[:3], lead)
    if kind == "cylinder":
        np.testing.assert_allclose(x[3:], pts, rtol=0, atol=4e-7 * max(1.0, float(np.abs(pts).max(initial=1))))
    else:
        assert np.array_equal(x[3:].view(np.uint32), pts.view(np.uint32))
    assert np.array_equal(v[3:], np.tile(np.float32(v0), (n, 1)))
    assert np.array_equal(part.particle_ids(), np.arange(3 + n, dtype=np.uint32))


def test_generate_overflow_adds_nothing_and_flags(gpu):
    part = api.PbfParticle(api.default_params(), 100, (8.0, 8.0, 8.0))
    part.set_particles(np.full((10, 3), 1.0, np.float32))
    n = part.generate(api.arrangement("volume", origin=(0, 0, 0), end=(1, 1, 1), space=0.2))
    assert n == 216
    assert part.num == 10
    assert part.flags() & L.PBF_FLAG_CAPACITY


def test_ids_follow_the_sort_across_steps(oracle, gpu):
    """ids after each step = the composition of the oracle's permutations."""
    sc = small_dam()
    params = stable_params()
    part, p = handle_for(sc, params)
    b = H.gpu_boundary(sc, "planes")
    ob = H.oracle_boundary(oracle, sc, "planes")
    ids = np.arange(sc.n, dtype=np.uint32)
    x, v = sc.x, sc.v
    for _ in range(3):
        api.one_step(part, b, sc.area, 4)
        r = oracle.step(p, ob, sc.area[0], sc.area[1], 4, x, v)
        ids = ids[r["perm"][:r["num"]]]
        x, v = r["x"], r["v"]
        assert np.array_equal(part.particle_ids(), ids)
    xb, vb = part.particles_by_id(sc.n)
    xr = np.full((sc.n, 3), np.nan, np.float32)
    xr[ids] = x
    assert np.array_equal(np.isnan(xb), np.isnan(xr))
    ok = ~np.isnan(xr[:, 0])
    assert H.pos_rel_err(xb[ok], xr[ok]) <= H.POS_RTOL


def test_restore_order_is_the_last_steps_input_order(oracle, gpu):
    """restoreOrder with a deletion: rows of deleted particles keep the
    caller's values (NaN here), the rest are x[perm^-1]."""
    sc = small_dam(scene_id=12)
    area = (sc.area[0], (sc.area[1][0], 0.35, sc.area[1][2]))  # deletes the upper part
    params = stable_params()
    p = H.resolved(params, sc)
    part = api.PbfParticle(p, sc.n, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    with pytest.raises(L.PbfError):
        part.restore_order(sc.n)  # no step since the particles were set
    api.one_step(part, H.gpu_boundary(sc, "planes"), area, 4)
    x, v = part.get_particles()
    perm = part.neighbor_debug()["perm"]
    num = part.num
    assert num < sc.n
    xr, vr = part.restore_order(sc.n)
    want = np.full((sc.n, 3), np.nan, np.float32)
    want[perm[:num]] = x
    assert np.array_equal(np.isnan(xr), np.isnan(want))
    ok = ~np.isnan(want[:, 0])
    assert np.array_equal(xr[ok], want[ok])
    r = oracle.step(p, H.oracle_boundary(oracle, sc, "planes"), area[0], area[1], 4, sc.x, sc.v)
    xo = np.full((sc.n, 3), np.nan, np.float32)
    xo[r["perm"][:r["num"]]] = r["x"]
    assert H.pos_rel_err(xr[ok], xo[ok]) <= H.POS_RTOL


def jet_arrangement():
    # the sphere scene's jet, pbf_sphere_sim.cpp:328 (spacing 0.05)
    return api.arrangement("rectangle", axis="x", axis_value=1.25, origin=(3.5, 2.5), end=(4.5, 3.5), space=0.05)


def test_emitter_follows_the_jet_rule(gpu):
    """Append iff num < 0.8 capacity, decided on the device; ids continue."""
    em = api.Emitter(arrangement=jet_arrangement(), velocity=(2.8, 0.0, 0.0))
    m = em.size
    assert m == 441
    cap = 3000
    part = api.PbfParticle(api.default_params(), cap, (8.0, 8.0, 8.0))
    part.set_particles(np.full((100, 3), 0.5, np.float32))
    num = 100
    for _ in range(8):
        part.emit(em, 0.8)
        if num < cap * 0.8 and num + m <= cap:
            num += m
        assert part.num == num
    assert num == 100 + 6 * m  # 2746 >= 2400 stops the jet
    ids = part.particle_ids()
    assert np.array_equal(ids, np.arange(num, dtype=np.uint32))
    x, v = part.get_particles()
    pts = A.rectangle("x", 1.25, (3.5, 2.5), (4.5, 3.5), 0.05)
    for k in range(6):
        blk = slice(100 + k * m, 100 + (k + 1) * m)
        assert np.array_equal(x[blk], pts)
        assert np.all(v[blk] == np.float32([2.8, 0.0, 0.0]))
    assert part.flags() == 0


def test_emitter_overflow_flags_capacity(gpu):
    em = api.Emitter(np.full((50, 3), 0.25, np.float32))
    part = api.PbfParticle(api.default_params(), 120, (8.0, 8.0, 8.0))
    part.set_particles(np.full((80, 3), 0.5, np.float32))
    part.emit(em, 1.0)  # 80 + 50 > 120
    assert part.num == 80
    assert part.flags() & L.PBF_FLAG_CAPACITY


def test_emit_then_step_matches_oracle(oracle, gpu):
    sc = small_dam(scene_id=13)
    params = stable_params()
    p = H.resolved(params, sc)
    jet = api.arrangement("rectangle", axis="x", axis_value=0.2, origin=(0.3, 0.2), end=(0.6, 0.5), space=0.05)
    pts = A.rectangle("x", 0.2, (0.3, 0.2), (0.6, 0.5), 0.05)
    em = api.Emitter(arrangement=jet, velocity=(1.0, 0.0, 0.0))
    part = api.PbfParticle(p, sc.n + len(pts), sc.domain_end)
    part.set_particles(sc.x, sc.v)
    part.emit(em, 1.0)
    api.one_step(part, H.gpu_boundary(sc, "planes"), sc.area, 4)
    x2 = np.concatenate([sc.x, pts]).astype(np.float32)
    v2 = np.concatenate([sc.v, np.tile(np.float32([1.0, 0, 0]), (len(pts), 1))]).astype(np.float32)
    sc2 = scenes.Scene(x2, v2, sc.domain_end, sc.area, sc.planes)
    r = H.run_oracle(oracle, sc2, params, "planes", 4)
    g = {"num": part.num, "n_in": len(x2)}
    g.update(part.neighbor_debug())
    H.assert_integer_parity(g, r, p)
    xg, vg = part.get_particles()
    assert H.pos_rel_err(xg, r["x"]) <= H.POS_RTOL
    assert np.array_equal(part.particle_ids(), r["perm"][:r["num"]])


def test_batch_generate_and_emit_equal_the_plain_handle(gpu):
    sc = small_dam(scene_id=14)
    params = stable_params()
    p = H.resolved(params, sc)
    jet = api.arrangement("rectangle", axis="x", axis_value=0.2, origin=(0.3, 0.2), end=(0.6, 0.5), space=0.05)
    blob = api.arrangement("volume", origin=(0.9, 0.6, 0.3), end=(1.1, 0.8, 0.5), space=0.05)
    em = api.Emitter(arrangement=jet, velocity=(1.0, 0.0, 0.0))
    cap = sc.n + 2000
    part = api.PbfParticle(p, cap, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    bnd = H.gpu_boundary(sc, "planes")
    batch = api.Batch(2, 2 * cap, 2 * (int(np.prod(p["grid_size"])) + 1), 30)
    other = small_dam(scene_id=15)
    batch.add_scene(p, other.n, other.domain_end, bnd, other.area, other.x, other.v)
    sid = batch.add_scene(p, cap, sc.domain_end, bnd, sc.area, sc.x, sc.v)
    for target in ("plain", "batch"):
        for step in range(3):
            if target == "plain":
                part.generate(blob) if step == 0 else part.emit(em, 0.9)
                api.one_step(part, bnd, sc.area, 4)
            else:
                batch.generate(sid, blob) if step == 0 else batch.emit(sid, em, 0.9)
                batch.step(4)
    xp, vp = part.get_particles()
    xb, vb = batch.get_scene(sid)
    assert np.array_equal(xp, xb) and np.array_equal(vp, vb)
    assert np.array_equal(part.particle_ids(), batch.particle_ids(sid))
