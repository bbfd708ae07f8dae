"""CUDA path vs the CPU oracle, through the C ABI (one step, then properties).

Integer work (hashes, offsets, stable permutation, cell ranges, neighbour
lists) must be bit-exact.  Positions after one step with 4 iterations must
agree with both the FP32 and FP64 oracles within 1e-5 relative
(denominator floored at 0.1 m); velocities within the same error divided by dt.
"""
import numpy as np
import pytest

import ssf_pbf_cuda_gb300 as pbf
from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _check_step(O, sc, params, mode="planes", iters=4, graph=True):
    g = H.run_gpu(sc, params, mode, iters, graph=graph)
    p = H.resolved(params, sc)
    r32 = H.run_oracle(O, sc, params, mode, iters)
    r64 = H.run_oracle(O, sc, params, mode, iters, f64=True)
    H.assert_integer_parity(g, r32, p)
    assert H.pos_rel_err(g["x"], r32["x"]) <= H.POS_RTOL
    assert H.pos_rel_err(g["x"], r64["x"]) <= H.POS_RTOL
    vt = H.vel_abs_tol(p["time_step"], r64["x"])
    assert np.abs(g["v"] - r32["v"]).max(initial=0) <= vt
    assert np.abs(g["v"] - r64["v"]).max(initial=0) <= vt
    assert g["flags"] == 0
    return g, r32


def test_config1_integer_pipeline_exact_config_physics(oracle, gpu):
    """Config 1 with the configured physics: the integer pipeline (computed
    before the first iteration) is bit-exact; iteration-0 lambda agrees."""
    sc = scenes.config1()
    params = api.config_params()
    g = H.run_gpu(sc, params, "planes", iters=1)
    r = H.run_oracle(oracle, sc, params, "planes", iters=1)
    H.assert_integer_parity(g, r, H.resolved(params, sc))


def test_config1_stable_physics_positions(oracle, gpu):
    # configured physics with s_corr k = 1e-4 (k = 0.1 is unstable at spacing 0.5h)
    _check_step(oracle, scenes.config1(), api.config_params(scorr_k=1e-4))


def test_config1_tensile_off(oracle, gpu):
    _check_step(oracle, scenes.config1(), api.config_params(tensile_mode=pbf.PBF_TENSILE_OFF))


def test_reference_mode_dam(oracle, gpu):
    """The reference's active step (reference s_corr, no XSPH/vorticity) with
    its own dam-break parameters."""
    _check_step(oracle, H.reflike_dam(), H.reflike_params())


def test_reference_mode_no_graph(oracle, gpu):
    _check_step(oracle, H.reflike_dam(16, scene_id=8), H.reflike_params(), graph=False)


def test_builtin_sphere_overload(oracle, gpu):
    """one_step without a boundary argument: the fixed inner sphere (3,3,3), r=3."""
    s = 0.05
    sc = scenes.dam_break(24, 24, 24, (7.0, 7.0, 7.0), scene_id=9, h=1.4 * s, spacing=s, origin=(2.4, 2.4, 2.4))
    sc.planes = (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    _check_step(oracle, sc, H.reflike_params(), mode="builtin")


@pytest.mark.parametrize("iters", [0, 1, 2, 7])
def test_iteration_counts(oracle, gpu, iters):
    _check_step(oracle, H.reflike_dam(12, scene_id=10 + iters), H.reflike_params(), iters=iters)


@pytest.mark.parametrize("n", [1, 2, 27, 33, 1000])
def test_small_random_cases(oracle, gpu, n):
    rng = np.random.default_rng(1234 + n)
    x = rng.uniform(0.5, 1.5, size=(n, 3)).astype(np.float32)
    v = rng.normal(0, 0.1, size=(n, 3)).astype(np.float32)
    sc = scenes.Scene(x, v, (2.0, 2.0, 2.0), ((-0.1,) * 3, (2.1,) * 3), scenes.box_planes((2.0, 2.0, 2.0)))
    _check_step(oracle, sc, api.config_params(scorr_k=1e-4))


def test_empty_scene(gpu):
    sc = scenes.Scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), (1.0, 1.0, 1.0),
                      ((0, 0, 0), (1, 1, 1)), scenes.box_planes((1.0, 1.0, 1.0)))
    g = H.run_gpu(sc, api.config_params(), debug=False)
    assert g["num"] == 0 and g["x"].shape == (0, 3)


def test_deletion_outside_area(oracle, gpu):
    """Particles predicted outside simulation_area are deleted (key = C, sorted last)."""
    rng = np.random.default_rng(77)
    x = rng.uniform(0.2, 1.8, size=(3000, 3)).astype(np.float32)
    v = np.zeros_like(x)
    v[::7, 0] = 200.0  # these leave [0, 2] in one step
    sc = scenes.Scene(x, v, (2.0, 2.0, 2.0), ((0, 0, 0), (2.0, 2.0, 2.0)), scenes.box_planes((2.0, 2.0, 2.0)))
    g, r = _check_step(oracle, sc, api.config_params(scorr_k=1e-4))
    assert r["num"] < 3000 and g["num"] == r["num"]


def test_nonfinite_flag(gpu):
    x = np.array([[0.5, 0.5, 0.5], [np.nan, 0.5, 0.5]], np.float32)
    sc = scenes.Scene(x, np.zeros_like(x), (1.0, 1.0, 1.0), ((-1e30,) * 3, (1e30,) * 3),
                      scenes.box_planes((1.0, 1.0, 1.0)))
    g = H.run_gpu(sc, api.config_params(), debug=False)
    assert g["flags"] & pbf.PBF_FLAG_NONFINITE


def test_collision_pass_limit_flag(gpu):
    """A bound of one collision pass is hit by particles outside the box; the
    step finishes and raises PBF_FLAG_COLLISION_LIMIT instead of looping."""
    rng = np.random.default_rng(5)
    x = rng.uniform(1.05, 1.2, size=(200, 3)).astype(np.float32)  # outside the [0,1]^3 walls
    sc = scenes.Scene(x, np.zeros_like(x), (1.0, 1.0, 1.0), ((-5,) * 3, (5,) * 3), scenes.box_planes((1.0, 1.0, 1.0)))
    g = H.run_gpu(sc, api.config_params(max_collision_passes=1), debug=False)
    assert g["flags"] & pbf.PBF_FLAG_COLLISION_LIMIT


def test_determinism_bitwise(gpu):
    sc = H.reflike_dam(16, scene_id=21)
    a = H.run_gpu(sc, H.reflike_params(), steps=3, debug=False)
    b = H.run_gpu(sc, H.reflike_params(), steps=3, debug=False)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])


def test_graph_and_stream_paths_agree(gpu):
    sc = H.reflike_dam(16, scene_id=22)
    a = H.run_gpu(sc, H.reflike_params(), steps=3, graph=True, debug=False)
    b = H.run_gpu(sc, H.reflike_params(), steps=3, graph=False, debug=False)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])


def test_multi_step_against_oracle(oracle, gpu):
    """Five steps, each compared after feeding the GPU state back to the oracle."""
    sc = H.reflike_dam(16, scene_id=23)
    params = H.reflike_params()
    p = H.resolved(params, sc)
    part = api.PbfParticle(p, sc.n, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    b = H.gpu_boundary(sc, "planes")
    x, v = sc.x, sc.v
    for _ in range(5):
        r = H.run_oracle(oracle, sc, params, "planes", 4, x=x, v=v)
        api.one_step(part, b, sc.area, 4)
        gx, gv = part.get_particles()
        assert H.pos_rel_err(gx, r["x"]) <= H.POS_RTOL
        x, v = gx, gv


def test_add_particles_and_external_pointer(oracle, gpu):
    import torch
    sc = H.reflike_dam(12, scene_id=24)
    params = H.resolved(H.reflike_params(), sc)
    part = api.PbfParticle(params, sc.n + 500, sc.domain_end)
    half = sc.n // 2
    part.set_particles(sc.x[:half], sc.v[:half])
    part.add_particles(sc.x[half:], sc.v[half:])
    assert part.num == sc.n
    xdev = torch.from_numpy(sc.x.copy()).cuda()
    api.one_step_external(part, xdev, H.gpu_boundary(sc, "planes"), sc.area, 4)
    torch.cuda.synchronize()
    r = H.run_oracle(oracle, sc, H.reflike_params(), "planes", 4)
    assert H.pos_rel_err(xdev.cpu().numpy()[:r["num"]], r["x"]) <= H.POS_RTOL


# ---- the neighbour walk's alias-class paths (wrapped power-of-two table) ----

@pytest.mark.parametrize("grid", [(4, 4, 4), (8, 4, 16), (16, 8, 4)])
def test_heavily_aliased_table(oracle, gpu, grid):
    """A 2.0 x 1.0 x 1.0 m block (20 x 10 x 10 cells of 0.1 m) over a table
    of 4-16 cells per axis: buckets mix up to 8 alias classes (cells 2G
    apart share a class); lists stay bit-exact."""
    sc = scenes.dam_break(40, 20, 20, (2.4, 2.4, 2.4), scene_id=sum(grid), grid=grid)
    _check_step(oracle, sc, api.config_params(scorr_k=1e-4))


@pytest.mark.parametrize("grid", [(2, 16, 16), (16, 4, 2), (1, 1, 1)])
def test_small_table_axes_walk_whole_buckets(oracle, gpu, grid):
    """Fewer than 4 cells on an axis: the reference visits a wrapped bucket
    more than once (duplicate list entries); reproduced exactly."""
    sc = scenes.dam_break(12, 12, 10, (1.6, 1.6, 1.6), scene_id=7 + sum(grid), grid=grid)
    g = H.run_gpu(sc, api.config_params(scorr_k=1e-4, max_pair_particle_num=64), "planes", 0)
    r = H.run_oracle(oracle, sc, api.config_params(scorr_k=1e-4, max_pair_particle_num=64), "planes", 0)
    H.assert_integer_parity(g, r, H.resolved(api.config_params(scorr_k=1e-4, max_pair_particle_num=64), sc))


def test_dense_bucket_over_255_members(oracle, gpu):
    """300 particles inside one cell (and its aliases): the bucket is walked
    whole, in sorted order."""
    rng = np.random.default_rng(99)
    dense = rng.uniform(0.81, 0.89, size=(300, 3)).astype(np.float32)
    rest = rng.uniform(0.1, 1.5, size=(2000, 3)).astype(np.float32)
    x = np.concatenate([dense, rest]).astype(np.float32)
    sc = scenes.Scene(x, np.zeros_like(x), (1.6, 1.6, 1.6), ((-0.1,) * 3, (1.7,) * 3),
                      scenes.box_planes((1.6, 1.6, 1.6)), grid=(8, 8, 8))
    p = H.resolved(api.config_params(scorr_k=1e-4), sc)
    g = H.run_gpu(sc, api.config_params(scorr_k=1e-4), "planes", 0)
    r = H.run_oracle(oracle, sc, api.config_params(scorr_k=1e-4), "planes", 0)
    H.assert_integer_parity(g, r, p)
