"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
analytic cases (kernel constants and normalisation, free fall, symmetric
pairs, exact lattice neighbourhoods, plane and sphere projections, hash wrap,
grid sizing) and, in test_golden_reference.py, by outputs of the reference's
own CUDA step."""
import math

import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import scenes

H = 0.1


def base_params(**kw):
    p = {
        "stable_density": 1000.0, "stable_distance": 0.05, "particle_mass": 0.125, "smoothing_length": H,
        "time_step": 1 / 120, "relaxation": 600.0, "xsph_parameter": 0.01, "vc_parameter": 0.0005,
        "body_force": [0.0, -9.8, 0.0], "max_pair_particle_num": 30, "tensile_mode": 0, "scorr_k": 0.1,
        "scorr_n": 4, "scorr_dq": 0.2, "xsph_mode": 0, "vorticity_mode": 0, "max_collision_passes": 64,
        "cell_width": H, "grid_size": [32, 32, 32],
    }
    p.update(kw)
    return p


def far_boundary(O):
    # one plane far away: never touched, and the builtin sphere is not used
    return O.Boundary(plane_pts=[[0, -100, 0]], plane_nrm=[[0, 1, 0]])


BIG = ((-1e6,) * 3, (1e6,) * 3)


def test_poly6_and_spiky_constants(oracle):
    inv_h = np.float32(1.0) / np.float32(H)
    w0 = oracle.wpoly6(0.0, float(inv_h))
    assert w0 == pytest.approx(315.0 / (64.0 * math.pi * H ** 3), rel=1e-6)
    d0 = oracle.wspiky_deriv(0.0, float(inv_h))
    assert d0 == pytest.approx(-45.0 / (math.pi * H ** 4), rel=1e-6)
    assert oracle.wpoly6(float(H) * 1.0001, float(inv_h)) == 0.0
    assert oracle.wspiky_deriv(float(H) * 1.0001, float(inv_h)) == 0.0


def test_poly6_normalisation():
    # integral of W over space = 1 (midpoint rule on a fine lattice)
    n = 80
    d = 2 * H / n
    c = (np.arange(n) + 0.5) * d - H
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    r2 = (x * x + y * y + z * z) / H ** 2
    w = np.where(r2 <= 1, 1.56668147065 / H ** 3 * (1 - r2) ** 3, 0.0)
    assert w.sum() * d ** 3 == pytest.approx(1.0, abs=2e-3)


def test_free_fall_single_particle(oracle):
    x = np.array([[1.0, 2.0, 3.0]], np.float32)
    v = np.array([[0.5, -1.0, 0.25]], np.float32)
    p = base_params()
    r = oracle.step(p, far_boundary(oracle), *BIG, 4, x, v)
    dt = np.float32(p["time_step"])
    g = np.array(p["body_force"], np.float32)
    vs = (g.astype(np.float64) * dt + v[0]).astype(np.float32)
    xs = (vs.astype(np.float64) * dt + x[0]).astype(np.float32)
    np.testing.assert_array_max_ulp(r["x"][0], xs, maxulp=1)
    assert r["num"] == 1 and r["nnb"][0] == 1  # only itself


def test_two_particle_symmetry(oracle):
    c = np.array([1.0, 1.0, 1.0])
    x = np.array([c - [0.025, 0, 0], c + [0.025, 0, 0]], np.float32)
    v = np.zeros_like(x)
    p = base_params(body_force=[0.0, 0.0, 0.0])
    for f64 in (False, True):
        r = oracle.step(p, far_boundary(oracle), *BIG, 4, x, v, f64=f64)
        xo = r["x"].astype(np.float64)
        assert np.allclose(xo.mean(axis=0), c, atol=1e-6)
        np.testing.assert_allclose(r["v"][0], -r["v"][1], atol=1e-6)
        assert abs(r["lambda0"][0] - r["lambda0"][1]) < 1e-9


def test_exact_lattice_neighbourhood_and_lambda(oracle):
    """A particle inside a perfect lattice at spacing 0.5h has exactly 27
    neighbours (|d|^2 < 4 in lattice units); its lambda0 equals the closed
    form from the lattice sums."""
    # dyadic h and spacing: every lattice coordinate is exact in float32
    h, s = 0.125, 0.0625
    m, rho0 = 1000.0 * s ** 3, 1000.0
    x = scenes.lattice(9, 9, 9, s, (1.0 + 0.5 * s,) * 3)
    p = base_params(body_force=[0.0, 0.0, 0.0], smoothing_length=h, cell_width=h, particle_mass=m,
                    grid_size=[32, 32, 32])
    r = oracle.step(p, far_boundary(oracle), *BIG, 1, x, np.zeros_like(x), f64=True)
    xs = r["x"]
    centre = np.argmin(np.abs(xs - xs.mean(axis=0)).sum(axis=1))
    assert r["nnb"][centre] == 27
    d = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], np.float64) * s
    rr = np.sqrt((d ** 2).sum(axis=1))
    alpha, beta = 1.56668147065 / h ** 3, -14.3239448745 / h ** 4
    W = alpha * (1 - (rr / h) ** 2) ** 3
    g = np.where(rr[:, None] > 0, (beta * (1 - rr / h) ** 2 / np.where(rr > 0, rr, 1))[:, None] * d, 0.0)
    C = W.sum() * m / rho0 - 1
    K = (g ** 2).sum() + (g.sum(axis=0) ** 2).sum()
    lam = C / ((m / rho0) ** 2 * K + 600.0)
    assert r["lambda0"][centre] == pytest.approx(lam, rel=1e-6)


def test_plane_projection(oracle):
    # falls through the floor y = 0 within one step -> projected onto it
    x = np.array([[1.0, 0.01, 1.0]], np.float32)
    v = np.array([[0.0, -5.0, 0.0]], np.float32)
    b = oracle.Boundary(plane_pts=[[0, 0, 0]], plane_nrm=[[0, 1, 0]])
    r = oracle.step(base_params(), b, *BIG, 1, x, v)
    assert abs(float(r["x"][0, 1])) < 1e-6
    assert r["x"][0, 0] == pytest.approx(1.0) and r["x"][0, 2] == pytest.approx(1.0)
    assert r["collision_passes"] >= 2


def test_inner_sphere_projection(oracle):
    c, rad = np.array([3.0, 3.0, 3.0]), 3.0
    x = np.array([[3.0, 6.5, 3.0]], np.float32)  # outside the fixed sphere
    r = oracle.step(base_params(body_force=[0, 0, 0]), None, *BIG, 1, x, np.zeros_like(x))
    dist = np.linalg.norm(r["x"][0].astype(np.float64) - c)
    assert dist == pytest.approx(rad - 1e-4 * 3.5, abs=1e-5)


def test_hash_wrap_and_negative_coordinates(oracle):
    xs = np.array([[-0.05, 0.05, 0.05], [0.05, -0.05, 0.05], [3.25, 0.05, 0.05], [0.05, 0.05, -1e-7]], np.float32)
    keys, perm, off = oracle.hash_sort(xs, 0.1, (32, 16, 16))
    # gx = floor(-0.5) = -1 -> 31;  gy = -1 -> 15;  gx = 32 -> 0;  gz = floor(-1e-6) = -1 -> 15
    assert list(keys) == [31, 15 * 32, 0, 15 * 32 * 16]


def test_area_deletion_key(oracle):
    xs = np.array([[0.5, 0.5, 0.5], [2.5, 0.5, 0.5]], np.float32)
    keys, perm, off = oracle.hash_sort(xs, 0.1, (16, 16, 16), area_min=(0, 0, 0), area_max=(1, 1, 1))
    C = 16 ** 3
    assert keys[1] == C and off[C] == 1 and perm[1] == 1


def test_calc_grid_size(oracle):
    assert oracle.calc_grid_size(0.2, (4.0, 2.0, 2.0)) == (32, 16, 16)
    assert oracle.calc_grid_size(0.14, (7.0, 7.0, 7.0)) == (64, 64, 64)
    with pytest.raises(ValueError):
        oracle.calc_grid_size(0.001, (7.0, 7.0, 7.0))


def test_stable_sort_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    xs = rng.uniform(-0.3, 1.9, size=(20000, 3)).astype(np.float32)
    keys, perm, off = oracle.hash_sort(xs, 0.1, (16, 8, 8))
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    C = 16 * 8 * 8
    cnt = np.bincount(keys, minlength=C + 1)
    assert np.array_equal(off[1:], np.cumsum(cnt))


def test_neighbour_sets_match_brute_force(oracle):
    """Below the cap the listed set equals all particles within h (pairs
    within 1e-5 of the cutoff are ambiguous in FP32 and skipped)."""
    rng = np.random.default_rng(11)
    x = rng.uniform(0.0, 0.8, size=(600, 3)).astype(np.float32)
    p = base_params(grid_size=[16, 16, 16], max_pair_particle_num=64, body_force=[0, 0, 0])
    r = oracle.step(p, far_boundary(oracle), *BIG, 0, x, np.zeros_like(x))
    x0 = x[r["perm"]].astype(np.float64)  # v = 0, g = 0 -> x* = x
    d2 = ((x0[:, None, :] - x0[None, :, :]) ** 2).sum(axis=2)
    for i in range(len(x0)):
        lst = set(r["nbr"][i, :r["nnb"][i]].tolist())
        amb = np.abs(d2[i] - H * H) < 1e-5 * H * H
        want = set(np.nonzero((d2[i] < H * H) & ~amb)[0].tolist())
        got = {j for j in lst if not amb[j]}
        assert got == want, i


def test_cap_keeps_first_in_traversal_order(oracle):
    """With the 29-slot cap, the kept neighbours are the first ones met in the
    z, y, x cell walk (ascending sorted index inside a cell)."""
    rng = np.random.default_rng(12)
    x = rng.uniform(0.0, 0.5, size=(3000, 3)).astype(np.float32)
    p = base_params(grid_size=[8, 8, 8], body_force=[0, 0, 0])
    r = oracle.step(p, far_boundary(oracle), *BIG, 0, x, np.zeros_like(x))
    p64 = base_params(grid_size=[8, 8, 8], body_force=[0, 0, 0], max_pair_particle_num=256)
    r64 = oracle.step(p64, far_boundary(oracle), *BIG, 0, x, np.zeros_like(x))
    assert r["nnb"].max() == 29
    for i in range(0, len(x), 97):
        full = r64["nbr"][i, :r64["nnb"][i]]
        assert np.array_equal(r["nbr"][i, :r["nnb"][i]], full[:29])


def test_f32_and_f64_oracles_agree_on_a_stable_scene(oracle):
    from tests import helpers as Hh
    sc = Hh.reflike_dam(12, scene_id=3)
    p = Hh.resolved(Hh.reflike_params(), sc)
    b = oracle.Boundary(plane_pts=sc.planes[0], plane_nrm=sc.planes[1])
    a = oracle.step(p, b, sc.area[0], sc.area[1], 4, sc.x, sc.v)
    c = oracle.step(p, b, sc.area[0], sc.area[1], 4, sc.x, sc.v, f64=True)
    assert Hh.pos_rel_err(a["x"], c["x"]) < 2e-6


def test_configured_physics_amplifies_rounding_over_iterations(oracle):
    """The benchmark's configured physics (spacing h/2, eps 600, textbook
    s_corr k = 0.1, n = 4) on the 32,768-particle dam, the same input in the
    FP32 and the FP64 oracle (the same neighbour lists and permutation): the
    rounding difference between the two, 6e-7 relative after one solver
    iteration, grows about a hundredfold per iteration, past 1e-3 by the
    third and to order one by the fourth.  So no FP32 implementation that is
    not bit-identical to the FP32 oracle can stay within 1e-5 of it at four
    iterations there; the GPU tests bound that physics at one iteration."""
    from ssf_pbf_cuda_gb300 import api
    from tests import helpers as Hh
    sc = scenes.config1()
    p = Hh.resolved(api.config_params(), sc)
    b = oracle.Boundary(plane_pts=sc.planes[0], plane_nrm=sc.planes[1])
    dist = []
    for iters in (1, 2, 3, 4):
        a = oracle.step(p, b, sc.area[0], sc.area[1], iters, sc.x, sc.v)
        c = oracle.step(p, b, sc.area[0], sc.area[1], iters, sc.x, sc.v, f64=True)
        assert np.array_equal(a["perm"], c["perm"])
        dist.append(Hh.pos_rel_err(a["x"], c["x"]))
    assert dist[0] < 1e-5 and dist[2] > 1e-3 and dist[3] > 1.0, dist
    assert all(dist[k + 1] > 10 * dist[k] for k in range(3)), dist


def test_collision_bound_reported(oracle):
    x = np.array([[1.1, 1.1, 1.1]], np.float32)
    b = oracle.Boundary(plane_pts=scenes.box_planes((1, 1, 1))[0], plane_nrm=scenes.box_planes((1, 1, 1))[1])
    p = base_params(max_collision_passes=1)
    r = oracle.step(p, b, *BIG, 1, x, np.zeros_like(x))
    assert r["collision_passes"] == -1
