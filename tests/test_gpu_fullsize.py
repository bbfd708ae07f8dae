"""Full-size workloads on the GPU, checked against the oracle where it is
fast (hash + stable counting sort in C) and through size-independent
properties elsewhere."""
import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H

pytestmark = pytest.mark.gpu


def gpu_sort_only(x, grid, cw):
    """The step's sort of x itself: zero velocity and gravity, no iterations."""
    p = api.default_params(body_force=[0.0, 0.0, 0.0], grid_size=list(grid), cell_width=cw, smoothing_length=cw)
    part = api.PbfParticle(p, len(x), (1.0, 1.0, 1.0))
    part.set_particles(x, np.zeros_like(x))
    api.one_step(part, None, ((-1e30,) * 3, (1e30,) * 3), 0)
    return part.neighbor_debug()


@pytest.mark.parametrize("kind", ["uniform", "blobs"])
def test_config3_neighbour_search_bit_exact(oracle, gpu, kind):
    """4,194,304 particles over 2^22 cells: hashes, stable permutation and
    cell ranges equal the oracle's stable counting sort."""
    x, grid, cw = scenes.config3(kind)
    d = gpu_sort_only(x, grid, cw)
    keys, perm, off = oracle.hash_sort(x, cw, grid)
    C = int(np.prod(grid))
    assert np.array_equal(d["perm"], perm)
    assert np.array_equal(d["sorted_hash"], keys[perm])
    ne = off[1:C + 1] > off[:C]
    assert np.array_equal(d["cell_start"] != 0xFFFFFFFF, ne)
    assert np.array_equal(d["cell_start"][ne], off[:C][ne]) and np.array_equal(d["cell_end"][ne], off[1:C + 1][ne])
    # size-independent properties
    assert np.all(np.diff(d["sorted_hash"].astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(d["perm"]), np.arange(len(x), dtype=np.uint32))


@pytest.mark.parametrize("n", [10000, 200000])
def test_single_cell_pile_is_sorted_stably(oracle, gpu, n):
    """Every particle in one cell.  The bucket's order is ascending input
    index (the stable sort's) at any size, bit-exact against the oracle's
    counting sort: 10,000 particles take the small-step path (ranked from
    the particle side), 200,000 the large-step path (ranked per cell); both
    hand the bucket to the block radix sort."""
    rng = np.random.default_rng(n)
    x = rng.uniform(0.31, 0.39, size=(n, 3)).astype(np.float32)
    x[: n // 10] = rng.uniform(0.0, 0.8, size=(n // 10, 3))  # and a few other buckets
    grid, cw = (8, 8, 8), 0.1
    d = gpu_sort_only(x, grid, cw)
    keys, perm, off = oracle.hash_sort(x, cw, grid)
    assert int(np.diff(off[: 8 * 8 * 8 + 1]).max()) > 4096
    assert np.array_equal(d["perm"], perm)
    assert np.array_equal(d["sorted_hash"], keys[perm])


@pytest.mark.parametrize("n", [50000, 300000])
def test_mass_deletion_is_sorted_stably(oracle, gpu, n):
    """A step that deletes about half its particles (far more than 4,096):
    the deleted bucket, last in the order, is stable too, and the live count
    and permutation equal the oracle's."""
    rng = np.random.default_rng(77 + n)
    x = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    grid, cw = (16, 16, 16), 0.1
    amin, amax = (0.0, 0.0, 0.0), (0.5, 1.0, 1.0)
    p = api.default_params(body_force=[0.0, 0.0, 0.0], grid_size=list(grid), cell_width=cw, smoothing_length=cw)
    part = api.PbfParticle(p, n, (1.0, 1.0, 1.0))
    part.set_particles(x, np.zeros_like(x))
    api.one_step(part, None, (amin, amax), 0)
    d = part.neighbor_debug()
    keys, perm, off = oracle.hash_sort(x, cw, grid, amin, amax)
    C = int(np.prod(grid))
    assert n - int(off[C]) > 4096  # deleted
    assert part.num == int(off[C])
    assert np.array_equal(d["perm"], perm)


def test_config2_single_large_step_properties(oracle, gpu):
    """1,048,576 particles, 2^21-cell table, the configured physics: the
    integer pipeline is bit-exact against the oracle, the permutation is a
    permutation, and after one step of one solver iteration (where the
    configured physics is still well conditioned) positions are within 1e-5
    relative and velocities within that error over dt of both the FP32 and
    the FP64 oracle."""
    sc = scenes.config2()
    params = api.config_params()
    g = H.run_gpu(sc, params, "planes", iters=1)
    r = H.run_oracle(oracle, sc, params, "planes", iters=1)
    H.assert_integer_parity(g, r, H.resolved(params, sc))
    assert np.array_equal(np.sort(g["perm"]), np.arange(sc.n, dtype=np.uint32))
    r64 = H.run_oracle(oracle, sc, params, "planes", iters=1, f64=True)
    for ref in (r, r64):
        assert H.pos_rel_err(g["x"], ref["x"]) <= H.POS_RTOL
        assert np.abs(g["v"] - ref["v"]).max(initial=0) <= H.vel_abs_tol(params["time_step"], ref["x"])


def _kinetic(p, v):
    return 0.5 * p["particle_mass"] * float((np.asarray(v, np.float64) ** 2).sum())


def _mean_density_error(oracle, p, x):
    """Mean |rho / rho0 - 1| with each particle's neighbour list from the
    oracle (a step of 0 iterations on x, FP64), W summed in FP64."""
    m, h = p["particle_mass"], p["smoothing_length"]
    rr = oracle.step(p, None, (-1e9,) * 3, (1e9,) * 3, 0, x, np.zeros_like(x), f64=True)
    x0 = np.asarray(x, np.float64)[rr["perm"][:rr["num"]]]
    rho = np.zeros(len(x0))
    for k in range(rr["nbr"].shape[1]):
        sel = rr["nnb"] > k
        q = rr["nbr"][sel, k]
        d2 = ((x0[sel] - x0[q]) ** 2).sum(axis=1)
        rho[sel] += m * 1.56668147065 / h ** 3 * np.clip(1 - d2 / h ** 2, 0, None) ** 3
    return float(np.abs(rho / p["stable_density"] - 1).mean())


# (lattice, box, scene id, steps): dam breaks with stable parameters, run up
# to where FP32 rounding alone keeps both statistics within a few 0.1% of
# FP64 (measured with the FP32 oracle: the 24^3 block within 1.5e-3 through
# step 70, then the splash makes the flow chaotic, 1.5e-2 at step 80; the
# 16^3 block within 5e-3 through step 50, 1.1e-2 at step 60)
LONG_RUNS = [((24, 24, 24), (2.5, 2.0, 2.0), 79, 60), ((16, 16, 16), (2.0, 1.5, 1.5), 77, 40)]


@pytest.mark.parametrize("lat,box,sid,steps", LONG_RUNS, ids=["24cubed_60", "16cubed_40"])
def test_long_run_statistics_match_fp64_oracle(oracle, gpu, lat, box, sid, steps):
    """Longer runs, checked statistically: every 20 steps the GPU run's mean
    density error and kinetic energy are within 1% of the FP64 oracle run
    from the same start (64 neighbour slots, s_corr k = 1e-4, the other
    configured physics unchanged)."""
    sc = scenes.dam_break(*lat, box, scene_id=sid)
    params = api.config_params(scorr_k=1e-4, max_pair_particle_num=64)
    p = H.resolved(params, sc)
    part = api.PbfParticle(p, sc.n, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    b = H.gpu_boundary(sc, "planes")
    xo, vo = sc.x, sc.v
    for s in range(1, steps + 1):
        api.one_step(part, b, sc.area, 4)
        r = H.run_oracle(oracle, sc, params, "planes", 4, f64=True, x=xo, v=vo)
        xo, vo = r["x"], r["v"]
        if s % 20 == 0:
            xg, vg = part.get_particles()
            assert len(xg) == len(xo)
            ke_g, ke_o = _kinetic(p, vg), _kinetic(p, vo)
            de_g, de_o = _mean_density_error(oracle, p, xg), _mean_density_error(oracle, p, xo)
            print(f"{lat} step {s}: kinetic energy {ke_g:.6g} vs {ke_o:.6g} ({abs(ke_g - ke_o) / ke_o:.2e}), "
                  f"mean density error {de_g:.6g} vs {de_o:.6g} ({abs(de_g - de_o) / de_o:.2e})")
            assert abs(ke_g - ke_o) <= 0.01 * ke_o
            assert abs(de_g - de_o) <= 0.01 * de_o


@pytest.mark.parametrize("grid", [(4, 4, 4), (16, 8, 8), (16, 16, 8), (16, 16, 16), (32, 16, 16),
                                  (32, 32, 16), (32, 32, 32), (64, 32, 32)])
def test_one_block_scan_every_table_size(oracle, gpu, grid):
    """Tables of up to 65,536 cells (plus the deleted bucket) are scanned by
    one block: up to 16 rounds of 1,024 cells held in registers (1, 2, 3, 5
    and 9 rounds here), larger tables round by round.  Cell ranges and the
    permutation equal the oracle's for a table of each size (particles spread
    over it, some cells empty)."""
    g = np.random.default_rng(sum(grid))
    cw = 0.1
    n = 3 * int(np.prod(grid)) // 4
    x = (g.random((n, 3)) * np.asarray(grid) * cw).astype(np.float32)
    d = gpu_sort_only(x, grid, cw)
    keys, perm, off = oracle.hash_sort(x, cw, grid)
    C = int(np.prod(grid))
    assert np.array_equal(d["perm"], perm)
    ne = off[1:C + 1] > off[:C]
    assert 0 < ne.sum() < C
    assert np.array_equal(d["cell_start"] != 0xFFFFFFFF, ne)
    assert np.array_equal(d["cell_start"][ne], off[:C][ne]) and np.array_equal(d["cell_end"][ne], off[1:C + 1][ne])


@pytest.mark.parametrize("max_pair", [30, 64, 100])
def test_large_step_list_slots(oracle, gpu, max_pair):
    """A large step (147,456 particles) collects each block's neighbour lists
    in shared memory when they fit (tile x slots x 4 B: 29.7 KB, 64.5 KB past
    the default 48 KB limit) and stores them directly when they do not
    (101 KB): in every case hashes, permutation, cell ranges and neighbour
    lists equal the oracle's."""
    sc = scenes.dam_break(64, 48, 48, (8.0, 4.0, 4.0), scene_id=90 + max_pair)
    params = api.config_params(max_pair_particle_num=max_pair, scorr_k=1e-4)
    g = H.run_gpu(sc, params, "planes", iters=1)
    r = H.run_oracle(oracle, sc, params, "planes", iters=1)
    H.assert_integer_parity(g, r, H.resolved(params, sc))


def _dense_cells_scene():
    """140,000 particles: 20,000 packed into eight cells (2,500 a cell, so
    buckets above 255 members, walked whole, and cells of far more than 32
    particles), the rest uniform over the box."""
    rng = np.random.default_rng(123)
    k = np.arange(20000) % 8
    corner = np.stack([(k & 1) * 0.1, ((k >> 1) & 1) * 0.1, ((k >> 2) & 1) * 0.1], axis=1) + 1.2
    dense = corner + rng.uniform(0.005, 0.095, size=(20000, 3))
    rest = rng.uniform(0.05, 3.15, size=(120000, 3))
    x = np.concatenate([dense, rest]).astype(np.float32)
    return scenes.Scene(x, np.zeros_like(x), (3.2, 3.2, 3.2), ((-0.1,) * 3, (3.3,) * 3),
                        scenes.box_planes((3.2, 3.2, 3.2)), grid=(16, 16, 16))


HARD_TABLES = {
    # buckets mixing up to 8 alias classes (cells 16 apart share a bucket)
    "aliased": lambda: scenes.dam_break(64, 48, 48, (8.0, 4.0, 4.0), scene_id=131, grid=(16, 16, 16)),
    # 2 cells on x: every bucket walked whole, wrapped buckets visited twice
    "small_axes": lambda: scenes.dam_break(64, 48, 48, (8.0, 4.0, 4.0), scene_id=132, grid=(2, 16, 16)),
    "dense_cells": _dense_cells_scene,
}


@pytest.mark.parametrize("case", sorted(HARD_TABLES))
def test_large_step_lists_on_hard_tables(oracle, gpu, case):
    """Large steps (over 131,072 particle slots: the per-cell rank, the
    one-lane walk) on hard tables: buckets mixing alias classes (walked
    through the class-grouped walk copy), an axis of 2 cells (buckets
    walked whole, wrapped cells visited twice, 64 list slots so the
    duplicates fit), and cells of 2,500 particles (buckets of more than 255
    members, walked whole; every list capped).  Hashes, permutation, cell
    ranges and lists equal the oracle's slot for slot."""
    sc = HARD_TABLES[case]()
    assert sc.n > 131072
    params = api.config_params(scorr_k=1e-4, max_pair_particle_num=64 if case == "small_axes" else 30)
    g = H.run_gpu(sc, params, "planes", iters=0)
    r = H.run_oracle(oracle, sc, params, "planes", iters=0)
    H.assert_integer_parity(g, r, H.resolved(params, sc))
