"""The benchmark workloads' own physics, unchanged (api.config_params():
textbook s_corr k = 0.1, n = 4, dq = 0.2h; XSPH c = 0.01 and vorticity
confinement eps = 0.0005 over the step's neighbour list), on the
32,768-particle dam and on a 32-scene slice of the batched workload.

At spacing h/2 with eps = 600 this physics is chaotic within one step: each
solver iteration amplifies a perturbation about a hundredfold.  On the CPU
the FP32 and FP64 oracles differ by 6e-7 (relative, 0.1 m floor) after one
iteration, 7e-5 after two, 4e-3 after three and ~30 after four, and moving
every input coordinate by one ulp moves the FP32 result by ~20.  So the
1e-5 single-step bound is asserted where the problem is well conditioned:
  - one iteration (lambda of iteration 0, delta-p, s_corr, collision, the
    velocity update and the post passes): positions within 1e-5 of both
    oracles, velocities within that error over dt;
  - four iterations: the integer pipeline (hashes, stable permutation, cell
    ranges, neighbour lists), which the iterations do not feed back into,
    bit for bit, and every particle finite.
The distances at two to four iterations are printed (pytest -s)."""
import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _assert_close(x, v, r, dt):
    assert H.pos_rel_err(x, r["x"]) <= H.POS_RTOL, H.pos_rel_err(x, r["x"])
    assert np.abs(np.asarray(v, np.float64) - r["v"]).max(initial=0) <= H.vel_abs_tol(dt, r["x"])


def test_config1_one_iteration(oracle, gpu):
    sc, p = scenes.config1(), api.config_params()
    g = H.run_gpu(sc, p, "planes", iters=1)
    for f64 in (False, True):
        r = H.run_oracle(oracle, sc, p, "planes", 1, f64=f64)
        H.assert_integer_parity(g, r, H.resolved(p, sc))
        _assert_close(g["x"], g["v"], r, p["time_step"])


def test_config1_four_iterations(oracle, gpu):
    sc, p = scenes.config1(), api.config_params()
    g = H.run_gpu(sc, p, "planes", iters=4)
    r = H.run_oracle(oracle, sc, p, "planes", 4)
    H.assert_integer_parity(g, r, H.resolved(p, sc))
    assert np.isfinite(g["x"]).all() and np.isfinite(g["v"]).all()
    for it in (2, 3, 4):
        gi = H.run_gpu(sc, p, "planes", iters=it, debug=False)
        r32 = H.run_oracle(oracle, sc, p, "planes", it)
        r64 = H.run_oracle(oracle, sc, p, "planes", it, f64=True)
        print(f"config 1, k = 0.1, {it} iterations: GPU vs FP32 oracle {H.pos_rel_err(gi['x'], r32['x']):.3g}, "
              f"vs FP64 {H.pos_rel_err(gi['x'], r64['x']):.3g}, FP32 vs FP64 {H.pos_rel_err(r32['x'], r64['x']):.3g}")


def _slice4():
    return [(sc, api.config_params()) for sc in scenes.config4(256)[:32]]


def _batch(items):
    n = sum(sc.n for sc, _ in items)
    cells = sum(int(np.prod(H.resolved(p, sc)["grid_size"])) + 1 for sc, p in items)
    b = api.Batch(len(items), n, cells, 30)
    ids = [b.add_scene(H.resolved(p, sc), sc.n, sc.domain_end, H.gpu_boundary(sc, "planes"), sc.area, sc.x, sc.v)
           for sc, p in items]
    return b, ids


def test_config4_slice_one_iteration(oracle, gpu):
    """32 scenes of the batched workload through the batched engine."""
    items = _slice4()
    b, ids = _batch(items)
    b.step(1)
    for (sc, p), sid in zip(items, ids):
        x, v = b.get_scene(sid)
        for f64 in (False, True):
            _assert_close(x, v, H.run_oracle(oracle, sc, p, "planes", 1, f64=f64), p["time_step"])


def test_config4_full_one_iteration(oracle, gpu):
    """The whole batched workload (256 scenes, 5,710,854 particles) in one
    batch, stepped through the packed-input step the benchmark times: every
    scene within 1e-5 relative of the FP32 and of the FP64 oracle after one
    iteration."""
    import torch
    items = [(sc, api.config_params()) for sc in scenes.config4(256)]
    b, ids = _batch(items)
    x = torch.from_numpy(np.concatenate([sc.x for sc, _ in items]).astype(np.float32)).cuda()
    v = torch.from_numpy(np.concatenate([sc.v for sc, _ in items]).astype(np.float32)).cuda()
    b.step_packed(1, x, v, [sc.n for sc, _ in items])
    for (sc, p), sid in zip(items, ids):
        xg, vg = b.get_scene(sid)
        for f64 in (False, True):
            _assert_close(xg, vg, H.run_oracle(oracle, sc, p, "planes", 1, f64=f64), p["time_step"])


def test_config4_slice_four_iterations(oracle, gpu):
    items = _slice4()
    b, ids = _batch(items)
    b.step(4)
    worst32 = worst64 = 0.0
    for (sc, p), sid in zip(items, ids):
        x, v = b.get_scene(sid)
        assert np.isfinite(x).all() and np.isfinite(v).all()
        r32 = H.run_oracle(oracle, sc, p, "planes", 4)
        assert len(x) == r32["num"]
        worst32 = max(worst32, H.pos_rel_err(x, r32["x"]))
        worst64 = max(worst64, H.pos_rel_err(x, H.run_oracle(oracle, sc, p, "planes", 4, f64=True)["x"]))
    print(f"config 4 slice, k = 0.1, 4 iterations: worst scene GPU vs FP32 {worst32:.3g}, vs FP64 {worst64:.3g}")
