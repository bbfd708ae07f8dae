"""The reference's scene simulators, headless, on the GPU: set-up, the jet
rule, and one step against the oracle."""
import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import api, simulators
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _oracle_step(oracle, sim, boundary, x, v):
    p = dict(sim.params)
    p["grid_size"] = list(api.resolve_grid(p, sim.domain[1]))
    return oracle.step(p, boundary, sim.domain[0], sim.domain[1], sim.iterations, x, v)


def test_sphere_sim_jet_and_first_step(oracle, gpu):
    sim = simulators.SphereSim()
    assert sim.particles_num == 121  # the set-up add: an 11 x 11 rectangle at spacing 0.1
    x0, v0 = sim.particle.get_particles()
    assert np.all(x0[:, 0] == np.float32(1.25)) and np.all(v0 == np.array([2.8, 0, 0], np.float32))
    sim.simulate_one_step()
    x1, v1 = sim.particle.get_particles()
    r = _oracle_step(oracle, sim, oracle.Boundary(inner=[[3.0, 3.0, 3.0, 3.0]]), x0, v0)
    assert x1.shape == r["x"].shape
    assert H.pos_rel_err(x1, r["x"]) <= H.POS_RTOL
    assert np.abs(v1 - r["v"]).max() <= H.vel_abs_tol(sim.time_step, r["x"])


def test_sphere_sim_jet_rule_and_containment(gpu):
    """A jet every 8th step while under 80% of 60,000 slots; the inner
    sphere keeps every particle within its radius."""
    sim = simulators.SphereSim()
    for _ in range(40):
        sim.simulate_one_step()
    assert sim.particles_num == 121 * 6
    assert sim.elapsed_step == 40 and sim.elapsed_seconds == pytest.approx(40 * sim.time_step)
    x = sim.particles_position()
    assert np.isfinite(x).all()
    r = np.linalg.norm(x.astype(np.float64) - 3.0, axis=1)
    assert r.max() <= 3.0 + 1e-4
    assert sim.particle.flags() == 0


def test_dam_sim_first_step_uses_the_builtin_sphere(oracle, gpu):
    sim = simulators.DamSim()
    assert sim.particles_num == 22 ** 3
    x0, v0 = sim.particle.get_particles()
    sim.simulate_one_step()
    x1, _ = sim.particle.get_particles()
    r = _oracle_step(oracle, sim, oracle.Boundary(builtin_sphere=True), x0, v0)
    assert x1.shape == r["x"].shape
    assert H.pos_rel_err(x1, r["x"]) <= H.POS_RTOL


def test_headless_main_loop_writes_frames(gpu, tmp_path):
    from ssf_pbf_cuda_gb300 import simulate
    out = simulate.main(["--scene", "sphere", "--steps", "16", "--frame-every", "8", "--out", str(tmp_path),
                         "--width", "320", "--height", "180"])
    assert out["particles"] == 121 * 3 and len(out["frames"]) == 2
    for f in out["frames"]:
        data = open(f, "rb").read()
        assert data.startswith(b"P6\n320 180\n255\n") and len(data) == len(b"P6\n320 180\n255\n") + 320 * 180 * 3
