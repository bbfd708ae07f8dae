"""Pinning against the reference's own CUDA step (fixtures made by
tests/golden/make_golden.py from the reference sources built for sm_103a).

CPU part: the oracle reproduces the reference's outputs.  GPU part: the
CUDA path reproduces them too.  Integers are compared on sort-invariant
forms (the reference's counting sort orders a cell's particles by atomic
arrival), positions within 1e-5 relative by particle id."""
import numpy as np
import pytest

from tests import helpers as H

FILES = H.golden_files()
pytestmark = pytest.mark.skipif(not FILES, reason="no golden fixtures generated yet")
IDS = [f.split("/")[-1][:-4] for f in FILES]


def oracle_outputs(O, sc, p, iters, fx, f64=False):
    r = O.step(p, H.golden_oracle_boundary(O, fx), sc.area[0], sc.area[1], iters, sc.x, sc.v, f64=f64)
    C = int(np.prod(p["grid_size"]))
    lay = H.oracle_reference_layout(r, p["max_pair_particle_num"], C)
    lay.update(num=r["num"], x=r["x"], v=r["v"])
    return lay, C


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_oracle_matches_reference_ieee(oracle, path):
    sc, p, iters, fx = H.golden_case(path)
    ref = H.reference_of(fx, "ieee")
    for f64 in (False, True):
        ours, C = oracle_outputs(oracle, sc, p, iters, fx, f64)
        rep = H.compare_to_reference(ours, ref, C)
        assert rep["neighbor_set_mismatches"] == 0
        assert rep["pos_rel_err"] <= H.POS_RTOL, rep
        assert rep["vel_abs_err"] <= H.vel_abs_tol(p["time_step"], ref["x"]), rep


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_oracle_close_to_reference_fast_math(oracle, path):
    """The shipped fast-math build: same integers, positions within 1e-4."""
    sc, p, iters, fx = H.golden_case(path)
    ref = H.reference_of(fx, "fast")
    if not ref:
        pytest.skip("fixture has no fast-math run (the scene touches the boundary)")
    ours, C = oracle_outputs(oracle, sc, p, iters, fx)
    rep = H.compare_to_reference(ours, ref, C)
    assert rep["pos_rel_err"] <= 1e-4, rep


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_cuda_matches_reference(gpu, path):
    from ssf_pbf_cuda_gb300 import api
    sc, p, iters, fx = H.golden_case(path)
    ref = H.reference_of(fx, "ieee")
    part = api.PbfParticle(p, sc.n + 64, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    api.one_step(part, H.golden_gpu_boundary(fx), sc.area, iters)
    x, v = part.get_particles()
    ours = part.neighbor_debug()
    ours.update(x=x, v=v)
    rep = H.compare_to_reference(ours, ref, int(np.prod(p["grid_size"])))
    assert rep["neighbor_set_mismatches"] == 0
    assert rep["pos_rel_err"] <= H.POS_RTOL, rep
    assert rep["vel_abs_err"] <= H.vel_abs_tol(p["time_step"], ref["x"]), rep
