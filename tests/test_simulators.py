"""Scene simulators on the CPU: their parameters restate the reference's
init conditions (no GPU needed: only host-side parameter set-up)."""
import numpy as np
import pytest

f32 = np.float32


@pytest.mark.parametrize("space, dt, k", [(0.1, 0.007, 2.0), (0.16, 0.015, 1.0)])
def test_init_params_follow_the_init_conditions(lib, space, dt, k):
    """pbf_sphere_init_cond.cpp:13-21 / pbf_dam_init_cond.cpp:13-21."""
    from ssf_pbf_cuda_gb300 import simulators
    p = simulators.init_params(space, dt, k)
    s = f32(space)
    assert p["stable_distance"] == float(s)
    assert p["particle_mass"] == float(f32((float(s) ** 3) * 1000.0))  # pow(float, 3) in double, stored as float
    assert p["smoothing_length"] == float(f32(1.4) * s)
    assert p["relaxation"] == float(f32(k) / (s * s))
    assert p["time_step"] == float(f32(dt))
    assert p["xsph_mode"] == 0 and p["vorticity_mode"] == 0  # inactive in the reference's step
    assert p["cell_width"] == p["smoothing_length"]


def test_renderer_scales_follow_the_target_height(lib):
    from ssf_pbf_cuda_gb300 import api
    d = api.ssf_default_params()
    e = api.ssf_default_params(width=640, height=360)
    assert e["blur_scale"] == pytest.approx(d["blur_scale"] / 2, rel=1e-6)
    assert e["point_scale"] == pytest.approx(d["point_scale"] / 2, rel=1e-6)
    assert api.ssf_default_params(height=360, blur_scale=5.0)["blur_scale"] == 5.0
