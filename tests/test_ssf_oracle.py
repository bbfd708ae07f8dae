"""Screen-space fluid rendering on the CPU: the library's reference camera
(host code, no GPU needed) against an independent restatement, and the
oracle's passes against closed-form cases."""
import numpy as np
import pytest

from oracle import ssf as S

f32 = np.float32


@pytest.fixture(scope="module")
def params(lib):
    from ssf_pbf_cuda_gb300 import api
    return api.ssf_default_params()


def test_default_camera_matches_controls_restatement(params):
    """pbf_ssf_params_init = controls.cpp's first frame, bit for bit."""
    cam = S.reference_camera(1280, 720)
    assert np.array_equal(params["projection"], cam["projection"])
    assert np.array_equal(params["view"], cam["view"])
    # tanf's last bit belongs to the maths library (the reference's was MSVC's)
    assert params["blur_scale"] == pytest.approx(float(cam["blur_scale"]), rel=1e-6)
    assert params["point_scale"] == pytest.approx(float(cam["point_scale"]), rel=0, abs=0)
    # glm::perspective takes the 45 as radians: tan(22.5) = tan(22.5 - 7 pi)
    assert params["projection"][5] == pytest.approx(1.0 / np.tan(22.5), rel=1e-5)
    assert (params["width"], params["height"], params["blur_passes"]) == (1280, 720, 3)
    assert params["point_radius"] == pytest.approx(0.18) and params["blur_radius"] == pytest.approx(5.5e-6)


def _centre_particle(params, dist):
    """A world point straight ahead of the camera at view depth -dist."""
    V = np.asarray(params["view"], np.float64).reshape(4, 4).T
    return (np.linalg.inv(V) @ np.array([0.0, 0.0, -dist, 1.0]))[:3].astype(f32)[None, :]


def _ndc_z(params, z_eye):
    Pm = np.asarray(params["projection"], np.float64)
    return (Pm[10] * z_eye + Pm[14]) / (Pm[11] * z_eye + Pm[15])


@pytest.mark.parametrize("mode", [0, 1])
def test_single_particle_footprint_and_depth(params, mode):
    """One particle on the view axis: the disc's area and its front depth."""
    p = dict(params, splat_mode=mode)
    f = S.frame(p)
    x = _centre_particle(p, 8.0)
    d = S.splat(f, x)
    r = p["point_radius"]
    Pm = np.asarray(p["projection"])
    if mode == 0:  # quad of side r, disc of diameter r in view space
        ax = 0.5 * r * Pm[0] / 8.0 * p["width"] / 2
        ay = 0.5 * r * Pm[5] / 8.0 * p["height"] / 2
    else:  # point of size r * scale / dist pixels, disc inscribed
        ax = ay = 0.5 * r * p["point_scale"] / 8.0
    covered = int((d < 1).sum())
    assert covered == pytest.approx(np.pi * ax * ay, rel=0.1)
    # the nearest fragment is near the disc centre, pushed up to r towards the
    # camera, and never nearer than that
    front = _ndc_z(p, -8.0 + r)
    assert front - 1e-7 <= float(d.min()) <= front + 1e-5
    assert float(d[d < 1].max()) == pytest.approx(_ndc_z(p, -8.0), abs=2e-4)


def test_particles_behind_or_beyond_clip_are_dropped(params):
    f = S.frame(params)
    V = np.asarray(params["view"], np.float64).reshape(4, 4).T
    Vi = np.linalg.inv(V)
    pts = [Vi @ np.array([0, 0, z, 1.0]) for z in (2.0, -0.05, -60.0)]  # behind, inside near, beyond far
    x = np.array([q[:3] for q in pts], f32)
    assert np.all(S.splat(f, x) == 1.0)


def test_empty_frame_is_the_clear_colour(params):
    f = S.frame(params)
    r = S.render(f, np.zeros((0, 3), f32))
    assert np.all(r["depth"] == 1) and np.all(r["blurred"] == 1)
    assert np.all(r["color"] == np.asarray(params["clear_color"], f32))
    assert np.all(r["rgba8"] == np.array([153, 153, 153, 255], np.uint8))


def test_blur_keeps_a_constant_depth_and_normals_of_a_plane(params):
    """A full-screen constant depth is a fixed point of the blur (the weights
    normalise) and a plane facing the camera has normal +z."""
    p = dict(params, width=96, height=64)
    f = S.frame(p)
    d = np.full((64, 96), 0.97, f32)
    b = S.blur(f, d)
    assert np.max(np.abs(b - d)) < 2e-6
    n = S.normal(f, d)
    assert np.allclose(n[..., :3], [0, 0, 1], atol=1e-4) and np.all(n[..., 3] == 1)


def test_blur_leaves_empty_pixels_and_thickness_zero_shows_background(params):
    p = dict(params, width=64, height=48, thickness=0.0)
    f = S.frame(p)
    d = np.ones((48, 64), f32)
    d[10:30, 20:40] = 0.98
    b = S.blur(f, d)
    assert np.all(b[d == 1] == 1)
    c, c8 = S.shade(f, d, S.normal(f, b))
    assert np.allclose(c[..., :3], 0.6, atol=1e-7)  # alpha 0: the clear colour shows through
