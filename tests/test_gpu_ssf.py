"""Headless screen-space fluid renderer on the GPU against the CPU oracle.

Pass by pass, each GPU pass is fed the GPU's own previous image, so one
kernel is checked at a time:
  depth splat   bit-exact (no FMA, IEEE sqrt and division on both sides);
  blur          |diff| <= 2e-6 in window depth (expf differs by a few ulps);
  normals       bit-exact;
  shading       |diff| <= 2e-5 per channel (expf / powf), 8-bit output
                within one level.
The whole frame from particles is then compared on the integer 8-bit image."""
import numpy as np
import pytest
import torch

from oracle import ssf as S
from ssf_pbf_cuda_gb300 import api, scenes

pytestmark = pytest.mark.gpu

BLUR_TOL = 2e-6
SHADE_TOL = 2e-5


def _frame(r):
    inv, inc = r.frame_constants()
    return S.frame(r.params, inv, inc)


def _images(r):
    return {k: r.image(k) for k in api.SSF_IMAGES}


def _dam():
    return scenes.dam_break(32, 32, 32, (4.0, 2.0, 2.0), scene_id=1)


def _cloud(n, seed):
    """Particles all around the camera: some behind it, some past the far
    plane, some straddling the image edges."""
    g = np.random.default_rng(seed)
    return (g.uniform(-1, 1, (n, 3)) * np.array([14, 10, 30]) + np.array([2, 4, -5])).astype(np.float32)


def _check_passes(r, x, f):
    g = _images(r)
    d = S.splat(f, x)
    assert np.array_equal(g["depth"], d), f"depth: {np.sum(g['depth'] != d)} pixels differ"
    if r.params["blur_passes"]:
        b = S.blur(f, g["blur_input"])
        assert np.max(np.abs(g["blurred"] - b)) <= BLUR_TOL
        assert np.array_equal(g["blurred"] == 1, b == 1)
    n = S.normal(f, g["blurred"])
    assert np.array_equal(g["normal"], n, equal_nan=True)
    c, c8 = S.shade(f, g["depth"], g["normal"])
    ok = np.isfinite(c)
    assert np.array_equal(ok, np.isfinite(g["color"]))
    assert np.max(np.abs(g["color"][ok] - c[ok])) <= SHADE_TOL
    assert np.max(np.abs(g["rgba8"].astype(int) - c8.astype(int))) <= 1
    return g


def test_dam_frame_pass_parity(gpu):
    r = api.SsfRenderer()
    sc = _dam()
    r.render(torch.from_numpy(sc.x).to(gpu))
    g = _check_passes(r, sc.x, _frame(r))
    assert int((g["depth"] < 1).sum()) > 20000
    assert r.launches == 8


@pytest.mark.parametrize("mode", [api.L.PBF_SSF_SPLAT_QUAD, api.L.PBF_SSF_SPLAT_SPRITE])
def test_clipped_cloud_odd_size_pass_parity(gpu, mode):
    """Odd image sides (quad partners past the edge), particles clipped by
    near / far and by the image borders, both splat forms."""
    r = api.SsfRenderer(width=333, height=197, splat_mode=mode)
    x = _cloud(20000, 5)
    r.render(x)
    g = _check_passes(r, x, _frame(r))
    covered = g["depth"] < 1
    assert covered[:, 0].any() and covered[0, :].any() and covered[:, -1].any()


def test_full_frame_against_oracle(gpu):
    """Particles in, 8-bit image out, the oracle running every pass itself."""
    r = api.SsfRenderer()
    sc = _dam()
    r.render(sc.x)
    o = S.render(_frame(r), sc.x, r.params["blur_passes"])
    g = _images(r)
    assert np.array_equal(g["depth"], o["depth"])
    assert np.array_equal(g["blurred"] == 1, o["blurred"] == 1)
    close = np.abs(g["blurred"] - o["blurred"]) <= 1e-5
    assert close.mean() >= 0.9999
    diff = np.abs(g["rgba8"].astype(int) - o["rgba8"].astype(int)).max(axis=2)
    assert (diff <= 1).mean() >= 0.9999


def test_zero_blur_passes_and_empty_frame(gpu):
    r = api.SsfRenderer(width=160, height=90, blur_passes=0)
    x = _cloud(3000, 9)
    r.render(x)
    g = _check_passes(r, x, _frame(r))
    assert np.array_equal(g["blurred"], g["depth"])
    assert r.launches == 5
    r.render(np.zeros((0, 3), np.float32))
    g = _images(r)
    assert np.all(g["depth"] == 1)
    assert np.all(g["rgba8"] == np.array([153, 153, 153, 255], np.uint8))
    assert r.launches == 3


def test_render_particles_and_scene_match_positions(gpu):
    """A handle's and a batch scene's resident particles (float4, count read
    on the device) render exactly like their positions handed over as AoS."""
    sc = _dam()
    params = api.config_params()
    part = api.PbfParticle(params, sc.n, sc.domain_end)
    part.set_particles(sc.x, sc.v)
    api.one_step(part, None, sc.area, 4)
    x, _ = part.get_particles()
    r = api.SsfRenderer()
    r.render_particles(part)
    a = _images(r)
    r.render(x)
    b = _images(r)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k

    bt = api.Batch(4, 4 * sc.n, 1 << 16)
    sid = bt.add_scene(params, sc.n, sc.domain_end, None, sc.area, sc.x, sc.v)
    bt.step(4)
    xs, _ = bt.get_scene(sid)
    r.render_scene(bt, sid)
    c = _images(r)
    r.render(xs)
    d = _images(r)
    for k in c:
        assert np.array_equal(c[k], d[k], equal_nan=True), k


def test_frames_repeat_bit_for_bit(gpu):
    r = api.SsfRenderer()
    x = torch.from_numpy(_cloud(50000, 3)).to(gpu)
    r.render(x)
    a = _images(r)
    r.render(x)
    b = _images(r)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_bad_parameters_are_rejected(gpu):
    base = api.ssf_default_params()
    proj = np.array(base["projection"])
    proj[4] = 0.1  # x_clip depending on y
    for bad in (dict(width=0), dict(height=9000), dict(splat_mode=2), dict(projection=proj),
                dict(point_radius=0.0), dict(near_plane=60.0)):
        with pytest.raises(api.L.PbfError):
            api.SsfRenderer(dict(base, **bad))
