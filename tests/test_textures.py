"""Texture restatement pins (CPU oracle): bitmap filters on images whose answer is
known in closed form, chessboard cell parity, mip-chain levels and the uv
derivatives of camera rays. GPU parity for the same textures is in
test_gpu_textures.py."""
import json
import math

import numpy as np
import pytest

import imgenc
from helpers import write


def _scene(tmp_path, params, assets):
    """A scene whose floor is a Disney material with the given parameters (textures
    are numbered in Disney's reading order: base_color, roughness, anisotropic, ...).
    Returns the scene text and directory."""
    bsdf = {"type": "disney", **params}
    sc = {
        "camera": {"type": "perspective", "fov": 40.0, "resolution": [8, 8], "origin": [0, 2, 3], "target": [0, 0, 0]},
        "sampler": {"type": "independent", "sample_count": 1, "seed": 1},
        "assets": [{"name": n, "type": t, "location": n + ".img", **o} for n, (t, o, _) in assets.items()],
        "scene": [{"to_world": {"rotate": {"axis": [1, 0, 0], "angle": -90.0}}, "shape": {"type": "rectangle"},
                   "bsdf": bsdf}],
        "accel": {"type": "embree"},
        "renderer": {"type": "path", "max_depth": 3},
    }
    _, text, d = write(tmp_path, "tex", sc, {n + ".img": data for n, (_, _, data) in assets.items()})
    return text, d


def _bitmap(name, **kw):
    return {"type": "bitmap", "asset_name": name, **kw}


def test_bilinear_reproduces_a_ramp(oracle, tmp_path):
    """On texel values v(x) = x, the bilinear filter returns u (W - 1) - 1/2 away from
    the edges (the half-texel shift of bitmap.cpp:200-214) and nearest returns the
    texel index u (W - 1) truncated."""
    W = 64
    img = np.tile(np.arange(W).reshape(1, W, 1), (4, 1, 1))
    text, d = _scene(tmp_path, {"roughness": _bitmap("ramp"), "anisotropic": _bitmap("ramp", filter="nearest")},
                     {"ramp": ("image_default", {"channel": 1}, imgenc.png(img))})
    o = oracle.OracleScene(text, d)
    u = np.linspace(0.05, 0.95, 101, dtype=np.float32)
    uv = np.stack([u, np.full_like(u, 0.5)], 1)
    lin = o.texture_eval(0, uv)[:, 0] * 255
    near = o.texture_eval(1, uv)[:, 0] * 255
    f = u.astype(np.float64) * (W - 1)
    assert np.allclose(lin, f - 0.5, atol=2e-3)
    assert np.array_equal(np.round(near), np.floor(f))
    o.close()


@pytest.mark.parametrize("flt", ["nearest", "bilinear", "trilinear", "anisotropic"])
def test_constant_image_under_every_filter(oracle, tmp_path, flt):
    img = np.full((32, 16, 3), [200, 100, 50])
    text, d = _scene(tmp_path, {"base_color": _bitmap("c", filter=flt, wrap="repeat")},
                     {"c": ("image_default", {"is_to_linear": False}, imgenc.png(img))})
    o = oracle.OracleScene(text, d)
    rng = np.random.default_rng(1)
    uv = rng.uniform(-2, 3, size=(500, 2)).astype(np.float32)
    duv = (rng.normal(size=(500, 4)) * 10.0 ** rng.uniform(-4, 0, size=(500, 1))).astype(np.float32)
    v = o.texture_eval(0, uv, duv)
    assert np.allclose(v, np.array([200, 100, 50], np.float32) / 255, rtol=1e-6)
    o.close()


def test_trilinear_selects_mip_levels(oracle, tmp_path):
    """With a footprint of 2^k texels the trilinear filter reads mip level k alone;
    on a 2-colour checker of 1-texel cells level 0 alternates and every coarser
    level of the tent pyramid is close to the mean colour (the last row and
    column are clamped, not wrapped, when levels are built: bitmap.cpp:172-178)."""
    W = 32
    yy, xx = np.mgrid[0:W, 0:W]
    img = ((xx + yy) % 2 * 255)[..., None]
    text, d = _scene(tmp_path, {"roughness": _bitmap("k", filter="trilinear", wrap="repeat")},
                     {"k": ("image_default", {"channel": 1}, imgenc.png(img))})
    o = oracle.OracleScene(text, d)
    levels = 1 + int(math.log2(W))
    rng = np.random.default_rng(2)
    uv = rng.uniform(0.2, 0.8, size=(200, 2)).astype(np.float32)
    for k in range(1, levels):
        width = 2.0 ** (k - (levels - 1))
        duv = np.tile(np.array([[width, 0, 0, width]], np.float32), (200, 1))
        v = o.texture_eval(0, uv, duv)[:, 0]
        assert np.allclose(v, 0.5, atol=2e-2), k
    fine = o.texture_eval(0, uv, np.zeros((200, 4), np.float32))[:, 0]
    assert fine.std() > 0.1
    o.close()


def test_chessboard_cells(oracle, tmp_path):
    """chessboard.cpp:36-58: colour_a where the two fractional halves agree."""
    cb = {"type": "chessboard", "to_uv": {"scale": [4, 3, 1], "translate": [0.25, 0, 0]},
          "color_a": [1, 0, 0], "color_b": [0, 0, 1]}
    text, d = _scene(tmp_path, {"base_color": cb}, {})
    o = oracle.OracleScene(text, d)
    rng = np.random.default_rng(3)
    uv = rng.uniform(-1, 2, size=(2000, 2)).astype(np.float32)
    v = o.texture_eval(0, uv)
    t = np.stack([uv[:, 0] * 4 + 0.25, uv[:, 1] * 3], 1).astype(np.float64)
    fr = t - np.floor(t)
    edge = (np.abs(fr - 0.5) < 1e-4).any(1) | (np.minimum(fr, 1 - fr) < 1e-4).any(1)
    want_a = (fr[:, 0] > 0.5) == (fr[:, 1] > 0.5)
    assert np.array_equal(v[~edge, 0] == 1, want_a[~edge])
    o.close()


def test_camera_uv_derivatives_of_a_facing_plane(oracle, tmp_path):
    """For a rectangle facing the camera, du/dx is one pixel's width on the plane over
    the rectangle's size: the renders with trilinear and bilinear filtering agree where
    the footprint is below one texel and the trilinear one blurs where it is larger."""
    W = 64
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, size=(W, W, 3))
    assets = {"n": ("image_default", {"is_to_linear": False}, imgenc.png(img))}

    def render(flt, dist, res=16):
        sc = {"camera": {"type": "perspective", "fov": 30.0, "resolution": [res, res], "origin": [0, 0, dist],
                         "target": [0, 0, 0]},
              "sampler": {"type": "independent", "sample_count": 1, "seed": 1},
              "assets": [{"name": "n", "type": "image_default", "location": "n.img", "is_to_linear": False}],
              "scene": [{"shape": {"type": "rectangle"}, "bsdf": {"type": "diffuse", "reflectance": _bitmap("n", filter=flt)}},
                        {"light": {"type": "point", "position": [0, 0, 50], "intensity": [2500, 2500, 2500]}}],
              "accel": {"type": "embree"}, "renderer": {"type": "path", "max_depth": 2}}
        _, text, d = write(tmp_path, "p_%s_%g" % (flt, dist), sc, {"n.img": assets["n"][2]})
        o = oracle.OracleScene(text, d)
        pix = np.arange(res * res, dtype=np.uint32)
        v = o.render_samples(pix, np.zeros(res * res, np.uint32))
        o.close()
        return v
    # at 0.8 a pixel covers < 1 texel (level < 0: plain bilinear); at 3.6 the
    # rectangle fills the 8-pixel-wide view and a pixel covers ~8 texels (level ~3)
    near_tri, near_bi = render("trilinear", 0.8), render("bilinear", 0.8)
    far_tri, far_bi = render("trilinear", 3.6, 8), render("bilinear", 3.6, 8)
    assert np.allclose(near_tri, near_bi, rtol=1e-6)
    assert far_tri.std() < 0.5 * far_bi.std()


def _sky_plane(tmp_path, name, radiance, assets=None):
    sc = {"camera": {"type": "perspective", "fov": 30.0, "resolution": [8, 8], "origin": [0, 3, 0.01],
                     "target": [0, 0, 0]},
          "sampler": {"type": "independent", "sample_count": 1, "seed": 1},
          "assets": [{"name": "s", "type": "image_hdr", "location": "s.hdr"}] if assets else [],
          "scene": [{"to_world": {"rotate": {"axis": [1, 0, 0], "angle": -90.0}, "scale": [50, 50, 1]},
                     "shape": {"type": "rectangle"}, "bsdf": {"type": "diffuse", "reflectance": 0.5}},
                    {"to_world": {"rotate": {"axis": [0, 1, 0], "angle": 20.0}},
                     "light": {"type": "skybox", "radiance": radiance}}],
          "accel": {"type": "embree"}, "renderer": {"type": "path", "max_depth": 2}}
    _, text, d = write(tmp_path, name, sc, assets)
    return text, d


def test_env_map_sampling(oracle, tmp_path):
    """A bitmap skybox is importance sampled by luminance (skybox.cpp:27-47, 213-233):
    under a uniform map the lit plane's radiance approaches the constant sky's
    R * L (the sampled directions are texel corners, so within a few percent), and
    doubling the map doubles it."""
    import imgenc
    ones = np.ones((32, 64, 3))
    text_c, d_c = _sky_plane(tmp_path, "const", 1.0)
    text_m, d_m = _sky_plane(tmp_path, "map", {"type": "bitmap", "asset_name": "s"}, {"s.hdr": imgenc.hdr(ones)})
    text_2, d_2 = _sky_plane(tmp_path, "map2", {"type": "bitmap", "asset_name": "s"}, {"s.hdr": imgenc.hdr(2 * ones)})
    n = 64
    pix = np.repeat(np.arange(n, dtype=np.uint32), 512)
    smp = np.tile(np.arange(512, dtype=np.uint32), n)
    vals = []
    for text, d in ((text_c, d_c), (text_m, d_m), (text_2, d_2)):
        o = oracle.OracleScene(text, d)
        vals.append(o.render_samples(pix, smp)[:, 0].mean())
        o.close()
    assert abs(vals[0] - 0.5) < 0.01
    assert abs(vals[1] - vals[0]) < 0.05 * vals[0]
    assert abs(vals[2] - 2 * vals[1]) < 1e-3 * vals[2]
