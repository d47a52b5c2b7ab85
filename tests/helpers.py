"""Shared test helpers: seeded scenes written to disk, direction batches."""
import json
import os

import numpy as np

from radiantiumplusplus_gb300 import scenes


def write(dirpath, name, scene, assets=None):
    d = os.path.join(str(dirpath), name)
    path = scenes.write_scene(d, scene, assets)
    with open(path) as fh:
        return path, fh.read(), d


def box(dirpath, w=64, h=64, spp=4, seed=1):
    return write(dirpath, "box_%dx%d_%d_%d" % (w, h, spp, seed), scenes.box_room(w, h, spp, seed))


def spheres(dirpath, n=300, emitters=5, w=96, h=64, spp=4):
    sc, assets = scenes.many_spheres(n_spheres=n, n_emitters=emitters, width=w, height=h, spp=spp)
    return write(dirpath, "spheres_%d_%dx%d" % (n, w, h), sc, assets)


def materials(dirpath, w=48, h=48, spp=4, seed=1):
    return write(dirpath, "materials_%dx%d_%d_%d" % (w, h, spp, seed), scenes.materials_room(w, h, spp, seed))


def lights(dirpath, w=48, h=48, spp=4, seed=1):
    return write(dirpath, "lights_%dx%d_%d_%d" % (w, h, spp, seed), scenes.lights_room(w, h, spp, seed))


def _jpeg_rgb(rgb, scans=None, restart=0, sampling=((2, 2), (1, 1), (1, 1))):
    """An RGB image as a JFIF YCbCr JPEG (imgenc.jpeg) with a mild quantiser."""
    import imgenc
    r, g, b = (rgb[..., k].astype(np.float64) for k in range(3))
    planes = [0.299 * r + 0.587 * g + 0.114 * b, -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
              0.5 * r - 0.418688 * g - 0.081312 * b + 128]
    q = [np.full(64, 3), np.full(64, 5), np.full(64, 5)]
    h, w = rgb.shape[:2]
    return imgenc.jpeg(planes, list(sampling), q, w, h, scans=scans, restart=restart)[0]


def textured_room_scene(w=48, h=48, spp=4, seed=1, renderer="path", jpeg=False):
    """Box room whose materials read textures of every kind: bitmaps from PNG
    (RGB and mono), Radiance HDR and OpenEXR assets with nearest / bilinear /
    trilinear / anisotropic filters and clamp / repeat wrapping, nested
    chessboards, a textured mask opacity and textured microfacet roughness.
    jpeg: the two PNG textures become JPEG files (a progressive 4:2:0 colour
    image, a sequential grey one with restart markers). Returns (scene dict,
    {file name: bytes})."""
    import imgenc
    rng = np.random.default_rng(11)
    yy, xx = np.mgrid[0:64, 0:64]
    tiles = ((xx // 8 + yy // 8) % 2)[..., None] * np.array([180, 60, 40]) + rng.integers(0, 60, (64, 64, 3))
    grain = (96 + 80 * np.sin(xx / 5.0) * np.cos(yy / 7.0))[..., None].astype(np.int64)
    hdr_img = np.stack([0.2 + 0.6 * xx / 63, 0.3 + 0.0 * yy, 0.8 - 0.5 * yy / 63], axis=2)[:32, :48]
    exr_img = {k: (0.3 + 0.6 * rng.random((16, 16))).astype(np.float16) for k in "RGB"}
    assets = {"tiles.png": imgenc.png(tiles.clip(0, 255)), "grain.png": imgenc.png(grain.clip(0, 255)),
              "sky.hdr": imgenc.hdr(hdr_img), "metal.exr": imgenc.exr(exr_img, 3)}
    if jpeg:
        prog = [((1, 2, 3), 0, 0, 0, 1), ((1,), 1, 5, 0, 2), ((1,), 6, 63, 0, 2), ((2,), 1, 63, 0, 1),
                ((3,), 1, 63, 0, 1), ((1,), 1, 63, 2, 1), ((1, 2, 3), 0, 0, 1, 0), ((1,), 1, 63, 1, 0),
                ((2,), 1, 63, 1, 0), ((3,), 1, 63, 1, 0)]
        assets["tiles.png"] = _jpeg_rgb(tiles.clip(0, 255), scans=prog)
        assets["grain.png"] = imgenc.jpeg([grain[..., 0].clip(0, 255)], [(1, 1)], [np.full(64, 2)], 64, 64,
                                          restart=5)[0]
    sc = scenes.box_room(w, h, spp, seed)
    if renderer == "vol_path":
        sc["renderer"] = {"type": "vol_path", "max_depth": 8, "rr_depth": 3}
    sc["assets"] = [
        {"name": "tiles", "type": "image_default", "location": "tiles.png"},
        {"name": "grain", "type": "image_default", "location": "grain.png", "channel": 1},
        {"name": "sky", "type": "image_hdr", "location": "sky.hdr", "is_flip_y": True},
        {"name": "metal", "type": "image_exr", "location": "metal.exr"},
    ]
    e = sc["scene"]
    e[0]["bsdf"] = {"type": "diffuse", "reflectance": {"type": "bitmap", "asset_name": "tiles", "filter": "trilinear",
                                                       "wrap": "repeat"}}
    e[0]["to_world"]["scale"] = [1.0, 1.0, 1.0]
    e[2]["bsdf"] = {"type": "rough_plastic", "alpha": 0.2, "diffuse": {
        "type": "chessboard", "to_uv": {"scale": [6, 6, 1]}, "remap": True,
        "color_a": {"type": "bitmap", "asset_name": "tiles", "filter": "anisotropic", "anisotropic_level": 4},
        "color_b": {"type": "chessboard", "color_a": [0.1, 0.5, 0.2], "color_b": 0.7, "to_uv": {"scale": [3, 3, 1]}}}}
    e[3]["bsdf"] = {"type": "plastic", "diffuse": [0.6, 0.1, 0.1],
                    "specular": {"type": "bitmap", "asset_name": "sky", "filter": "bilinear"}}
    e[5]["bsdf"] = {"type": "disney", "base_color": {"type": "bitmap", "asset_name": "tiles", "filter": "nearest"},
                    "roughness": {"type": "bitmap", "asset_name": "grain", "wrap": "repeat"}, "metallic": 0.3}
    e[6]["bsdf"] = {"type": "mask", "opacity": {"type": "chessboard", "color_a": 0.9, "color_b": 0.2,
                                                "to_uv": {"scale": [4, 2, 1]}},
                    "nested": {"type": "diffuse", "reflectance": 0.8}}
    e.append({"shape": {"type": "sphere", "center": [0.45, 0.85, 0.35], "radius": 0.25},
              "bsdf": {"type": "rough_metal", "reflectance": {"type": "bitmap", "asset_name": "metal"},
                       "alpha": {"type": "bitmap", "asset_name": "grain", "filter": "trilinear"}}})
    # environment map seen through the open front of the room: importance-sampled HDR sky
    e.append({"to_world": {"rotate": {"axis": [0, 1, 0], "angle": 30.0}},
              "light": {"type": "skybox", "radiance": {"type": "bitmap", "asset_name": "sky"}}})
    return sc, assets


def textured_light_room(w=48, h=48, spp=4, seed=1, renderer="path"):
    """Box room lit by its ceiling rectangle with a bitmap radiance (an 8 x 6
    Radiance HDR pattern with a black row): the light's luminance distribution
    drives its position samples (area.cpp:93-115). Returns (scene dict, assets)."""
    import imgenc
    yy, xx = np.mgrid[0:6, 0:8]
    img = np.stack([4.0 + 20.0 * xx / 7, 2.0 + 14.0 * yy / 5, 8.0 * ((xx + yy) % 2) + 1.0], axis=2)
    img[2] = 0.0
    sc = scenes.box_room(w, h, spp, seed)
    sc["assets"] = [{"name": "glow", "type": "image_hdr", "location": "glow.hdr"}]
    sc["scene"][-1]["light"] = {"type": "area", "radiance": {"type": "bitmap", "asset_name": "glow",
                                                               "filter": "nearest"}}
    if renderer != "path":
        sc["renderer"] = {"type": renderer, "max_depth": 6}
    return sc, {"glow.hdr": imgenc.hdr(img)}


def chessboard_light_room(w=48, h=48, spp=4, seed=1, renderer="path", shape="rect", a=(30.0, 14.0, 3.0),
                          b=(3.0, 6.0, 24.0), ceiling=(1.0, 0.8, 0.3)):
    """Box room lit by an emitter whose radiance is a chessboard (a 1 x 1 texture to
    the light, chessboard.cpp:30-31): the shape is sampled uniformly and the texture
    read at each sample's uv (area.cpp:45-58). shape "rect": the ceiling rectangle;
    "cube": a small cube hanging below the ceiling (a mesh with per-face uvs; its
    samples carry interpolated uvs; the ceiling rectangle keeps a constant
    radiance `ceiling`). Returns (scene dict, assets)."""
    sc = scenes.box_room(w, h, spp, seed)
    chess = {"type": "chessboard", "color_a": list(a), "color_b": list(b),
             "to_uv": {"scale": [3.0, 2.0, 1.0]}}
    if shape == "rect":
        sc["scene"][-1]["light"] = {"type": "area", "radiance": chess}
    else:
        sc["scene"][-1]["light"]["radiance"] = list(ceiling)
        sc["scene"].append({"to_world": {"translate": [0.1, 1.55, 0.2], "rotate": {"axis": [1, 1, 0], "angle": 30.0},
                                         "scale": [0.18, 0.18, 0.18]},
                            "shape": {"type": "cube"}, "light": {"type": "area", "radiance": chess}})
    if renderer != "path":
        sc["renderer"] = {"type": renderer, "max_depth": 6}
    return sc, {}


def textured_projection_room(w=48, h=48, spp=4, seed=1, renderer="path"):
    """Box room with a dimmed area light and a projection light whose irradiance
    is a 16 x 12 PNG slide (aspect 4:3 sets the projector's frustum,
    projection.cpp:23-39). Returns (scene dict, assets)."""
    import imgenc
    yy, xx = np.mgrid[0:12, 0:16]
    img = np.stack([40 + 200 * (xx // 4 % 2), 60 + 15 * yy, 220 - 12 * xx], axis=2)
    sc = scenes.box_room(w, h, spp, seed)
    sc["assets"] = [{"name": "slide", "type": "image_default", "location": "slide.png"}]
    sc["scene"][-1]["light"]["radiance"] = [2.0, 1.5, 0.5]
    sc["scene"].append({"to_world": {"translate": [0.2, 1.3, 2.2], "rotate": {"axis": [0, 1, 0], "angle": 180.0}},
                        "light": {"type": "projection", "fov": 35.0, "scale": [1.5, 1.2, 1.0],
                                  "irradiance": {"type": "bitmap", "asset_name": "slide", "filter": "bilinear"}}})
    if renderer != "path":
        sc["renderer"] = {"type": renderer, "max_depth": 6}
    return sc, {"slide.png": imgenc.png(img.clip(0, 255))}


def textured(dirpath, w=48, h=48, spp=4, seed=1, renderer="path", jpeg=False):
    sc, assets = textured_room_scene(w, h, spp, seed, renderer, jpeg)
    return write(dirpath, "textured_%s_%dx%d_%d_%d%s" % (renderer, w, h, spp, seed, "_jpeg" if jpeg else ""), sc,
                 assets)


def volume(dirpath, w=48, h=48, spp=4, grid=32, max_depth=32):
    sc, assets = scenes.volume_box(width=w, height=h, spp=spp, grid=grid, max_depth=max_depth)
    return write(dirpath, "vol_%dx%d_%d" % (w, h, grid), sc, assets)


def volume_variant(dirpath, variant, w=32, h=32):
    """The fBm volume box (24^3 grid) with its cube made an index-matched boundary
    (no BSDF), or with a glass sphere of homogeneous medium beside it."""
    sc, assets = scenes.volume_box(width=w, height=h, spp=1, grid=24)
    cube = sc["scene"][0]
    if variant == "index_matched":
        del cube["bsdf"]
    elif variant == "homogeneous_sphere":
        sc["scene"].append({"to_world": {"translate": [1.6, 0.8, 0.6], "scale": [0.6, 0.6, 0.6]},
                            "shape": {"type": "sphere"},
                            "bsdf": {"type": "rough_glass", "int_ior": 1.4, "ext_ior": 1.0, "alpha": 0.1},
                            "in_medium": {"type": "homogeneous", "sigma_t": [1.5, 2.0, 2.5], "albedo": 0.8,
                                          "scale": 1.0, "phase": {"type": "isotropic_phase"}}})
    else:
        raise ValueError(variant)
    return write(dirpath, "vol_" + variant, sc, assets)


def directions(rng, n):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d.astype(np.float32)


BSDFS = [
    {"type": "diffuse", "reflectance": [0.3, 0.6, 0.9]},
    {"type": "rough_metal", "alpha": 0.2},
    {"type": "rough_metal", "alpha_u": 0.08, "alpha_v": 0.4},
    {"type": "rough_metal", "alpha": 0.3, "distribution": "beckmann"},
    {"type": "rough_metal", "alpha": 0.25, "sample_visible": False},
    {"type": "rough_glass", "int_ior": 1.5, "ext_ior": 1.0, "alpha": 0.15},
    {"type": "rough_glass", "int_ior": 1.33, "ext_ior": 1.0, "alpha": 0.05},
    {"type": "disney", "base_color": [0.8, 0.3, 0.2], "roughness": 0.4, "metallic": 0.3, "spec_trans": 0.4,
     "clearcoat": 0.7, "clearcoat_gloss": 0.5, "sheen": 0.6, "sheen_tint": 0.3, "spec_tint": 0.5,
     "flatness": 0.3, "anisotropic": 0.4},
    {"type": "disney", "base_color": [0.5, 0.5, 0.5], "roughness": 0.7},
    {"type": "disney", "base_color": [0.9, 0.8, 0.1], "roughness": 0.2, "metallic": 1.0, "specular": 0.8},
    {"type": "two_side", "two_side": {"type": "rough_metal", "alpha": 0.3}},
    {"type": "perfect_mirror"},
    {"type": "perfect_mirror", "reflectance": [0.9, 0.7, 0.5], "eta": [0.2, 0.92, 1.1], "k": [3.9, 2.45, 2.14]},
    {"type": "perfect_glass"},
    {"type": "perfect_glass", "int_ior": 1.33, "ext_ior": 1.0, "reflectance": [0.9, 0.8, 0.7],
     "transmittance": [0.6, 0.8, 1.0]},
    {"type": "plastic", "diffuse": [0.2, 0.5, 0.8]},
    {"type": "plastic", "diffuse": [0.6, 0.3, 0.1], "specular": 0.5, "no_linear": True, "int_ior": 1.6},
    {"type": "rough_plastic", "diffuse": [0.2, 0.5, 0.8], "alpha": 0.2},
    {"type": "rough_plastic", "alpha": 0.3, "distribution": "beckmann", "no_linear": True},
    {"type": "rough_plastic", "alpha": 0.15, "sample_visible": False},
    {"type": "mask", "opacity": 0.4, "nested": {"type": "rough_metal", "alpha": 0.2}},
    {"type": "mask", "opacity": 0.7, "nested": {"type": "two_side", "two_side": {"type": "plastic"}}},
    {"type": "two_side", "out_side": {"type": "mask", "opacity": 0.5, "nested": {"type": "diffuse"}},
     "in_side": {"type": "perfect_glass"}},
]


def bsdf_json(b):
    return json.dumps(b)


def close_to(a, b):
    """Per-sample agreement used by the integrator parity tests: every channel
    within 1e-3 relative (absolute floor 1e-4)."""
    return (np.abs(a - b) <= 1e-3 * np.maximum(np.abs(b), 1e-1)).all(axis=1)


def ulp_sensitive(o, pix, smp, lo, seeds=32, max_calls=50000):
    """Which of these samples change (beyond close_to) when the harness
    (tests/hostemu: the device code on the host, bit-identical to the oracle)
    moves transcendental results by one or two ulps. The GPU's math library
    and the oracle's libm differ only in such last-ulp rounding, so a GPU
    sample that differs from the oracle's must be one of these. First `seeds`
    random nudge streams over the whole batch; then, for each sample not yet
    shown to flip, rendered alone, every one of its transcendental calls in
    turn moved by -2, -1, +1 and +2 ulps."""
    import hemu_lib
    h = hemu_lib.HemuScene(o.json_text, o.base_dir)
    sens = np.zeros(len(pix), bool)
    try:
        exact = h.render_samples(pix, smp, o.seed)
        assert ((exact.view(np.uint32) == lo.view(np.uint32)) | (np.isnan(exact) & np.isnan(lo))).all()
        for k in range(1, seeds + 1):
            hemu_lib.set_nudge(k * 7919)
            sens |= ~close_to(h.render_samples(pix, smp, o.seed), lo)
        hemu_lib.set_nudge(0)
        for i in np.where(~sens)[0]:
            p1, s1 = pix[i:i + 1], smp[i:i + 1]
            h.render_samples(p1, s1, o.seed)
            calls = min(int(hemu_lib.last_calls()), max_calls)
            for c in range(calls):
                for u in (-2, -1, 1, 2):
                    hemu_lib.set_nudge_target(c, u)
                    if not close_to(h.render_samples(p1, s1, o.seed), lo[i:i + 1])[0]:
                        sens[i] = True
                        break
                if sens[i]:
                    break
            hemu_lib.set_nudge_target(-1, 0)
    finally:
        hemu_lib.set_nudge(0)
        hemu_lib.set_nudge_target(-1, 0)
        h.close()
    return sens


def sample_parity(g, o, spp, min_frac, explain=True):
    """Every pixel's first `spp` samples through the GPU kernels and the oracle
    on identical PCG streams. At least `min_frac` agree (close_to), the sample
    means agree within 2%, and (explain) every sample that disagrees is one
    whose result flips under one- or two-ulp nudges of the transcendentals. Returns
    (fraction agreeing, GPU samples, oracle samples)."""
    W, H = g.width, g.height
    pix = np.repeat(np.arange(W * H, dtype=np.uint32), spp)
    smp = np.tile(np.arange(spp, dtype=np.uint32), W * H)
    return sample_parity_at(g, o, pix, smp, min_frac, explain)


def sample_parity_at(g, o, pix, smp, min_frac, explain=True):
    """sample_parity over given (pixel, sample) pairs."""
    lg = g.render_samples(pix, smp)
    lo = o.render_samples(pix, smp)
    close = close_to(lg, lo)
    frac = close.mean()
    mg, mo = lg.mean(0), lo.mean(0)
    assert frac >= min_frac, "only %.4f of samples agree" % frac
    assert np.all(np.abs(mg - mo) <= 0.02 * np.abs(mo) + 1e-6), (mg, mo)
    if explain and not close.all():
        bad = np.where(~close)[0]
        sens = ulp_sensitive(o, pix[bad], smp[bad], lo[bad])
        assert sens.all(), "%d of %d differing samples do not depend on last-ulp rounding: %s" % (
            (~sens).sum(), len(bad), [(int(pix[i]), int(smp[i])) for i in bad[~sens][:5]])
    return frac, lg, lo


def _disney(rng):
    b = {"type": "disney"}
    if rng.uniform() < 0.8:
        b["base_color"] = rng.uniform(0, 1, 3).round(6).tolist()
    for k in ("metallic", "roughness", "specular", "spec_tint", "spec_trans", "anisotropic", "sheen", "sheen_tint",
              "clearcoat", "clearcoat_gloss", "flatness"):
        r = rng.uniform()
        if r < 0.5:
            b[k] = float(np.float32(rng.uniform()))
        elif r < 0.6:
            b[k] = 0.0  # present but zero: the reference's "present" flags need nonzero
    return b


def bsdf_sweep(n_disney, seed=11):
    """Seeded parameter sets over the many-spheres materials' ranges."""
    rng = np.random.default_rng(seed)
    out = [dict(b) for b in BSDFS]
    out += [_disney(rng) for _ in range(n_disney)]
    for a in [0.0, 1e-4, 1e-3] + list(rng.uniform(0, 0.3, 40)):
        out.append({"type": "rough_glass", "int_ior": 1.5, "ext_ior": 1.0, "alpha": float(np.float32(a))})
    out.append({"type": "rough_glass", "int_ior": 1.33, "ext_ior": 1.0, "alpha": 0.0})
    for _ in range(60):
        b = {"type": "rough_metal", "distribution": "ggx" if rng.uniform() < 0.7 else "beckmann",
             "sample_visible": bool(rng.uniform() < 0.8)}
        if rng.uniform() < 0.3:
            b["alpha_u"] = float(np.float32(rng.uniform(0.05, 0.5)))
            b["alpha_v"] = float(np.float32(rng.uniform(0.05, 0.5)))
        else:
            b["alpha"] = float(np.float32(rng.uniform(0.05, 0.5)))
        out.append(b)
    for _ in range(20):
        out.append({"type": "diffuse", "reflectance": rng.uniform(0.1, 0.9, 3).round(6).tolist()})
    return out
