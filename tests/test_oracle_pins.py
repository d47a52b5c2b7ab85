"""Known-answer pins for the CPU oracle (the reference ships no tests or golden
data, so these come from closed forms and from the estimator's own identities)."""
import json
import math

import numpy as np
import pytest

from helpers import BSDFS, bsdf_json, box, directions


def test_fresnel_dielectric_closed_forms(oracle):
    L = oracle.lib()
    out = np.zeros(4, np.float32)
    p = out.ctypes.data_as(__import__("ctypes").c_void_p)
    for eta in (1.33, 1.5, 2.4):
        L.orc_fresnel_dielectric(1.0, eta, p)
        assert abs(out[0] - ((eta - 1) / (eta + 1)) ** 2) < 1e-6      # normal incidence
        L.orc_fresnel_dielectric(0.05, 1.0 / eta, p)
        assert out[0] == 1.0                                            # total internal reflection
    L.orc_fresnel_dielectric(0.3, 1.0, p)
    assert out[0] == 0.0                                                # index matched


def test_fresnel_conductor_normal_incidence(oracle):
    L = oracle.lib()
    eta = np.array([0.2, 0.92, 1.1], np.float32)
    k = np.array([3.9, 2.45, 2.14], np.float32)
    out = np.zeros(3, np.float32)
    vp = lambda a: a.ctypes.data_as(__import__("ctypes").c_void_p)
    L.orc_fresnel_conductor(1.0, vp(eta), vp(k), vp(out))
    expect = ((eta - 1) ** 2 + k ** 2) / ((eta + 1) ** 2 + k ** 2)
    assert np.allclose(out, expect, rtol=1e-5)


@pytest.mark.parametrize("ggx", [1, 0])
@pytest.mark.parametrize("alpha", [(0.1, 0.1), (0.3, 0.3), (0.15, 0.5)])
def test_microfacet_normalisation(oracle, ggx, alpha):
    """Integral of D(m) cos(theta_m) over the hemisphere is 1."""
    L = oracle.lib()
    import ctypes
    n_t, n_p = 2000, 256
    th = (np.arange(n_t) + 0.5) / n_t * (math.pi / 2)
    ph = (np.arange(n_p) + 0.5) / n_p * 2 * math.pi
    total = 0.0
    m = np.zeros(3, np.float32)
    mp = m.ctypes.data_as(ctypes.c_void_p)
    for t in th[::4]:
        row = 0.0
        for p in ph[::4]:
            m[:] = (math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t))
            row += L.orc_microfacet_d(ggx, alpha[0], alpha[1], mp)
        total += row * math.cos(t) * math.sin(t)
    total *= (math.pi / 2 / (n_t / 4)) * (2 * math.pi / (n_p / 4))
    assert abs(total - 1.0) < 0.03


@pytest.mark.parametrize("bsdf", BSDFS, ids=lambda b: b["type"] + "_" + str(abs(hash(bsdf_json(b))) % 1000))
def test_sample_matches_eval_and_pdf(oracle, bsdf):
    """Sample() returns f and pdf consistent with Eval()/Pdf() at the sampled direction
    (for the lobes that have a density: delta lobes and mask pass-through do not)."""
    rng = np.random.default_rng(5)
    n = 4096
    wi = directions(rng, n)
    wi[:, 2] = np.abs(wi[:, 2])
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    js = bsdf_json(bsdf)
    wo, pdf, f, eta, typ = oracle.bsdf_sample(js, wi, u)
    ok = (pdf > 0) & ((typ & (4 | 32)) == 0)
    f2, pdf2 = oracle.bsdf_eval(js, wi[ok], wo[ok])
    assert np.allclose(pdf[ok], pdf2, rtol=2e-3, atol=1e-6)
    assert np.allclose(f[ok], f2, rtol=2e-3, atol=1e-6)


def test_diffuse_white_furnace(oracle):
    """E[f / pdf] of a white Lambertian is 1 for any incident direction."""
    rng = np.random.default_rng(2)
    n = 20000
    wi = np.tile(np.array([[0.3, 0.1, 0.948683]], np.float32), (n, 1))
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    wo, pdf, f, _, _ = oracle.bsdf_sample('{"type":"diffuse","reflectance":1.0}', wi, u)
    w = f[:, 0] / pdf
    assert abs(w.mean() - 1.0) < 1e-5


def test_pdf_integrates_to_at_most_one(oracle):
    rng = np.random.default_rng(3)
    n = 200000
    wo = directions(rng, n)
    for b in BSDFS:
        wi = np.tile(np.array([[0.2, -0.3, 0.932738]], np.float32), (n, 1))
        _, pdf = oracle.bsdf_eval(bsdf_json(b), wi, wo)
        integral = pdf.mean() * 4 * math.pi
        assert integral < 1.05, (b, integral)


def test_pcg_stream_reference_values(oracle):
    """PCG32 (O'Neill) stepping: state' = state * 6364136223846793005 + 1442695040888963407."""
    L = oracle.lib()
    M = 2 ** 64

    def splitmix(z):
        z = (z + 0x9E3779B97F4A7C15) % M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) % M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) % M
        return z ^ (z >> 31)

    def nxt(s):
        old = s
        s = (old * 6364136223846793005 + 1442695040888963407) % M
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return s, ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    for pixel, sample, seed in [(0, 0, 0), (12345, 7, 1), (2 ** 31, 3, 99)]:
        init = splitmix(splitmix(seed) ^ ((pixel << 32) | sample))
        s, _ = nxt(0)
        s = (s + init) % M
        s, _ = nxt(s)
        for k in range(4):
            s, v = nxt(s)
            assert L.orc_pcg_u32(pixel, sample, seed, k) == v


def test_box_room_energy_is_plausible(oracle, scene_dir):
    path, text, d = box(scene_dir, 32, 32, 16)
    o = oracle.OracleScene(text, d)
    film, stats = o.render()
    assert np.isfinite(film).all() and film.min() >= 0
    m = film.mean(axis=(0, 1))
    assert 0.05 < m[0] < 1.0 and m[0] > m[2]  # warm emitter: red dominates blue
    assert stats[2] == 32 * 32 * 16


def _fresnel_dielectric(c, eta):
    """Unpolarised dielectric Fresnel reflectance for light arriving from outside (numpy)."""
    c = np.asarray(c, np.float64)
    st2 = (1 - c * c) / eta ** 2
    ct = np.sqrt(np.maximum(0, 1 - st2))
    rs = (c - eta * ct) / (c + eta * ct)
    rp = (eta * c - ct) / (eta * c + ct)
    r = 0.5 * (rs ** 2 + rp ** 2)
    return np.where(st2 >= 1, 1.0, r)


def test_perfect_mirror_closed_forms(oracle):
    """Mirror direction, unit pdf; f = R * F with F = 1 for the default purely imaginary
    index (eta 0, k 1) and ((n-1)^2+k^2)/((n+1)^2+k^2) at normal incidence."""
    rng = np.random.default_rng(8)
    wi = directions(rng, 512)
    wi[:, 2] = np.abs(wi[:, 2]) + 1e-3
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    u = rng.uniform(size=(512, 3)).astype(np.float32)
    wo, pdf, f, _, typ = oracle.bsdf_sample('{"type":"perfect_mirror","reflectance":[0.9,0.7,0.5]}', wi, u)
    assert np.allclose(wo, wi * np.array([-1, -1, 1], np.float32))
    assert (pdf == 1).all() and (typ == (4 | 8)).all()
    assert np.allclose(f, [0.9, 0.7, 0.5], rtol=1e-5)
    n, k = np.array([0.2, 0.92, 1.1]), np.array([3.9, 2.45, 2.14])
    js = json.dumps({"type": "perfect_mirror", "eta": n.tolist(), "k": k.tolist()})
    _, _, f, _, _ = oracle.bsdf_sample(js, np.array([[0, 0, 1]], np.float32), u[:1])
    assert np.allclose(f[0], ((n - 1) ** 2 + k ** 2) / ((n + 1) ** 2 + k ** 2), rtol=1e-5)
    f, p = oracle.bsdf_eval(js, wi, directions(rng, 512))
    assert (f == 0).all() and (p == 0).all()


def test_perfect_glass_fresnel_and_snell(oracle):
    """Reflection is chosen with probability F (numpy closed form), the refracted
    direction obeys Snell's law, and f / pdf is 1 (reflection) or 1 / eta^2 (refraction)."""
    rng = np.random.default_rng(9)
    n = 4096
    wi = directions(rng, n)
    wi[:, 2] = np.abs(wi[:, 2]) + 1e-3
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    eta = 1.5 / 1.0
    wo, pdf, f, e, typ = oracle.bsdf_sample('{"type":"perfect_glass","int_ior":1.5,"ext_ior":1.0}', wi, u)
    F = _fresnel_dielectric(wi[:, 2], eta)
    refl = (typ & 8) != 0
    assert np.mean(refl == (u[:, 0] <= F)) > 0.999
    assert np.allclose(pdf[refl], F[refl], rtol=1e-4)
    assert np.allclose(pdf[~refl], 1 - F[~refl], rtol=1e-4, atol=1e-6)
    sin_i = np.hypot(wi[~refl, 0], wi[~refl, 1])
    sin_t = np.hypot(wo[~refl, 0], wo[~refl, 1])
    assert np.allclose(sin_t, sin_i / eta, atol=1e-5) and (wo[~refl, 2] < 0).all()
    assert np.allclose(f[refl, 0] / pdf[refl], 1.0, rtol=1e-5)
    assert np.allclose(f[~refl, 0] / pdf[~refl], 1 / eta ** 2, rtol=1e-5)
    assert np.allclose(e[~refl], eta, rtol=1e-6) and (e[refl] == 1).all()


def test_plastic_diffuse_lobe_closed_form(oracle):
    """plastic Eval = R / pi * (1 - F(wi)) (1 - F(wo)) cos(wo) / (eta^2 (1 - Fdr)), with the
    internal diffuse Fresnel reflectance Fdr integrated numerically (the reference's
    polynomial fit agrees within 0.2%)."""
    rng = np.random.default_rng(10)
    wi, wo = directions(rng, 2048), directions(rng, 2048)
    wi[:, 2] = np.abs(wi[:, 2]) + 1e-3
    wo[:, 2] = np.abs(wo[:, 2]) + 1e-3
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    eta = 1.49 / 1.000277
    th = np.linspace(0, np.pi / 2, 200001)
    fdr = np.trapezoid(_fresnel_dielectric(np.cos(th), 1 / eta) * 2 * np.sin(th) * np.cos(th), th)
    R = np.array([0.2, 0.5, 0.8])
    f, pdf = oracle.bsdf_eval(json.dumps({"type": "plastic", "diffuse": R.tolist()}), wi, wo)
    fi, fo = _fresnel_dielectric(wi[:, 2], eta), _fresnel_dielectric(wo[:, 2], eta)
    want = R[None] / np.pi * ((1 - fi) * (1 - fo) * wo[:, 2] / (eta ** 2 * (1 - fdr)))[:, None]
    assert np.allclose(f, want, rtol=2e-3)
    w = 1.0 / (1.0 + (R @ [0.212671, 0.715160, 0.072169]))  # specular share of the mean luminance
    pd = (1 - fi) * (1 - w)
    assert np.allclose(pdf, wo[:, 2] / np.pi * pd / (pd + fi * w), rtol=1e-4)


def test_mask_pass_through(oracle):
    """mask: lobeXi >= opacity passes the ray through (Null, pdf 1 - opacity, f 1); otherwise
    the nested BSDF scaled by the opacity; Eval and Pdf scale by the opacity."""
    rng = np.random.default_rng(12)
    n = 2048
    wi = directions(rng, n)
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    js = '{"type":"mask","opacity":0.35,"nested":{"type":"diffuse","reflectance":0.8}}'
    wo, pdf, f, _, typ = oracle.bsdf_sample(js, wi, u)
    through = u[:, 0] >= np.float32(0.35)
    assert (typ[through] == 32).all() and np.allclose(wo[through], -wi[through])
    assert np.allclose(pdf[through], 0.65) and (f[through] == 1).all()
    wo2 = directions(rng, n)
    f1, p1 = oracle.bsdf_eval(js, wi, wo2)
    f0, p0 = oracle.bsdf_eval('{"type":"diffuse","reflectance":0.8}', wi, wo2)
    assert np.allclose(f1, f0 * np.float32(0.35), rtol=1e-6) and np.allclose(p1, p0 * np.float32(0.35), rtol=1e-6)


def _direct_light_scene(light_entity, res=48):
    """Camera looking straight down at a large Lambertian plane (y = 0, reflectance
    0.5); max_depth 2 keeps only the light sample at the first hit."""
    return {
        "camera": {"type": "perspective", "fov": 60.0, "resolution": [res, res],
                   "origin": [0.0, 6.0, 0.0], "target": [0.0, 0.0, 0.0], "up": [0.0, 0.0, -1.0]},
        "sampler": {"type": "independent", "sample_count": 1, "seed": 4},
        "scene": [{"to_world": {"rotate": {"axis": [1, 0, 0], "angle": -90.0}, "scale": [20, 20, 1]},
                   "shape": {"type": "rectangle"}, "bsdf": {"type": "diffuse", "reflectance": 0.5}},
                  light_entity],
        "accel": {"type": "embree"},
        "renderer": {"type": "path", "max_depth": 2, "rr_depth": 8},
    }


def _plane_hits(o, n):
    r = o.camera_rays(np.arange(n, dtype=np.uint32), 0).astype(np.float64)
    t = -r[:, 1] / r[:, 5]
    return r[:, :3] + t[:, None] * r[:, 4:7]


def test_point_light_direct_closed_form(oracle):
    """A point light of intensity I at height h over a Lambertian plane: the first-hit
    radiance is R / pi * I * cos(theta) / d^2 (inverse-square falloff, point.cpp:33-49)."""
    I = np.array([2.0, 1.0, 0.5])
    sc = _direct_light_scene({"light": {"type": "point", "position": [0.5, 2.0, -0.3], "intensity": I.tolist()}})
    o = oracle.OracleScene(json.dumps(sc), "")
    n = o.width * o.height
    L = o.render_samples(np.arange(n, dtype=np.uint32), np.zeros(n, np.uint32))
    P = _plane_hits(o, n)
    d = np.array([0.5, 2.0, -0.3]) - P
    d2 = (d * d).sum(1)
    want = 0.5 / np.pi * I[None] * (d[:, 1] / np.sqrt(d2) / d2)[:, None]
    assert np.allclose(L, want, rtol=1e-4)
    o.close()


def test_projection_light_footprint(oracle):
    """A projection light at height h aimed straight down lights the square
    |x|, |z| <= h tan(fov / 2) of the plane; inside it the first-hit radiance is the
    constant R * E / h^2 (the cos(theta) / cos(alpha) of projection.cpp:70-72 cancel on a
    plane facing the light), outside it is 0."""
    h, fov = 2.0, 40.0
    E = np.array([3.0, 2.0, 1.0])
    sc = _direct_light_scene({"to_world": {"translate": [0, h, 0], "rotate": {"axis": [1, 0, 0], "angle": 90.0}},
                              "light": {"type": "projection", "fov": fov, "irradiance": E.tolist()}})
    o = oracle.OracleScene(json.dumps(sc), "")
    n = o.width * o.height
    L = o.render_samples(np.arange(n, dtype=np.uint32), np.zeros(n, np.uint32))
    P = _plane_hits(o, n)
    half = h * math.tan(math.radians(fov / 2))
    inside = (np.abs(P[:, 0]) < half * 0.98) & (np.abs(P[:, 2]) < half * 0.98)
    outside = (np.abs(P[:, 0]) > half * 1.02) | (np.abs(P[:, 2]) > half * 1.02)
    assert inside.sum() > 50 and outside.sum() > 50
    assert np.allclose(L[inside], 0.5 * E[None] / h ** 2, rtol=1e-4)
    assert (L[outside] == 0).all()
    o.close()


def test_textured_projection_footprint(oracle, scene_dir):
    """A bitmap irradiance (an 8 x 4 slide, left half E1, right half E2) sets the
    projector's aspect (projection.cpp:23-39): the lit footprint is twice as long
    along one axis as along the other, and inside it the first-hit radiance is
    R * E(uv) * scale / h^2 with E one of the two halves (nearest filter)."""
    import imgenc
    from helpers import write
    h, fov = 2.0, 40.0
    E1, E2 = np.array([200, 40, 40]), np.array([20, 60, 220])
    slide = np.zeros((4, 8, 3), np.int64)
    slide[:, :4], slide[:, 4:] = E1, E2
    sc = _direct_light_scene({"to_world": {"translate": [0, h, 0], "rotate": {"axis": [1, 0, 0], "angle": 90.0}},
                              "light": {"type": "projection", "fov": fov, "scale": [2.0, 2.0, 2.0],
                                        "irradiance": {"type": "bitmap", "asset_name": "slide",
                                                       "filter": "nearest"}}})
    sc["assets"] = [{"name": "slide", "type": "image_default", "location": "slide.png"}]
    _, text, d = write(scene_dir, "proj_slide", sc, {"slide.png": imgenc.png(slide)})
    o = oracle.OracleScene(text, d)
    n = o.width * o.height
    L = o.render_samples(np.arange(n, dtype=np.uint32), np.zeros(n, np.uint32))
    P = _plane_hits(o, n)
    lit = L.sum(axis=1) > 0
    ext = np.abs(P[lit][:, [0, 2]]).max(axis=0)
    assert abs(ext.max() / ext.min() - 2.0) < 0.1, ext
    half = h * math.tan(math.radians(fov / 2))
    assert abs(ext.max() / half - 1.0) < 0.05, (ext, half)
    lin = lambda c: np.where(c / 255.0 <= 0.04045, c / 255.0 / 12.92, ((c / 255.0 + 0.055) / 1.055) ** 2.4)
    want = [0.5 * 2.0 * lin(E) / h ** 2 for E in (E1, E2)]
    near = [np.isclose(L[lit], w[None], rtol=2e-3).all(axis=1) for w in want]
    assert (near[0] | near[1]).all() and near[0].sum() > 20 and near[1].sum() > 20
    o.close()


def test_ao_closed_forms(oracle, scene_dir):
    """ao.cpp:22-36: 1 on an open plane, 1/2 next to a (large) wall — every direction
    towards the wall's side of the hemisphere hits it — and 0 for misses."""
    from helpers import write
    sc = {"camera": {"type": "perspective", "fov": 20.0, "resolution": [16, 16], "origin": [0, 5, 0.01],
                     "target": [0, 0, 0]},
          "sampler": {"type": "independent", "sample_count": 1, "seed": 2},
          "scene": [{"to_world": {"rotate": {"axis": [1, 0, 0], "angle": -90.0}, "scale": [1000, 1000, 1]},
                     "shape": {"type": "rectangle"}}],
          "accel": {"type": "embree"}, "renderer": {"type": "ao"}}
    _, text, d = write(scene_dir, "ao_open", sc)
    o = oracle.OracleScene(text, d)
    n = 256 * 64
    pix = np.repeat(np.arange(256, dtype=np.uint32), 64)
    smp = np.tile(np.arange(64, dtype=np.uint32), 256)
    v = o.render_samples(pix, smp)
    assert np.allclose(v, 1.0, rtol=1e-6)
    o.close()
    sc["scene"].append({"to_world": {"translate": [0, 0, -0.3], "scale": [1000, 1000, 1]}, "shape": {"type": "rectangle"}})
    _, text, d = write(scene_dir, "ao_wall", sc)
    o = oracle.OracleScene(text, d)
    v = o.render_samples(pix, smp)[:, 0]
    assert abs(v.mean() - 0.5) < 0.01, v.mean()
    o.close()


def test_particle_tracer_agrees_with_path_tracer(oracle, scene_dir):
    """particle_tracer (particle_tracer.cpp) and path estimate the same image: on the
    Lambertian box room their film means agree to within the light tracer's noise."""
    from helpers import write
    from radiantiumplusplus_gb300 import scenes
    sc = scenes.box_room(16, 16, 256, max_depth=8)
    _, text, d = write(scene_dir, "pt_path", sc)
    o = oracle.OracleScene(text, d)
    ref, _ = o.render()
    o.close()
    sc["renderer"] = {"type": "particle_tracer", "max_depth": 8}
    sc["sampler"]["sample_count"] = 200000
    _, text, d = write(scene_dir, "pt_particle", sc)
    o = oracle.OracleScene(text, d)
    film = o.render_particle(threads=0)
    o.close()
    m, r = film.reshape(-1, 3).mean(0), ref.reshape(-1, 3).mean(0)
    assert np.all(np.abs(m - r) < 0.04 * r), (m, r)


@pytest.mark.parametrize("room,mis", [("box_room", True), ("box_room", False), ("materials_room", True)])
def test_bdpt_agrees_with_path_tracer(oracle, scene_dir, room, mis):
    """bdpt (bdpt.cpp) and path estimate the same image when every strategy can
    reach every path (area light, unbounded depth): the MIS weights (balance
    heuristic, or uniform with use_mis false) sum to one over the strategies, so
    the film means agree to within the noise. materials_room adds delta (mirror,
    glass, plastic) and layered lobes and the importance-transport BSDF calls."""
    from helpers import write
    from radiantiumplusplus_gb300 import scenes
    w = 16 if room == "box_room" else 24
    sc = getattr(scenes, room)(w, w, 4096, max_depth=-1)
    _, text, d = write(scene_dir, "bd_path_" + room, sc)
    o = oracle.OracleScene(text, d)
    ref, _ = o.render()
    o.close()
    sc["renderer"] = {"type": "bdpt", "use_mis": mis}
    sc["sampler"]["sample_count"] = 2048 if room == "box_room" else 1024
    _, text, d = write(scene_dir, "bd_bdpt_" + room, sc)
    o = oracle.OracleScene(text, d)
    film = o.render_bdpt()
    o.close()
    m, r = film.reshape(-1, 3).mean(0), ref.reshape(-1, 3).mean(0)
    assert np.all(np.abs(m - r) < 0.03 * r), (m, r)


def test_bdpt_rejects_directional_light(oracle):
    """The directional light is an extension with no SampleLe; bdpt scenes with one
    are refused when loaded."""
    from radiantiumplusplus_gb300 import scenes
    sc = scenes.box_room(8, 8, 1)
    sc["scene"].append({"light": {"type": "directional", "direction": [0, -1, 0], "irradiance": [1, 1, 1]}})
    sc["renderer"] = {"type": "bdpt"}
    with pytest.raises(RuntimeError, match="directional"):
        oracle.OracleScene(json.dumps(sc), "")


def test_textured_area_light_seen_directly(oracle, scene_dir):
    """area.cpp:42-45 with a bitmap: a camera facing the emitter sees its texels
    (nearest filter: texel floor(u (w - 1)), bitmap.cpp:181-191), laid out by the
    rectangle's uv (rectangle.cpp:202-217); an emitter shape other than a
    rectangle is refused (only the rectangle has EvalParamSurface,
    shape.cpp:27-29)."""
    import imgenc
    from helpers import write
    texels = np.full((3, 3, 3), 0.5)
    texels[:2, :2] = [[[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]], [[0.0, 0.0, 3.0], [4.0, 4.0, 4.0]]]
    sc = {"camera": {"type": "perspective", "fov": 10.0, "resolution": [16, 16], "origin": [0, 0, 5],
                     "target": [0, 0, 0]},
          "sampler": {"type": "independent", "sample_count": 1, "seed": 2},
          "assets": [{"name": "q", "type": "image_hdr", "location": "q.hdr"}],
          "scene": [{"to_world": {"scale": [2, 2, 1]}, "shape": {"type": "rectangle"},
                     "light": {"type": "area", "radiance": {"type": "bitmap", "asset_name": "q",
                                                            "filter": "nearest"}}}],
          "accel": {"type": "embree"}, "renderer": {"type": "path", "max_depth": 1}}
    hdr = imgenc.hdr(texels, rle=False)  # scanlines narrower than 8 are stored flat
    _, text, d = write(scene_dir, "tex_light_direct", sc, {"q.hdr": hdr})
    o = oracle.OracleScene(text, d)
    film, _ = o.render()
    o.close()
    q = imgenc.rgbe(texels)
    dec = q[..., :3] * np.ldexp(1.0, q[..., 3:4].astype(int) - 136)  # the RGBE values the decoder returns
    corners = film[[1, 1, 14, 14], [1, 14, 1, 14]]
    got = {tuple(np.round(c, 3)) for c in corners}
    want = {tuple(np.round(c, 3)) for c in dec[:2, :2].reshape(-1, 3)}
    assert got == want, (got, want)
    sc["scene"][0]["shape"] = {"type": "sphere", "radius": 1.0}
    sc["scene"][0]["to_world"] = {"translate": [0, 0, 0]}
    _, text, d = write(scene_dir, "tex_light_sphere", sc, {"q.hdr": hdr})
    with pytest.raises(RuntimeError, match="EvalParamSurface"):
        oracle.OracleScene(text, d)


@pytest.mark.parametrize("shape", ["rect", "cube"])
def test_chessboard_area_light_is_linear_in_its_colours(oracle, scene_dir, shape):
    """A chessboard radiance leaves the light's sampling untouched (uniform shape
    samples, area.cpp:55-58), so the renders with colours (a, b) and (b, a) add up,
    pixel by pixel, to the render of the constant a + b with the same seed (the
    cube room's ceiling light is kept at radiance 0, so it is counted once)."""
    from helpers import chessboard_light_room, write
    a, b = (30.0, 14.0, 3.0), (3.0, 6.0, 24.0)
    films = []
    for i, (ca, cb) in enumerate([(a, b), (b, a)]):
        sc, _ = chessboard_light_room(16, 16, 16, shape=shape, a=ca, b=cb, ceiling=(0, 0, 0))
        _, text, d = write(scene_dir, "chess_lin_%s_%d" % (shape, i), sc)
        o = oracle.OracleScene(text, d)
        films.append(o.render()[0])
        o.close()
    sc, _ = chessboard_light_room(16, 16, 16, shape=shape, ceiling=(0, 0, 0))
    emitter = sc["scene"][-1]["light"]
    emitter["radiance"] = [x + y for x, y in zip(a, b)]
    _, text, d = write(scene_dir, "chess_lin_%s_c" % shape, sc)
    o = oracle.OracleScene(text, d)
    ref, _ = o.render()
    o.close()
    assert np.allclose(films[0] + films[1], ref, rtol=1e-4, atol=1e-6)
    assert not np.allclose(films[0], films[1], rtol=0.05)  # the two colourings light the room differently


def test_chessboard_area_light_seen_directly(oracle, scene_dir):
    """A camera facing a chessboard emitter sees colour_a where the fractional
    parts of the to_uv-mapped uv fall on the same side of 1/2, colour_b elsewhere
    (chessboard.cpp:35-56). The particle tracer's emitter-point splats, which
    read the texture at position samples' uvs (rectangle.cpp:221-230), draw the
    same pattern as the path tracer's hits (rectangle.cpp:202-217). A sphere
    emitter is refused: its samples carry no uv (sphere.cpp:250-320)."""
    from helpers import write
    red, blue = [4.0, 0.0, 0.0], [0.0, 0.0, 4.0]
    sc = {"camera": {"type": "perspective", "fov": 10.0, "resolution": [16, 16], "origin": [0, 0, 5],
                     "target": [0, 0, 0]},
          "sampler": {"type": "independent", "sample_count": 1, "seed": 2},
          "scene": [{"to_world": {"scale": [2, 2, 1]}, "shape": {"type": "rectangle"},
                     "light": {"type": "area", "radiance": {"type": "chessboard", "color_a": red,
                                                            "color_b": blue,
                                                            "to_uv": {"scale": [2, 2, 1]}}}}],
          "accel": {"type": "embree"}, "renderer": {"type": "path", "max_depth": 1}}
    _, text, d = write(scene_dir, "chess_light_direct", sc)
    o = oracle.OracleScene(text, d)
    film, _ = o.render()
    o.close()
    diag = {tuple(film[i, j]) for i, j in [(1, 1), (14, 14)]}
    anti = {tuple(film[i, j]) for i, j in [(1, 14), (14, 1)]}  # the view spans tuv 0.78..1.22 on both axes
    assert len(diag) == 1 and len(anti) == 1 and diag | anti == {tuple(red), tuple(blue)}, (diag, anti)
    assert {tuple(c) for c in film.reshape(-1, 3)} == {tuple(red), tuple(blue)}
    sc["renderer"] = {"type": "particle_tracer", "max_depth": 1}
    sc["sampler"]["sample_count"] = 40000
    _, text, d = write(scene_dir, "chess_light_particle", sc)
    o = oracle.OracleScene(text, d)
    pt = o.render_particle(threads=0)
    o.close()
    redder = film[..., 0] > film[..., 2]
    inner = np.zeros_like(redder)
    inner[1:-1, 1:-1] = True  # pixels away from the emitter's edge
    agree = (pt[..., 0] > pt[..., 2]) == redder
    assert agree[inner].mean() >= 0.9, agree[inner].mean()
    sc["scene"][0]["shape"] = {"type": "sphere", "radius": 1.0}
    sc["scene"][0]["to_world"] = {"translate": [0, 0, 0]}
    _, text, d = write(scene_dir, "chess_light_sphere", sc)
    with pytest.raises(RuntimeError, match="sphere"):
        oracle.OracleScene(text, d)
