"""Integrator parity: the wavefront `path` kernels and the `vol_path` kernel vs
the CPU oracle, sample by sample on identical PCG streams, plus film-level
checks (job film, z-test of the mean against a high-spp oracle reference).

Per-sample tolerance: every channel within 1e-3 relative (absolute floor
1e-4). The device code compiled for the host equals the oracle bit for bit
(tests/test_hostemu_parity.py); on the GPU only CUDA's sinf/cosf/logf/expf/
powf/... round differently from glibc's in the last ulp, and a path can take
the other branch of a roulette or lobe decision that sits on such a boundary.
Required: >= 99.5% of `path` samples (>= 99% for `vol_path`, whose free
flights and transmittance take many logf/expf per path) agree, and every
sample that does not is shown to flip under one- or two-ulp nudges of the
transcendentals in the host harness. bdpt (not emulated by the harness) keeps
a fraction bound only.
"""

import os

import numpy as np
import pytest

from helpers import box, lights, materials, sample_parity, spheres, volume, volume_variant, write
from radiantiumplusplus_gb300 import scenes

pytestmark = pytest.mark.gpu


def _sample_parity(g, o, spp, min_frac, explain=True):
    return sample_parity(g, o, spp, min_frac, explain)


def test_path_samples_box(rad, oracle, scene_dir):
    path, text, d = box(scene_dir, 48, 48, 4)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    frac, _, _ = _sample_parity(g, o, 4, 0.995)
    g.close()


def test_path_samples_materials(rad, oracle, scene_dir):
    """Delta BSDFs (mirror, glass, plastic's specular lobe), mask pass-through and
    two-sided layered materials in one room."""
    path, text, d = materials(scene_dir, 48, 48, 4)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 4, 0.995)
    g.close()


def test_path_samples_spheres(rad, oracle, scene_dir):
    path, text, d = spheres(scene_dir, 400, 6, 64, 48)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 2, 0.995)
    g.close()


def test_volpath_samples(rad, oracle, scene_dir):
    path, text, d = volume(scene_dir, 32, 32, 2, grid=24)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 2, 0.99)
    g.close()


@pytest.mark.parametrize("variant", ["index_matched", "homogeneous_sphere"])
def test_volpath_media_variants(rad, oracle, scene_dir, variant):
    """vol_path through an index-matched boundary and through a homogeneous
    medium in a glass sphere: samples against the oracle, and the wavefront's
    film equals the persistent kernel's."""
    path, text, d = volume_variant(scene_dir, variant)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 2, 0.99)
    films = []
    for persistent in (False, True):
        j = g.submit(spp=4, seed=9, vol_persistent=persistent)
        j.wait()
        films.append(j.film())
        j.close()
    assert np.array_equal(films[0], films[1]) and films[0].mean() > 0
    g.close()


def test_ao_samples(rad, oracle, scene_dir):
    """Renderer `ao` (ao.cpp): the first hit and one cosine-sampled visibility ray."""
    sc = scenes.box_room(48, 48, 4)
    sc["renderer"] = {"type": "ao"}
    path, text, d = write(scene_dir, "ao_box", sc)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 4, 0.995)
    film = g.render()
    ref, _ = o.render()
    assert abs(film.mean() - ref.mean()) < 1e-3 * ref.mean()
    g.close()


@pytest.mark.parametrize("light", ["area", "sky", "point"])
def test_particle_tracer_film(rad, oracle, scene_dir, light):
    """Renderer `particle_tracer`: the job's film (light paths splatted with atomics)
    against the oracle's film of the same light paths. Splat order differs, and a
    path can take the other branch on a 1-ulp transcendental difference, so the
    check is per pixel within 2% for >= 90% of lit pixels and the film mean
    within 1%."""
    sc = scenes.materials_room(24, 24, 1)
    if light == "sky":
        sc["scene"].append({"light": {"type": "skybox", "radiance": [0.4, 0.5, 0.6]}})
    elif light == "point":
        sc["scene"].append({"light": {"type": "point", "position": [0.2, 1.5, 0.3], "intensity": [2, 2, 2]}})
    sc["renderer"] = {"type": "particle_tracer", "max_depth": 6}
    sc["sampler"]["sample_count"] = 60000
    path, text, d = write(scene_dir, "particle_" + light, sc)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    film = g.render()
    ref = o.render_particle()
    lit = ref.sum(axis=2) > 1e-3
    close = (np.abs(film - ref) <= 0.02 * np.abs(ref) + 1e-6).all(axis=2)
    assert close[lit].mean() >= 0.9, close[lit].mean()
    assert abs(film.mean() - ref.mean()) < 0.01 * ref.mean()
    with pytest.raises(rad.RadError):
        g.render_samples(np.zeros(1, np.uint32), np.zeros(1, np.uint32))
    g.close()


@pytest.mark.parametrize("light", ["area", "sky", "point", "projection", "textured", "nomis"])
def test_bdpt_samples_and_film(rad, oracle, scene_dir, light):
    """Renderer `bdpt` (bdpt.cpp): each pixel sample's camera-side radiance (the
    MIS-weighted t >= 2 connections) through rad_render_samples against the oracle
    on identical streams; then the job film (camera side plus the t = 1 splats,
    added with atomics) against the oracle's film: mean within 2%, and most lit
    pixels within 5% (a sample can take the other branch on a 1-ulp
    transcendental difference, and splat order differs)."""
    from helpers import textured_room_scene
    assets = None
    if light == "textured":
        sc, assets = textured_room_scene(24, 24, 16)
    else:
        sc = scenes.materials_room(24, 24, 16)
    if light == "sky":
        sc["scene"].append({"light": {"type": "skybox", "radiance": [0.4, 0.5, 0.6]}})
    elif light == "point":
        sc["scene"].append({"light": {"type": "point", "position": [0.2, 1.5, 0.3], "intensity": [2, 2, 2]}})
    elif light == "projection":
        sc["scene"].append({"to_world": {"translate": [0.2, 1.3, 2.2], "rotate": {"axis": [0, 1, 0], "angle": 180.0}},
                            "light": {"type": "projection", "fov": 28.0, "irradiance": [2.0, 1.6, 1.2],
                                      "scale": [1.5, 1.5, 1.5]}})
    sc["renderer"] = {"type": "bdpt", "max_depth": 6, "use_mis": light != "nomis"}
    path, text, d = write(scene_dir, "bdpt_" + light, sc, assets)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 4, 0.95, explain=False)
    film = g.render()
    ref = o.render_bdpt()
    lit = ref.sum(axis=2) > 1e-3
    close = (np.abs(film - ref) <= 0.05 * np.abs(ref) + 1e-5).all(axis=2)
    assert close[lit].mean() >= 0.6, close[lit].mean()
    assert abs(film.mean() - ref.mean()) < 0.02 * ref.mean(), (film.mean(), ref.mean())
    g.close()


@pytest.mark.parametrize("light", ["area", "projection", "chess_rect", "chess_cube"])
@pytest.mark.parametrize("renderer", ["path", "vol_path", "bdpt", "particle_tracer"])
def test_textured_light(rad, oracle, scene_dir, renderer, light):
    """area: a bitmap radiance on the emitter rectangle: its texels seen at hits,
    the luminance distribution behind position samples (light paths), the
    reference's zero-density direction samples (no next-event estimation from a
    bitmap light) and its direction density in the MIS weights. projection: a
    bitmap slide looked up at the light-space uv of each direction or emitted ray.
    chess_*: a chessboard radiance on a rectangle or a cube: uniform shape samples
    (next-event estimation included) read at the sample's uv."""
    from helpers import chessboard_light_room, textured_light_room, textured_projection_room
    if light.startswith("chess"):
        sc, assets = chessboard_light_room(24, 24, 4, renderer=renderer, shape=light[6:])
    else:
        make = textured_light_room if light == "area" else textured_projection_room
        sc, assets = make(24, 24, 4, renderer=renderer)
    if renderer == "particle_tracer":
        sc["sampler"]["sample_count"] = 60000
    path, text, d = write(scene_dir, "texlight_%s_%s" % (light, renderer), sc, assets)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    if renderer == "particle_tracer":
        film = g.render()
        ref = o.render_particle()
        lit = ref.sum(axis=2) > 1e-3
        close = (np.abs(film - ref) <= 0.02 * np.abs(ref) + 1e-6).all(axis=2)
        assert close[lit].mean() >= 0.9, close[lit].mean()
        assert abs(film.mean() - ref.mean()) < 0.01 * ref.mean()
    else:
        _sample_parity(g, o, 4, {"path": 0.995, "vol_path": 0.99}.get(renderer, 0.95), renderer != "bdpt")
    g.close()


@pytest.mark.parametrize("case", ["depth0", "depth1", "depth2", "rr0", "nolight", "onlysky"])
def test_bdpt_edge_cases(rad, oracle, scene_dir, case):
    """bdpt at the edges of its loops: max_depth 0-2 (the camera subpath stops
    after its first vertices, connections are not limited by max_depth), Russian
    roulette from the first bounce, a scene without lights (no light subpath, the
    reference would index light -1) and a sky as the only light (infinite-light
    subpaths and their density fix-up)."""
    sc = scenes.box_room(16, 16, 8)
    sc["renderer"] = {"type": "bdpt"}
    if case.startswith("depth"):
        sc["renderer"]["max_depth"] = int(case[-1])
    elif case == "rr0":
        sc["renderer"]["rr_depth"] = 0
    elif case == "nolight":
        del sc["scene"][-1]["light"]
    elif case == "onlysky":
        del sc["scene"][-1]["light"]
        sc["scene"][2]["to_world"]["translate"] = [0, 1, -3]  # open the back of the room a little
        sc["scene"].append({"light": {"type": "skybox", "radiance": [0.8, 0.9, 1.0]}})
    path, text, d = write(scene_dir, "bdpt_edge_" + case, sc)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    frac, lg, lo = _sample_parity(g, o, 8, 0.95, explain=False)
    film = g.render()
    ref = o.render_bdpt()
    if case == "nolight":
        assert not lo.any() and not lg.any() and not film.any() and not ref.any()
    else:
        assert abs(film.mean() - ref.mean()) < 0.02 * ref.mean(), (film.mean(), ref.mean())
    g.close()


def test_path_samples_lights(rad, oracle, scene_dir):
    """Point and projection lights (delta lights: no MIS weight on their samples) beside
    an area emitter."""
    path, text, d = lights(scene_dir, 48, 48, 4)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 4, 0.995)
    g.close()


def test_volpath_samples_point_light(rad, oracle, scene_dir):
    """vol_path with a point light and a projection light in place of the distant light:
    their samples are attenuated through the medium like any other."""
    sc, assets = scenes.volume_box(width=32, height=32, spp=2, grid=24)
    sc["scene"][2] = {"light": {"type": "point", "position": [1.5, 3.0, 1.0], "intensity": [30.0, 30.0, 30.0]}}
    sc["scene"].append({"to_world": {"translate": [0.0, 1.0, 3.0], "rotate": {"axis": [0, 1, 0], "angle": 180.0}},
                        "light": {"type": "projection", "fov": 30.0, "irradiance": [4.0, 3.0, 2.0]}})
    path, text, d = write(scene_dir, "vol_point_32", sc, assets)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    _sample_parity(g, o, 2, 0.99)
    g.close()


def test_job_film_matches_samples(rad, scene_dir):
    """The job film is the per-pixel mean of the same samples (sum in sample order, x 1/spp)."""
    path, text, d = box(scene_dir, 32, 32, 4)
    g = rad.Scene.from_file(path)
    film = g.render()
    W, H = 32, 32
    pix = np.repeat(np.arange(W * H, dtype=np.uint32), 4)
    smp = np.tile(np.arange(4, dtype=np.uint32), W * H)
    L = g.render_samples(pix, smp).reshape(H * W, 4, 3)
    acc = np.zeros((H * W, 3), np.float32)
    for s in range(4):
        li = L[:, s]
        bad = np.isnan(li).any(1) | np.isinf(li[:, 0]) | (li[:, 0] < 0)
        acc = acc + np.where(bad[:, None], 0, li).astype(np.float32)
    ref = (acc * np.float32(1.0 / 4)).reshape(H, W, 3)
    assert np.array_equal(film, ref)
    g.close()


def test_job_film_vs_oracle(rad, oracle, scene_dir):
    path, text, d = box(scene_dir, 48, 48, 8)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    fg = g.render()
    fo, _ = o.render()
    rel = np.abs(fg - fo) / np.maximum(np.abs(fo), 1e-2)
    assert (rel.max(axis=2) < 1e-3).mean() > 0.95
    assert abs(fg.mean() - fo.mean()) < 1e-3 * fo.mean()
    g.close()


def test_ztest_against_oracle_reference(rad, oracle, scene_dir):
    """Per-pixel z-test of the 64-spp GPU mean against a high-spp oracle mean."""
    W = H = 24
    path, text, d = box(scene_dir, W, H, 64, seed=5)
    g = rad.Scene.from_file(path)
    ref_path, ref_text, ref_d = box(scene_dir, W, H, 2048, seed=99)
    o = oracle.OracleScene(ref_text, ref_d)
    ref, _ = o.render()
    pix = np.repeat(np.arange(W * H, dtype=np.uint32), 64)
    smp = np.tile(np.arange(64, dtype=np.uint32), W * H)
    L = g.render_samples(pix, smp).reshape(H, W, 64, 3).astype(np.float64)
    mean = L.mean(2)
    var = L.var(2, ddof=1)
    se = np.sqrt(var / 64 + var / 2048) + 1e-6
    z = np.abs(mean - ref) / se
    frac = (z > 4).mean()
    assert frac < 0.02, "z-test failed on %.3f of pixel channels" % frac
    rel_mse = np.mean((mean - ref) ** 2 / (ref ** 2 + 1e-2))
    assert rel_mse < 0.05
    g.close()


def _vol_replicas(s, n, spp, seed0, **flags):
    out = []
    for k in range(n):
        j = s.submit(spp=spp, seed=seed0 + k, **flags)
        j.wait()
        out.append(j.film())
        j.close()
    return np.stack(out)


@pytest.mark.parametrize("base,flags", [({}, {"vol_fp16": True}),
                                        ({"vol_real_depth": True}, {"vol_bricks": True}),
                                        ({"vol_real_depth": True}, {"vol_bricks": True, "vol_fp16": True})])
def test_volpath_modes_keep_the_expectation(rad, scene_dir, base, flags):
    """The fp16 grid and the brick majorants change which samples are drawn, not
    what they estimate: per-pixel Welch z-test of independent replicas. Bricks are
    compared with the global majorant under the same estimator (null collisions
    free, underflow-free transmittance ratios), since the reference's depth rule
    ties truncation to the majorant."""
    path, text, d = volume(scene_dir, 24, 24, 4, grid=32)
    s = rad.Scene.from_file(path)
    a = _vol_replicas(s, 8, 256, 1, **base)
    b = _vol_replicas(s, 8, 256, 101, **flags)
    se = np.sqrt(a.var(0, ddof=1) / a.shape[0] + b.var(0, ddof=1) / b.shape[0]) + 1e-7
    z = (b.mean(0) - a.mean(0)) / se
    assert np.mean(np.abs(z) < 3.5) >= 0.98, np.mean(np.abs(z) < 3.5)
    am, bm = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))
    zt = (bm.mean() - am.mean()) / np.sqrt(am.var(ddof=1) / am.size + bm.var(ddof=1) / bm.size)
    assert abs(zt) < 4.0, zt
    s.close()


@pytest.mark.parametrize("flags", [{}, {"vol_fp16": True}, {"vol_real_depth": True}, {"vol_bricks": True},
                                   {"vol_bricks": True, "vol_fp16": True}])
def test_volpath_wavefront_equals_persistent(rad, scene_dir, flags):
    """The per-event wavefront (default) and the persistent kernel run the same
    loop parts in the same order per path: job films, ray counts and the 256^3
    fBm frame's samples are bit-identical."""
    path, text, d = volume(scene_dir, 48, 40, 4, grid=32)
    s = rad.Scene.from_file(path)
    films, rays = [], []
    for persistent in (False, True):
        j = s.submit(spp=6, seed=17, vol_persistent=persistent, **flags)
        j.wait()
        films.append(j.film())
        st = j.stats()
        rays.append((st["rays_closest"], st["rays_shadow"]))
        j.close()
    assert np.array_equal(films[0], films[1]) and films[0].mean() > 0
    assert rays[0] == rays[1]
    s.close()


def test_volpath_wavefront_fbm_256(rad, scene_dir):
    """The bench's volume (256^3 fBm grid, depth 32) at 128x128, 4 spp: both
    schedules give the same film, and the wavefront's samples match
    rad_render_samples."""
    sc, assets = scenes.volume_box(width=128, height=128, spp=4, grid=256)
    path = scenes.write_scene(os.path.join(str(scene_dir), "fbm256_wf"), sc, assets)
    s = rad.Scene.from_file(path)
    films = []
    for persistent in (False, True):
        j = s.submit(spp=4, seed=3, vol_persistent=persistent)
        j.wait()
        films.append(j.film())
        j.close()
    assert np.array_equal(films[0], films[1]) and films[0].mean() > 0
    pix = np.repeat(np.arange(128 * 128, dtype=np.uint32), 4)
    smp = np.tile(np.arange(4, dtype=np.uint32), 128 * 128)
    L = s.render_samples(pix, smp, seed=3).reshape(128 * 128, 4, 3).astype(np.float64)
    L[~np.isfinite(L).all(-1) | (L[..., 0] < 0)] = 0.0
    assert np.allclose(L.mean(1).reshape(128, 128, 3), films[0], rtol=1e-5, atol=1e-6)
    s.close()


@pytest.mark.gpu
def test_consecutive_jobs_reuse_buffers_and_graphs(rad, scene_dir):
    """A finished job's film, statistics buffers and captured wave graphs serve the
    scene's next job (same film; the graphs when the samples per wave match): a run
    of jobs with equal and different spp and first samples returns, bit for bit,
    the film each job gives on a freshly loaded scene."""
    path, _, _ = write(scene_dir, "reuse_box", scenes.box_room(32, 32, 4))
    runs = [(4, 0), (4, 100), (2, 7), (4, 100), (1, 3)]
    sc = rad.Scene.from_file(path)
    films = []
    for spp, first in runs:
        j = sc.submit(spp=spp, first_sample=first)
        j.wait()
        films.append(j.film())
        j.close()
    sc.close()
    for (spp, first), f in zip(runs, films):
        fresh = rad.Scene.from_file(path)
        j = fresh.submit(spp=spp, first_sample=first)
        j.wait()
        ref = j.film()
        j.close()
        fresh.close()
        assert np.array_equal(f, ref), (spp, first)
    assert np.array_equal(films[1], films[3])
