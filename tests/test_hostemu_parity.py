"""The renderer's device code, compiled for the host (tests/hostemu: the BVH8
traversal, scene, BSDF and light functions and the wavefront kernels of
k_path.cu / k_vol.cu, run one lane at a time), against the oracle, bit for bit.

Both sides call the host libm for transcendentals, so any difference here is a
difference of algorithm. Covered: camera rays; closest and any hits on the
box room and on the full 3.2 M-triangle many-spheres field; every BSDF's
eval / pdf / sample on seeded sweeps over the parameter ranges of the
many-spheres materials (Disney with each key present or absent, rough glass
down to alpha = 0); per-sample radiance of `path`, `ao` and `vol_path` on the
small parity scenes, the 256x256 box room, the 1920x1080 many-spheres frame
and the 256^3 fBm volume.
"""
import json
import os

import numpy as np
import pytest

import hemu_lib
from helpers import (box, bsdf_sweep, directions, lights, materials, spheres, textured, volume, volume_variant,
                     write)
from radiantiumplusplus_gb300 import scenes


def _same(a, b):
    """Bitwise equality, NaN equal to NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype == np.float32:
        return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
    return a == b


@pytest.fixture(scope="module")
def field(tmp_path_factory, oracle):
    """The many-spheres stress frame: 10,000 icospheres (3.2 M triangles), 1920x1080, depth 16."""
    d = str(tmp_path_factory.mktemp("field"))
    sc, assets = scenes.many_spheres(n_spheres=10000, width=1920, height=1080, spp=1, max_depth=16, seed=2)
    path = scenes.write_scene(d, sc, assets)
    with open(path) as fh:
        text = fh.read()
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    yield h, o
    h.close()
    o.close()


def test_camera_rays_bit_exact(oracle, scene_dir, field):
    path, text, d = box(scene_dir, 64, 48, 1)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    rng = np.random.default_rng(1)
    for sc_h, sc_o, npix in ((h, o, 64 * 48), field + (1920 * 1080,)):
        pix = rng.integers(0, npix, 20000).astype(np.uint32)
        for sample in (0, 7, 123456):
            assert _same(sc_h.camera_rays(pix, sample, sc_o.seed), sc_o.camera_rays(pix, sample)).all()
    h.close()


def _trace_both(h, o, rays):
    hh, ho = h.trace(rays), o.trace(rays)
    assert _same(hh, ho).all(1).mean() == 1.0, "closest hits differ on %d rays" % (~_same(hh, ho).all(1)).sum()
    po = ho[:, 3].view(np.uint32)
    short = rays.copy()
    short[:, 7] = np.where(po != 0xFFFFFFFF, ho[:, 0] * np.float32(0.999), np.float32(1e3))
    for r in (rays, short):
        ah, ao = h.trace(r, True), o.trace(r, True)
        assert np.array_equal(ah[:, 3].view(np.uint32), ao[:, 3].view(np.uint32))
    return ho


def test_trace_many_spheres_field_bit_exact(field):
    """Closest hit (t, u, v, primitive id, sidedness) and occlusion on the
    3.2 M-triangle field: camera rays and random rays from inside the field."""
    h, o = field
    rng = np.random.default_rng(3)
    n = 1 << 18
    cam = o.camera_rays(rng.integers(0, 1920 * 1080, n).astype(np.uint32), 0)
    org = rng.uniform(0.0, 100.0, (n, 3))
    rnd = np.concatenate([org, np.zeros((n, 1)), directions(rng, n), np.full((n, 1), 3.4e38)], 1).astype(np.float32)
    for rays in (cam, rnd):
        hits = _trace_both(h, o, rays)
        assert (hits[:, 3].view(np.uint32) != 0xFFFFFFFF).mean() > 0.5


def test_trace_box_edge_cases_bit_exact(oracle, scene_dir):
    path, text, d = box(scene_dir)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    rays = np.array([
        [0, 1, 0.5, 0, 0, 0, -1, 3.4e38],
        [0, 1, 0.5, 0, 1, 0, 0, 3.4e38],
        [0, 1, 5, 0, 0, 0, 1, 3.4e38],
        [0, 1, 0.5, 0, 0, 0, -1, 0.1],
        [-1, 1, 0, 0, 1, 0, 0, 3.4e38],
        [0, 0, 0, 0, 0, -1, 0, 3.4e38],
        [0, 1, 0, 0, 1e-30, 0, -1, 3.4e38],  # denormal-sized direction component
        [0.3, 0.4, 0.2, 0, 0, 1, 0, 3.4e38],  # straight up from inside the box
    ], dtype=np.float32)
    rng = np.random.default_rng(5)
    n = 1 << 16
    org = rng.uniform((-1, 0, -1), (1, 2, 1), (n, 3))
    rnd = np.concatenate([org, np.zeros((n, 1)), directions(rng, n), np.full((n, 1), 3.4e38)], 1).astype(np.float32)
    _trace_both(h, o, np.concatenate([rays, rnd]))
    h.close()


def test_bsdf_sweep_bit_exact(oracle):
    """Eval / pdf / sample of 2,000 Disney parameter sets (every parameter
    U[0, 1], each key present, present-and-zero or absent), rough glass at
    alpha in {0, 1e-4, 1e-3} and U[0, 0.3] (alpha = 0 is the degenerate D that
    microfacet.cpp:151 guards), rough metal and diffuse: 64 direction pairs
    and 64 samples each, identical bits."""
    rng = np.random.default_rng(12)
    bad = []
    for b in bsdf_sweep(2000):
        js = json.dumps(b)
        wi, wo = directions(rng, 64), directions(rng, 64)
        wi[:8, 2] = np.abs(wi[:8, 2])  # a few same-hemisphere pairs for the reflection lobes
        wo[:8, 2] = np.abs(wo[:8, 2])
        fh, ph = hemu_lib.bsdf_eval(js, wi, wo)
        fo, po = oracle.bsdf_eval(js, wi, wo)
        u = rng.uniform(0, 1, (64, 3)).astype(np.float32)
        sh = hemu_lib.bsdf_sample(js, wi, u)
        so = oracle.bsdf_sample(js, wi, u)
        ok = _same(fh, fo).all() and _same(ph, po).all() and all(_same(x, y).all() for x, y in zip(sh, so))
        if not ok:
            bad.append(js)
    assert not bad, "%d parameter sets differ, e.g. %s" % (len(bad), bad[:3])


def _samples_bit_exact(h, o, n, seed=7, npix=None, vol_mode=0):
    rng = np.random.default_rng(seed)
    npix = npix or o.width * o.height
    pix = rng.integers(0, npix, n).astype(np.uint32)
    smp = rng.integers(0, 1 << 16, n).astype(np.uint32)
    lh = h.render_samples(pix, smp, o.seed, vol_mode)
    lo = o.render_samples(pix, smp)
    same = _same(lh, lo).all(1)
    assert same.all(), "%d of %d samples differ" % ((~same).sum(), n)
    assert np.abs(lo).sum() > 0


def _ao_box(d):
    sc = scenes.box_room(48, 48, 4)
    sc["renderer"] = {"type": "ao"}
    return write(d, "hemu_ao", sc)


def _textured_light(d):
    from helpers import textured_light_room
    sc, assets = textured_light_room()
    return write(d, "hemu_tlight", sc, assets)


@pytest.mark.parametrize("which", ["box", "materials", "lights", "spheres", "textured", "textured_light", "ao",
                                   "volume"])
def test_render_samples_bit_exact(oracle, scene_dir, which):
    """Per-sample Li of the wavefront kernels (generate, extend, the shade
    classes, shadow; or the vol_path kernel) equals the oracle's Path::Li /
    VolPath::Li bit for bit, 4,096 random (pixel, sample) pairs per scene."""
    make = {"box": lambda d: box(d, 48, 48, 4), "materials": materials, "lights": lights,
            "spheres": lambda d: spheres(d, 300, 4, 48, 32, 4), "textured": textured,
            "textured_light": _textured_light, "ao": _ao_box, "volume": lambda d: volume(d, 32, 32, 4, grid=24)}
    path, text, d = make[which](scene_dir)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    _samples_bit_exact(h, o, 4096)
    h.close()


def test_mixed_wave_bit_exact(oracle, scene_dir):
    """A mixed wave (the serving loop's several jobs in one launch of each stage,
    each path with its job's scene, pixels, samples and seed: the MIX kernels)
    gives every path of every job its scene's oracle Path::Li bit for bit."""
    made = [box(scene_dir, 24, 16, 4), materials(scene_dir, 20, 20, 4, 2), spheres(scene_dir, 200, 3, 24, 16, 4)]
    hs = [hemu_lib.HemuScene(text, d) for _, text, d in made]
    os_ = [oracle.OracleScene(text, d) for _, text, d in made]
    npix = [o.width * o.height for o in os_]
    spw, sample0 = 3, 17
    outs = hemu_lib.render_mixed(hs, npix, spw, sample0, [o.seed for o in os_])
    for o, n, lh in zip(os_, npix, outs):
        pix = np.tile(np.arange(n, dtype=np.uint32), spw)
        smp = np.repeat(np.arange(sample0, sample0 + spw, dtype=np.uint32), n)
        lo = o.render_samples(pix, smp)
        same = _same(lh, lo).all(1)
        assert same.all(), "%d of %d samples differ" % ((~same).sum(), same.size)
        assert np.abs(lo).sum() > 0
    for h in hs:
        h.close()


def test_render_samples_box_room_256_bit_exact(oracle, scene_dir):
    """The box room at its stated size: 256x256, depth 8, Russian roulette from 3."""
    path, text, d = box(scene_dir, 256, 256, 64)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    _samples_bit_exact(h, o, 16384)
    h.close()


def test_render_samples_many_spheres_field_bit_exact(field):
    h, o = field
    _samples_bit_exact(h, o, 8192, seed=9)


def test_render_samples_fbm_volume_256_bit_exact(oracle, tmp_path):
    """vol_path on the 256^3 fBm density grid (sigma_t scale 20, albedo 0.9,
    HG g = 0.6, rough-glass box, depth 32), at a reduced frame."""
    sc, assets = scenes.volume_box(width=96, height=96, spp=1, max_depth=32, grid=256)
    path = scenes.write_scene(str(tmp_path), sc, assets)
    with open(path) as fh:
        text = fh.read()
    h, o = hemu_lib.HemuScene(text, str(tmp_path)), oracle.OracleScene(text, str(tmp_path))
    _samples_bit_exact(h, o, 4096, seed=13)
    _samples_bit_exact(h, o, 4096, seed=14, vol_mode=VOL_WAVEFRONT)
    h.close()
    o.close()


VOL_WAVEFRONT = 256  # hemu_render_samples: run vol_path as the per-event wavefront


@pytest.mark.parametrize("variant", ["index_matched", "homogeneous_sphere"])
def test_volume_media_variants_bit_exact(oracle, scene_dir, variant):
    """vol_path through an index-matched boundary (a medium in a shape without a
    BSDF: the path crosses it and continues in the next loop iteration) and
    through a homogeneous medium in a glass sphere next to the grid, with both
    schedules (persistent kernel and per-event wavefront) against the oracle."""
    path, text, d = volume_variant(scene_dir, variant)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    _samples_bit_exact(h, o, 2048, seed=31)
    _samples_bit_exact(h, o, 2048, seed=32, vol_mode=VOL_WAVEFRONT)
    h.close()


def test_volume_wavefront_bit_exact(oracle, scene_dir):
    """The per-event wavefront schedule of vol_path (a kernel per loop part over
    queues, state stored between parts) gives every path the radiance of the
    persistent schedule and of the oracle, bit for bit; with the opt-in
    estimators (real depth, brick majorants) it equals the persistent kernel."""
    path, text, d = volume(scene_dir, 32, 32, 4, grid=24)
    h, o = hemu_lib.HemuScene(text, d), oracle.OracleScene(text, d)
    _samples_bit_exact(h, o, 4096, seed=21, vol_mode=VOL_WAVEFRONT)
    rng = np.random.default_rng(5)
    pix = rng.integers(0, o.width * o.height, 2048).astype(np.uint32)
    smp = rng.integers(0, 1 << 16, 2048).astype(np.uint32)
    for mode in (4, 1):  # kVolRealDepth, kVolBricks
        a = h.render_samples(pix, smp, o.seed, mode)
        b = h.render_samples(pix, smp, o.seed, mode | VOL_WAVEFRONT)
        assert _same(a, b).all(), mode
        assert np.abs(a).sum() > 0
    h.close()


def test_ulp_explanation_discriminates(oracle, scene_dir):
    """The GPU parity tests accept a differing sample only if one- or two-ulp
    moves of its transcendental results flip it in the harness. That must not
    hold for samples in general, or it would explain away a real device bug:
    of random vol_path samples (the most ulp-sensitive renderer here) almost
    none flip."""
    from helpers import ulp_sensitive
    path, text, d = volume(scene_dir, 32, 32, 4, grid=24)
    o = oracle.OracleScene(text, d)
    rng = np.random.default_rng(17)
    pix = rng.integers(0, 32 * 32, 48).astype(np.uint32)
    smp = rng.integers(0, 1 << 16, 48).astype(np.uint32)
    lo = o.render_samples(pix, smp)
    sens = ulp_sensitive(o, pix, smp, lo)
    assert sens.mean() <= 0.1, sens.mean()
