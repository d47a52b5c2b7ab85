"""GPU parity at the benchmark configurations, not only on small scenes:

* the many-spheres stress frame (10,000 icospheres, 3.2 M triangles, 1920x1080,
  depth 16) -- closest and any hits of 2^20 camera rays and 2^20 random rays
  against the oracle's intersector, identical bits (hit acceptance is
  t in (tmin, best) with the lower primitive id winning an exact tie, in both,
  so the result does not depend on the BVH); and per-sample radiance at random
  pixels of the frame;
* the volumetric scene with its 256^3 fBm density grid (sigma_t scale 20,
  albedo 0.9, HG g = 0.6, rough-glass box, depth 32) at a reduced frame:
  per-sample radiance.

Per-sample agreement and its explanation are those of helpers.sample_parity.
"""
import numpy as np
import pytest

from helpers import directions, sample_parity, sample_parity_at
from radiantiumplusplus_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def field(rad, oracle, tmp_path_factory):
    d = str(tmp_path_factory.mktemp("cfg_field"))
    sc, assets = scenes.many_spheres(n_spheres=10000, width=1920, height=1080, spp=1, max_depth=16, seed=2)
    path = scenes.write_scene(d, sc, assets)
    g = rad.Scene.from_file(path)
    o = oracle.OracleScene.from_file(path)
    yield g, o
    g.close()
    o.close()


def _same(a, b):
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def test_trace_many_spheres_field(field):
    g, o = field
    rng = np.random.default_rng(21)
    n = 1 << 20
    cam = o.camera_rays(rng.integers(0, 1920 * 1080, n).astype(np.uint32), 0)
    org = rng.uniform(0.0, 100.0, (n, 3))
    rnd = np.concatenate([org, np.zeros((n, 1)), directions(rng, n), np.full((n, 1), 3.4e38)], 1).astype(np.float32)
    for rays in (cam, rnd):
        hg, ho = g.trace(rays), o.trace(rays)
        same = _same(hg, ho).all(1)
        assert same.all(), "%d of %d closest hits differ" % ((~same).sum(), n)
        assert (ho[:, 3].view(np.uint32) != 0xFFFFFFFF).mean() > 0.5
        short = rays.copy()
        po = ho[:, 3].view(np.uint32)
        short[:, 7] = np.where(po != 0xFFFFFFFF, ho[:, 0] * np.float32(0.999), np.float32(1e3))
        for r in (rays, short):
            assert np.array_equal(g.trace(r, True)[:, 3].view(np.uint32), o.trace(r, True)[:, 3].view(np.uint32))


def test_path_samples_many_spheres_field(field):
    g, o = field
    rng = np.random.default_rng(22)
    n = 1 << 16
    pix = rng.integers(0, 1920 * 1080, n).astype(np.uint32)
    smp = rng.integers(0, 256, n).astype(np.uint32)
    sample_parity_at(g, o, pix, smp, 0.995)


def test_volpath_samples_fbm_256(rad, oracle, tmp_path):
    sc, assets = scenes.volume_box(width=96, height=96, spp=1, max_depth=32, grid=256)
    path = scenes.write_scene(str(tmp_path), sc, assets)
    g, o = rad.Scene.from_file(path), oracle.OracleScene.from_file(path)
    sample_parity(g, o, 2, 0.99)
    g.close()
    o.close()
