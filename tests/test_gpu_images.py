"""Image-level parity: GPU renders against high-spp oracle references
(tests/golden, made by tests/golden/make_references.py from the oracle's
Path::Li / VolPath::Li).

* 64 spp: a per-pixel z-test of the GPU mean. Each pixel channel's error is
  scaled by the standard error of the 64-sample mean (from the GPU samples'
  own variance, plus the reference's); at most 1% of pixel channels may lie
  beyond 4 standard errors (Monte Carlo means at 64 spp are heavy tailed, so
  the fraction allowed is far above a normal tail's 6e-5, but a biased
  estimator fails it wholesale), and the frame means agree within 3 standard
  errors.
* converged: the GPU job film at many samples per pixel reaches
  relMSE < 1e-3 against the reference, relMSE = mean over pixel channels of
  (x - ref)^2 / (ref^2 + 1e-2 * mean(ref)^2).
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_references as refs  # noqa: E402

pytestmark = pytest.mark.gpu


def _reference(name):
    d = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return d["mean"].astype(np.float64), int(d["spp"])


def _scene(rad, scene_dir, name):
    from radiantiumplusplus_gb300 import scenes
    sc, assets = refs.scene_of(name)
    path = scenes.write_scene(os.path.join(str(scene_dir), "img_" + name), sc, assets)
    return rad.Scene.from_file(path)


def rel_mse(x, ref):
    eps = 1e-2 * ref.mean() ** 2
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + eps)))


@pytest.mark.parametrize("name", refs.NAMES)
def test_64spp_ztest_against_reference(rad, scene_dir, name):
    ref, ref_spp = _reference(name)
    s = _scene(rad, scene_dir, name)
    H, W = ref.shape[:2]
    spp = 64
    pix = np.repeat(np.arange(W * H, dtype=np.uint32), spp)
    smp = np.tile(np.arange(spp, dtype=np.uint32), W * H)
    L = s.render_samples(pix, smp).reshape(H, W, spp, 3).astype(np.float64)
    bad = np.isnan(L).any(-1) | np.isinf(L[..., 0]) | (L[..., 0] < 0)  # dropped as the film drops them
    L[bad] = 0.0
    mean = L.mean(2)
    var = L.var(2, ddof=1)
    se = np.sqrt(var / spp + var / ref_spp) + 1e-7
    z = np.abs(mean - ref) / se
    frac = float((z > 4).mean())
    assert frac < 0.01, "%s: %.4f of pixel channels beyond 4 standard errors" % (name, frac)
    se_frame = np.sqrt(var.sum() / spp) / mean.size
    assert abs(mean.mean() - ref.mean()) < 3 * se_frame + 1e-3 * ref.mean(), (name, mean.mean(), ref.mean())
    # the job film of the same samples is their mean (sample_renderer.cpp:109-114)
    film = s.render(spp=spp)
    assert np.allclose(film, mean, rtol=1e-5, atol=1e-6)
    s.close()


@pytest.mark.parametrize("name,spp", [("box_room_256", 16384), ("many_spheres_96x54", 65536),
                                      ("fbm_volume_64", 65536)])
def test_converged_relmse_below_1e3(rad, scene_dir, name, spp):
    ref, ref_spp = _reference(name)
    s = _scene(rad, scene_dir, name)
    j = s.submit(spp=spp, seed=424242)
    j.wait()
    film = j.film().astype(np.float64)
    j.close()
    s.close()
    r = rel_mse(film, ref)
    assert r < 1e-3, "%s: relMSE %.2e at %d spp" % (name, r, spp)
