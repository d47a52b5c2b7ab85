"""GPU kernels vs the CPU oracle on identical inputs, through the C ABI.

Tolerances: BSDF eval/pdf agree within 1e-5 relative (values below 1e-30 are
compared absolutely); hit primitive ids and sidedness are identical except
where two hit distances lie within 2 ulp; camera rays within 4 ulp.
"""
import numpy as np
import pytest

from helpers import BSDFS, bsdf_json, box, directions, spheres

pytestmark = pytest.mark.gpu

REL = 1e-5


def _close(a, b, rel=REL, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    return both_nan | (np.abs(a - b) <= rel * np.maximum(np.abs(b), floor)) | (a == b)


@pytest.mark.parametrize("bsdf", BSDFS, ids=lambda b: b["type"] + "_" + str(abs(hash(bsdf_json(b))) % 1000))
def test_bsdf_eval_pdf(rad, oracle, bsdf):
    rng = np.random.default_rng(7)
    n = 1 << 16
    wi, wo = directions(rng, n), directions(rng, n)
    js = bsdf_json(bsdf)
    f_g, p_g = rad.bsdf_eval(js, wi, wo)
    f_o, p_o = oracle.bsdf_eval(js, wi, wo)
    assert _close(f_g, f_o).all(), "eval mismatch in %d records" % (~_close(f_g, f_o)).any(axis=1).sum()
    assert _close(p_g, p_o).all(), "pdf mismatch in %d records" % (~_close(p_g, p_o)).sum()


@pytest.mark.parametrize("bsdf", BSDFS, ids=lambda b: b["type"] + "_" + str(abs(hash(bsdf_json(b))) % 1000))
def test_bsdf_sample(rad, oracle, bsdf):
    rng = np.random.default_rng(11)
    n = 1 << 16
    wi = directions(rng, n)
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    js = bsdf_json(bsdf)
    wo_g, p_g, f_g, e_g, t_g = rad.bsdf_sample(js, wi, u)
    wo_o, p_o, f_o, e_o, t_o = oracle.bsdf_sample(js, wi, u)
    ok = p_o > 0
    # transcendentals (sin/cos/log/pow/erf) are CUDA's own: allow 1e-5 relative on directions too
    assert (_close(p_g, p_o, 1e-4) | (~ok & (p_g <= 0))).mean() > 0.999
    assert _close(wo_g[ok], wo_o[ok], 1e-4, 1e-6).all(axis=1).mean() > 0.999
    assert _close(f_g[ok], f_o[ok], 1e-4).all(axis=1).mean() > 0.999
    assert (t_g[ok] == t_o[ok]).mean() > 0.999


def _ulp_close(a, b, ulps):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    with np.errstate(invalid="ignore"):
        d = np.abs(a.astype(np.float64) - b)
        return (a == b) | (d <= ulps * np.spacing(np.maximum(np.abs(a), np.abs(b))))


def test_camera_rays(rad, oracle, scene_dir):
    path, text, d = box(scene_dir, 64, 48)
    g = rad.Scene.from_file(path)
    o = oracle.OracleScene(text, d)
    pix = np.arange(64 * 48, dtype=np.uint32)
    rg, ro = g.camera_rays(pix, 3), o.camera_rays(pix, 3)
    assert _ulp_close(rg, ro, 4).all()
    g.close()


def _hit_parity(hg, ho):
    pg, po = hg[:, 3].view(np.uint32), ho[:, 3].view(np.uint32)
    same = pg == po
    # allowed differences: both hit, distances within 2 ulp (a tie)
    tie = (~same) & (pg != 0xFFFFFFFF) & (po != 0xFFFFFFFF) & _ulp_close(hg[:, 0], ho[:, 0], 2)
    assert (same | tie).all(), "hit id mismatch on %d rays" % (~(same | tie)).sum()
    assert (hg[same, 0] == ho[same, 0]).all()
    assert (hg[same, 4].view(np.uint32) == ho[same, 4].view(np.uint32)).all()
    return same.mean()


@pytest.mark.parametrize("which", ["box", "spheres"])
def test_trace_batch(rad, oracle, scene_dir, which):
    path, text, d = box(scene_dir) if which == "box" else spheres(scene_dir, 2000, 8)
    g = rad.Scene.from_file(path)
    o = oracle.OracleScene(text, d)
    rng = np.random.default_rng(3)
    n = 1 << 17
    pix = rng.integers(0, g.width * g.height, n).astype(np.uint32)
    cam = o.camera_rays(pix, 0)
    lo, hi = ((-1, 0, -1), (1, 2, 1)) if which == "box" else ((0, 0, 0), (100, 100, 100))
    org = rng.uniform(lo, hi, (n, 3))
    dr = directions(rng, n)
    rnd = np.concatenate([org, np.zeros((n, 1)), dr, np.full((n, 1), 3.4e38)], 1).astype(np.float32)
    for rays in (cam, rnd):
        hg, ho = g.trace(rays), o.trace(rays)
        _hit_parity(hg, ho)
        po = ho[:, 3].view(np.uint32)
        r2 = rays.copy()
        r2[:, 7] = np.where(po != 0xFFFFFFFF, ho[:, 0] * 0.999, 1e3).astype(np.float32)
        ag, ao = g.trace(r2, True), o.trace(r2, True)
        assert (ag[:, 3].view(np.uint32) == ao[:, 3].view(np.uint32)).mean() > 0.9999
    g.close()


def test_trace_edge_cases(rad, oracle, scene_dir):
    path, text, d = box(scene_dir)
    g = rad.Scene.from_file(path)
    o = oracle.OracleScene(text, d)
    rays = np.array([
        [0, 1, 0.5, 0, 0, 0, -1, 3.4e38],       # axis-aligned, hits back wall
        [0, 1, 0.5, 0, 1, 0, 0, 3.4e38],        # straight up into the emitter
        [0, 1, 5, 0, 0, 0, 1, 3.4e38],          # leaves the open box: miss
        [0, 1, 0.5, 0, 0, 0, -1, 0.1],          # tmax before any surface
        [-1, 1, 0, 0, 1, 0, 0, 3.4e38],         # origin on the left wall plane
        [0, 0, 0, 0, 0, -1, 0, 3.4e38],         # origin on the floor, pointing down
    ], dtype=np.float32)
    _hit_parity(g.trace(rays), o.trace(rays))
    empty = np.zeros((0, 8), np.float32)
    assert g.trace(empty).shape == (0, 5)
    g.close()


def test_bsdf_sweep_eval_pdf(rad, oracle):
    """Seeded sweep over the many-spheres materials' parameter ranges (helpers.
    bsdf_sweep): 10,000 Disney parameter sets (every parameter U[0, 1], each
    key present, present-and-zero or absent), rough glass at alpha in {0,
    1e-4, 1e-3} and U[0, 0.3], rough metal (GGX / Beckmann, isotropic and
    anisotropic, visible-normal sampling on and off) and diffuse, 64 direction
    pairs each: every eval and pdf within 1e-5 relative of the oracle's."""
    from helpers import bsdf_sweep
    rng = np.random.default_rng(31)
    bad = []
    for b in bsdf_sweep(10000, seed=31):
        js = bsdf_json(b)
        wi, wo = directions(rng, 64), directions(rng, 64)
        wi[:16, 2] = np.abs(wi[:16, 2])
        wo[:16, 2] = np.abs(wo[:16, 2])
        f_g, p_g = rad.bsdf_eval(js, wi, wo)
        f_o, p_o = oracle.bsdf_eval(js, wi, wo)
        if not (_close(f_g, f_o).all() and _close(p_g, p_o).all()):
            bad.append(js)
    assert not bad, "%d parameter sets differ, e.g. %s" % (len(bad), bad[:3])


def test_bsdf_sweep_sample(rad, oracle):
    """Bsdf::Sample over 2,000 Disney parameter sets and the rough glass /
    rough metal sweep: directions, pdf and f within 1e-4 relative (they pass
    through sin / cos / sqrt of the sample), sampled lobe types identical, for
    >= 99.9% of records."""
    from helpers import bsdf_sweep
    rng = np.random.default_rng(32)
    ok_all = []
    for b in bsdf_sweep(2000, seed=32):
        js = bsdf_json(b)
        wi = directions(rng, 64)
        u = rng.uniform(size=(64, 3)).astype(np.float32)
        wo_g, p_g, f_g, e_g, t_g = rad.bsdf_sample(js, wi, u)
        wo_o, p_o, f_o, e_o, t_o = oracle.bsdf_sample(js, wi, u)
        ok = (_close(p_g, p_o, 1e-4) & _close(wo_g, wo_o, 1e-4, 1e-6).all(axis=1) & _close(f_g, f_o, 1e-4).all(axis=1)
              & (t_g == t_o) & _close(e_g, e_o))
        ok_all.append(ok)
    frac = np.concatenate(ok_all).mean()
    assert frac >= 0.999, frac
