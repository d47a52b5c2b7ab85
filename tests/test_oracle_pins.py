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


@pytest.mark.parametrize("bsdf", BSDFS[:8], ids=lambda b: b["type"])
def test_sample_matches_eval_and_pdf(oracle, bsdf):
    """Sample() returns f and pdf consistent with Eval()/Pdf() at the sampled direction."""
    rng = np.random.default_rng(5)
    n = 4096
    wi = directions(rng, n)
    wi[:, 2] = np.abs(wi[:, 2])
    u = rng.uniform(size=(n, 3)).astype(np.float32)
    js = bsdf_json(bsdf)
    wo, pdf, f, eta, typ = oracle.bsdf_sample(js, wi, u)
    ok = pdf > 0
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
    for b in BSDFS[:8]:
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
