"""The guide-network oracle pinned on the CPU: fp16 rounding against numpy,
analytic gradients against finite differences, mixtures normalised."""
import numpy as np
import pytest

from oracle_lib import (GUIDE_NW, OracleGuide, guide_mix_pdf, guide_random_params, guide_random_queries,
                        guide_random_records, lib)

LO, HI = [-1.0, -2.0, 0.5], [3.0, 2.0, 4.0]


def test_half_rounding_matches_numpy():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=20000) * 10.0 ** rng.uniform(-9, 5, 20000),
                        [0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e-8, 3e-8, 6.1e-5, -6.0e-5, 2049.0, 2051.0]])
    x = x.astype(np.float32)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).astype(np.float32)
    ours = np.array([lib().orc_half_round(float(v)) for v in x], dtype=np.float32)
    assert np.array_equal(ours, ref)


def test_level_resolutions():
    g = OracleGuide(10, LO, HI, guide_random_params(10, 1))
    assert g.res[0] == 16 and g.res[-1] == 512
    assert np.all(np.diff(g.res.astype(np.int64)) > 0)


def test_emulated_forward_close_to_exact():
    g = OracleGuide(12, LO, HI, guide_random_params(12, 2))
    q = guide_random_queries(200, LO, HI, 3)
    raw16, _ = g.forward(q, exact=False)
    raw64, _ = g.forward(q, exact=True)
    scale = np.abs(raw64).max()
    assert np.abs(raw16 - raw64).max() < 2e-2 * scale


def test_mixture_is_normalised_and_consistent():
    g = OracleGuide(10, LO, HI, guide_random_params(10, 4))
    q = guide_random_queries(6, LO, HI, 5)
    raw, mix = g.forward(q, exact=True)
    assert np.allclose(mix[:, 32:40].sum(axis=1), 1.0, atol=1e-6)
    assert np.all((mix[:, 40] > 0) & (mix[:, 40] < 0.6))
    # integrate each mixture over the sphere (Fibonacci lattice)
    n = 400000
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    phi = np.pi * (1 + 5 ** 0.5) * i
    r = np.sqrt(1 - z * z)
    dirs = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1).astype(np.float32)
    for k in range(mix.shape[0]):
        m = np.repeat(mix[k:k + 1], n, axis=0)
        # lobes this sharp need the lattice to resolve them; clamp kappa for the check
        m[:, 3:32:4] = np.minimum(m[:, 3:32:4], 200.0)
        integral = guide_mix_pdf(m, dirs).mean() * 4 * np.pi
        assert abs(integral - 1.0) < 2e-3


@pytest.mark.parametrize("seed", [0, 1])
def test_gradient_matches_finite_differences(seed):
    """Central differences of the exact-mode loss. A step can straddle a ReLU
    kink, so nearly all (not all) sampled parameters must agree to 1e-3."""
    log2t = 8
    params = guide_random_params(log2t, 10 + seed, table_scale=0.3, weight_scale=0.7)
    recs = guide_random_records(24, LO, HI, 20 + seed, w_max=1.0)
    g = OracleGuide(log2t, LO, HI, params)
    grad, loss = g.grad(recs, exact=True)
    assert np.isfinite(loss) and loss != 0.0
    rng = np.random.default_rng(seed)
    n_table = g.n_table
    touched = np.flatnonzero(np.abs(grad[:n_table]) > 1e-4 * np.abs(grad[:n_table]).max())
    idx = np.concatenate([rng.choice(touched, 30, replace=False),
                          n_table + rng.choice(GUIDE_NW - 7 * 64, 90, replace=False)])
    rel = []
    for i in idx:
        h = 1e-4 * max(1.0, abs(float(params[i])))
        vals = []
        for s in (+1, -1):
            p2 = params.astype(np.float64)
            p2[i] += s * h
            vals.append(OracleGuide(log2t, LO, HI, p2.astype(np.float32)).grad(recs, exact=True)[1])
        h_eff = (np.float64(np.float32(params[i] + h)) - np.float64(np.float32(params[i] - h))) / 2.0
        fd = (vals[0] - vals[1]) / (2 * h_eff)
        rel.append(abs(fd - grad[i]) / (max(abs(fd), abs(grad[i])) + 1e-7))
    rel = np.array(rel)
    assert np.mean(rel < 1e-3) >= 0.95, np.sort(rel)[-8:]
    assert rel.max() < 5e-2


def test_emulated_gradient_close_to_exact():
    log2t = 9
    params = guide_random_params(log2t, 30)
    recs = guide_random_records(64, LO, HI, 31)
    g = OracleGuide(log2t, LO, HI, params)
    g16, l16 = g.grad(recs, exact=False)
    g64, l64 = g.grad(recs, exact=True)
    assert abs(l16 - l64) < 1e-2 * abs(l64)
    n_table = g.n_table
    for a, b in ((g16[:n_table], g64[:n_table]), (g16[n_table:], g64[n_table:])):
        assert np.linalg.norm(a - b) < 3e-2 * np.linalg.norm(b)
