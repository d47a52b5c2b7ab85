"""Textures on the GPU vs the CPU oracle, through the C ABI: every texture of a
scene that uses each filter, wrap mode, asset format and a nested chessboard,
looked up at the same uv and uv derivatives; then whole-path parity on the
textured room (camera-ray differentials feed the trilinear / anisotropic floors).

Tolerances: nearest, bilinear and chessboard lookups are bit-exact; trilinear
and anisotropic lookups take log2f / expf from CUDA and the oracle from glibc,
so their level weights can differ in the last bit (and, on a 1-ulp boundary, the
level itself): trilinear >= 97% bit-exact; trilinear and anisotropic >= 99.95%
within 2e-3 relative."""
import numpy as np
import pytest

from helpers import sample_parity, textured

pytestmark = pytest.mark.gpu


def _uv_batch(n, seed):
    rng = np.random.default_rng(seed)
    uv = rng.uniform(-1.5, 2.5, size=(n, 2)).astype(np.float32)
    scale = 10.0 ** rng.uniform(-5, 0, size=(n, 1))
    duv = (rng.normal(size=(n, 4)) * scale).astype(np.float32)
    duv[: n // 8] = 0  # no differentials (every bounce after the first)
    return uv, duv


def test_texture_lookups_match(rad, oracle, scene_dir):
    path, text, d = textured(scene_dir, 16, 16, 1)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    n = o.texture_count()
    assert n == 15
    uv, duv = _uv_batch(20000, 3)
    # textures 0 and 13 are trilinear, 2 anisotropic, 1 a chessboard over 2; the
    # others (nearest / bilinear bitmaps, chessboards, constants) are bit-exact
    exact = {0: 0.97, 13: 0.97, 1: 0.0, 2: 0.0}  # EWA sums of expf weights: last bits differ
    for t in range(n):
        a = g.texture_eval(t, uv, duv)
        b = o.texture_eval(t, uv, duv)
        same = (a == b).all(axis=1)
        close = np.isclose(a, b, rtol=2e-3, atol=1e-6).all(axis=1)
        assert same.mean() >= exact.get(t, 1.0), (t, same.mean())
        assert close.mean() >= (0.9995 if t in exact else 1.0), (t, np.argwhere(~close)[:5].ravel(), a[~close][:3],
                                                                b[~close][:3])
    with pytest.raises(rad.RadError):
        g.texture_eval(n, uv[:1])
    g.close()


@pytest.mark.parametrize("renderer,jpeg", [("path", False), ("vol_path", False), ("path", True)])
def test_textured_room_samples(rad, oracle, scene_dir, renderer, jpeg):
    """jpeg: the colour and grey bitmaps are read from JPEG files (progressive
    4:2:0, sequential grey with restart markers) by the library's decoder."""
    path, text, d = textured(scene_dir, 48, 48, 4, renderer=renderer, jpeg=jpeg)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    sample_parity(g, o, 4, 0.995 if renderer == "path" else 0.99)
    g.close()


def test_textured_job_film(rad, oracle, scene_dir):
    """A whole job on the textured room (textured materials run in the generic
    shade class) matches the oracle's film mean."""
    path, text, d = textured(scene_dir, 48, 48, 16)
    g, o = rad.Scene.from_file(path), oracle.OracleScene(text, d)
    film = g.render()
    ref, _ = o.render()
    assert abs(film.mean() - ref.mean()) < 0.02 * ref.mean()
    g.close()
