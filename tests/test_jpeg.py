"""JPEG assets (image_default -> stbi_load). Files come from the T.81 encoder in
tests/imgenc.py; the library's decoder must return, bit for bit, what a numpy
restatement of stb_image's sample pipeline makes of the encoder's quantised
coefficients (16-bit dequantisation, the integer islow inverse DCT, the
triangle-filter chroma upsampling with its row stepping, the fixed-point YCbCr ->
RGB, CMYK / YCCK combination, grey output). Entropy decoding (sequential and
progressive scans, restart intervals) is therefore checked exactly; the
restated IDCT is checked against the mathematical one, and a high-quality round
trip against the encoded image."""
import numpy as np
import pytest

import imgenc


def _f2f(x):
    return int(np.float32(x) * np.float32(4096) + np.float32(0.5))


def _idct1d(s):
    s0, s1, s2, s3, s4, s5, s6, s7 = s
    p1 = (s2 + s6) * _f2f(0.5411961)
    t2 = p1 + s6 * _f2f(-1.847759065)
    t3 = p1 + s2 * _f2f(0.765366865)
    t0, t1 = (s0 + s4) * 4096, (s0 - s4) * 4096
    x0, x3, x1, x2 = t0 + t3, t0 - t3, t1 + t2, t1 - t2
    o0, o1, o2, o3 = s7, s5, s3, s1
    p5 = (o0 + o2 + o1 + o3) * _f2f(1.175875602)
    q1 = p5 + (o0 + o3) * _f2f(-0.899976223)
    q2 = p5 + (o1 + o2) * _f2f(-2.562915447)
    q3 = (o0 + o2) * _f2f(-1.961570560)
    q4 = (o1 + o3) * _f2f(-0.390180644)
    t3 = o3 * _f2f(1.501321110) + q1 + q4
    t2 = o2 * _f2f(3.072711026) + q2 + q3
    t1 = o1 * _f2f(2.053119869) + q2 + q4
    t0 = o0 * _f2f(0.298631336) + q1 + q3
    return (x0, x1, x2, x3), (t0, t1, t2, t3)


def _idct(d):
    """(..., 64) dequantised row-major blocks -> (..., 8, 8) samples 0..255."""
    d = d.reshape(d.shape[:-1] + (8, 8)).astype(np.int64)
    (x0, x1, x2, x3), (t0, t1, t2, t3) = _idct1d([d[..., k, :] for k in range(8)])  # columns
    cols = [(x0 + 512 + t3) >> 10, (x1 + 512 + t2) >> 10, (x2 + 512 + t1) >> 10, (x3 + 512 + t0) >> 10,
            (x3 + 512 - t0) >> 10, (x2 + 512 - t1) >> 10, (x1 + 512 - t2) >> 10, (x0 + 512 - t3) >> 10]
    v = np.stack(cols, axis=-2)  # [..., row, column]
    (x0, x1, x2, x3), (t0, t1, t2, t3) = _idct1d([v[..., :, k] for k in range(8)])  # rows
    b = 65536 + (128 << 17)
    rows = [(x0 + b + t3) >> 17, (x1 + b + t2) >> 17, (x2 + b + t1) >> 17, (x3 + b + t0) >> 17,
            (x3 + b - t0) >> 17, (x2 + b - t1) >> 17, (x1 + b - t2) >> 17, (x0 + b - t3) >> 17]
    return np.clip(np.stack(rows, axis=-1), 0, 255)


def _wrap16(v):
    return ((v + 32768) % 65536) - 32768


def _upsample_row(near, far, w, hs, vs):
    near, far = near[:w].astype(np.int64), far[:w].astype(np.int64)
    if hs == 1 and vs == 1:
        return near
    if hs == 1 and vs == 2:
        return (3 * near + far + 2) >> 2
    if hs == 2 and vs == 1:
        if w == 1:
            return np.array([near[0], near[0]])
        out = np.zeros(2 * w, np.int64)
        out[0::2][1:] = (3 * near[1:] + near[:-1] + 2) >> 2
        out[1::2][:-1] = (3 * near[:-1] + near[1:] + 2) >> 2
        out[0], out[-1] = near[0], near[-1]
        out[-2] = (3 * near[-2] + near[-1] + 2) >> 2  # stb weights the last pair the other way round
        return out
    if hs == 2 and vs == 2:
        t = 3 * near + far
        if w == 1:
            return np.array([(t[0] + 2) >> 2] * 2)
        out = np.zeros(2 * w, np.int64)
        out[1:-1:2] = (3 * t[:-1] + t[1:] + 8) >> 4
        out[2::2] = (3 * t[1:] + t[:-1] + 8) >> 4
        out[0], out[-1] = (t[0] + 2) >> 2, (t[-1] + 2) >> 2
        return out
    return np.repeat(near, hs)


def _ycc(y, cb, cr):
    kcr, kcrg, kcbg, kcb = (_f2f(c) << 8 for c in (1.402, 0.71414, 0.34414, 1.772))
    yf = (y << 20) + (1 << 19)
    vr, vb = cr - 128, cb - 128
    r = (yf + vr * kcr) >> 20
    g = (yf + vr * -kcrg + ((vb * -kcbg) & -65536)) >> 20
    b = (yf + vb * kcb) >> 20
    return np.clip(np.stack([r, g, b], axis=-1), 0, 255)


def _blinn(x, y):
    t = x * y + 128
    return (t + (t >> 8)) >> 8


def _luma(r, g, b):
    return (r * 77 + g * 150 + 29 * b) >> 8


def expected(coef, comps, qt, X, Y, req, is_rgb=False, adobe=None):
    """stb_image's samples for the quantised coefficients -> (Y, X, req) uint8."""
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    nc = len(comps)
    decode_n = 1 if (nc == 3 and req < 3 and not is_rgb) else nc
    rows = []
    for c in comps[:decode_n]:
        blocks = _wrap16(_wrap16(coef[c["id"]]) * qt[c["id"]])
        s = _idct(blocks)  # (by, bx, 8, 8)
        plane = s.transpose(0, 2, 1, 3).reshape(s.shape[0] * 8, s.shape[1] * 8)
        hs, vs = hmax // c["h"], vmax // c["v"]
        cy = -(-Y * c["v"] // vmax)
        wl = -(-X // hs)
        ystep, ypos, l0, l1 = vs >> 1, 0, 0, 0
        out = []
        for _ in range(Y):
            bot = ystep >= (vs >> 1)
            out.append(_upsample_row(plane[l1 if bot else l0], plane[l0 if bot else l1], wl, hs, vs)[:X])
            ystep += 1
            if ystep >= vs:
                ystep, l0 = 0, l1
                ypos += 1
                if ypos < cy:
                    l1 += 1
        rows.append(np.array(out))
    co = rows
    if req == 3:
        if nc == 3:
            px = np.stack(co, axis=-1) if is_rgb else _ycc(*co)
        elif nc == 4:
            if adobe == 0:
                px = np.stack([_blinn(co[k], co[3]) for k in range(3)], axis=-1)
            elif adobe == 2:
                px = _blinn(255 - _ycc(*co[:3]), co[3][..., None])
            else:
                px = _ycc(*co[:3])
        else:
            px = np.repeat(co[0][..., None], 3, axis=-1)
    else:
        if is_rgb:
            px = _luma(*co)
        elif nc == 4 and adobe == 0:
            px = _luma(*[_blinn(co[k], co[3]) for k in range(3)])
        elif nc == 4 and adobe == 2:
            px = _blinn(255 - co[0], co[3])
        else:
            px = co[0]
        px = px[..., None]
    return px.astype(np.uint8)


def _quant(rng, n, big=False):
    q = rng.integers(1, 24, size=(n, 64))
    if big:
        q[:, 10:] = rng.integers(256, 400, size=(n, 54))
    return q


PROG = [((1, 2, 3), 0, 0, 0, 1), ((1,), 1, 5, 0, 2), ((1,), 6, 63, 0, 2), ((2,), 1, 63, 0, 1), ((3,), 1, 63, 0, 1),
        ((1,), 1, 63, 2, 1), ((1, 2, 3), 0, 0, 1, 0), ((1,), 1, 63, 1, 0), ((2,), 1, 63, 1, 0), ((3,), 1, 63, 1, 0)]
PROG1 = [((1,), 0, 0, 0, 2), ((1,), 1, 9, 0, 1), ((1,), 10, 63, 0, 3), ((1,), 10, 63, 3, 2), ((1,), 0, 0, 2, 1),
         ((1,), 10, 63, 2, 1), ((1,), 1, 9, 1, 0), ((1,), 10, 63, 1, 0), ((1,), 0, 0, 1, 0)]
ADOBE = lambda t: b"\xff\xee\x00\x0eAdobe\x00\x64\x00\x00\x00\x00" + bytes([t])  # noqa: E731
JFIF = b"\xff\xe0\x00\x10JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00"

# (name, components, sampling, size, options)
CASES = [
    ("grey", 1, [(1, 1)], (37, 23), {}),
    ("grey_h2v2", 1, [(2, 2)], (19, 9), {}),
    ("444", 3, [(1, 1)] * 3, (37, 23), {"app": (JFIF,)}),
    ("422", 3, [(2, 1), (1, 1), (1, 1)], (37, 23), {}),
    ("420", 3, [(2, 2), (1, 1), (1, 1)], (37, 23), {}),
    ("440", 3, [(1, 2), (1, 1), (1, 1)], (21, 30), {}),
    ("411", 3, [(4, 1), (1, 1), (1, 1)], (45, 17), {}),
    ("luma_sub", 3, [(1, 1), (1, 2), (1, 2)], (16, 17), {}),
    ("420_1px", 3, [(2, 2), (1, 1), (1, 1)], (1, 1), {}),
    ("420_3x2", 3, [(2, 2), (1, 1), (1, 1)], (3, 2), {}),
    ("420_restart", 3, [(2, 2), (1, 1), (1, 1)], (70, 41), {"restart": 3}),
    ("420_separate_scans", 3, [(2, 2), (1, 1), (1, 1)], (37, 23), {"scans": [(1,), (2, 3)]}),
    ("444_q16", 3, [(1, 1)] * 3, (24, 16), {"big": True}),
    ("rgb_ids", 3, [(1, 1)] * 3, (20, 12), {"ids": [82, 71, 66]}),
    ("rgb_adobe", 3, [(1, 1)] * 3, (20, 12), {"app": (ADOBE(0),)}),
    ("cmyk", 4, [(1, 1)] * 4, (20, 12), {"app": (ADOBE(0),)}),
    ("ycck", 4, [(2, 2), (1, 1), (1, 1), (2, 2)], (20, 12), {"app": (ADOBE(2),)}),
    ("four_plain", 4, [(1, 1)] * 4, (20, 12), {}),
    ("prog_420", 3, [(2, 2), (1, 1), (1, 1)], (45, 30), {"scans": PROG}),
    ("prog_420_restart", 3, [(2, 2), (1, 1), (1, 1)], (45, 30), {"scans": PROG, "restart": 2}),
    ("prog_grey", 1, [(1, 1)], (53, 29), {"scans": PROG1}),
    ("prog_grey_restart", 1, [(1, 1)], (53, 29), {"scans": PROG1, "restart": 5}),
]


def _make(name, nc, sampling, size, opt, seed):
    rng = np.random.default_rng(seed)
    X, Y = size
    yy, xx = np.mgrid[0:Y, 0:X]
    planes = []
    for k in range(nc):  # smooth ramps plus noise: many coefficient magnitudes
        base = 128 + 90 * np.sin(0.21 * (k + 1) * xx + 0.13 * yy + k) * np.cos(0.17 * yy - 0.05 * k * xx)
        planes.append(np.clip(base + rng.normal(0, 25, size=(Y, X)), 0, 255))
    q = _quant(rng, nc, opt.get("big", False))
    data, coef, comps, qt = imgenc.jpeg(planes, sampling, q, X, Y, ids=opt.get("ids"), scans=opt.get("scans"),
                                        restart=opt.get("restart", 0), app=opt.get("app", ()))
    return data, coef, comps, qt


@pytest.mark.parametrize("name,nc,sampling,size,opt", CASES, ids=[c[0] for c in CASES])
def test_jpeg_decode_matches_restated_pipeline(oracle, tmp_path, name, nc, sampling, size, opt):
    data, coef, comps, qt = _make(name, nc, sampling, size, opt, seed=len(name))
    X, Y = size
    path = tmp_path / (name + ".jpg")
    path.write_bytes(data)
    is_rgb = nc == 3 and (opt.get("ids") == [82, 71, 66] or any(a[4:9] == b"Adobe" for a in opt.get("app", ())))
    adobe = None
    for a in opt.get("app", ()):
        if a[4:9] == b"Adobe":
            adobe = a[15]
    for req in (3, 1):
        got = oracle.image_load({"type": "image_default", "channel": req, "is_to_linear": False,
                                 "is_flip_y": False}, path)
        want = expected(coef, comps, qt, X, Y, req, is_rgb, adobe)
        assert got.shape == (Y, X, req)
        assert np.array_equal(got, (want / np.float32(255)).astype(np.float32)), (
            req, np.abs(got * 255 - want).max())
    flipped = oracle.image_load({"type": "image_default", "is_to_linear": False}, path)  # is_flip_y defaults true
    assert np.array_equal(flipped, (expected(coef, comps, qt, X, Y, 3, is_rgb, adobe)[::-1] /
                                    np.float32(255)).astype(np.float32))


def test_jpeg_islow_idct_is_within_one_level_of_the_exact_transform():
    """The restated integer IDCT against the mathematical 8x8 inverse DCT (+128,
    rounded, clamped) on random blocks of realistic magnitudes: at most one level
    apart (IEEE 1180-style accuracy)."""
    rng = np.random.default_rng(7)
    n = 4000
    scale = 600.0 / (1 + np.arange(64) % 8 + np.arange(64) // 8)
    d = np.round(rng.laplace(0, 1, size=(n, 64)) * scale).astype(np.int64)
    got = _idct(d)
    m = imgenc._DCT
    exact = np.einsum("ux,nuv,vy->nxy", m, d.reshape(n, 8, 8).astype(np.float64), m)
    want = np.clip(np.floor(exact + 128.5), 0, 255)
    assert np.abs(got - want).max() <= 1
    assert (got == want).mean() > 0.97


def test_jpeg_round_trip_reproduces_the_image(oracle, tmp_path):
    """Quantiser 1 everywhere, 4:4:4 YCbCr from an RGB image with the JFIF
    transform: the decoded RGB is within a few levels of the original."""
    rng = np.random.default_rng(3)
    Y, X = 24, 40
    yy, xx = np.mgrid[0:Y, 0:X]
    rgb = np.stack([128 + 100 * np.sin(0.2 * xx + 0.1 * yy), 128 + 90 * np.cos(0.15 * yy),
                    60 + 3 * xx + rng.uniform(0, 20, (Y, X))], axis=-1).clip(0, 255)
    r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
    yc = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
    data, coef, comps, qt = imgenc.jpeg([yc, cb, cr], [(1, 1)] * 3, np.ones((3, 64)), X, Y, app=(JFIF,))
    (tmp_path / "rt.jpg").write_bytes(data)
    got = oracle.image_load({"type": "image_default", "is_to_linear": False, "is_flip_y": False}, tmp_path / "rt.jpg")
    assert np.abs(got * 255 - rgb).max() < 3.5


@pytest.mark.parametrize("name", ["flower.jpg", "china.jpg"])
def test_jpeg_camera_files_decode(oracle, tmp_path, name):
    """Two JPEG photographs shipped with scikit-learn (when it is installed):
    they decode to their frame size with plausible colour statistics, and the
    grey request is the decoded Y plane, close to the luma of the colour decode."""
    sk = pytest.importorskip("sklearn")
    import os
    path = os.path.join(os.path.dirname(sk.__file__), "datasets", "images", name)
    if not os.path.exists(path):
        pytest.skip("sample image absent")
    rgb = oracle.image_load({"type": "image_default", "is_to_linear": False, "is_flip_y": False}, path)
    assert rgb.shape == (427, 640, 3)
    assert 0.15 < rgb.mean() < 0.85 and rgb.std() > 0.1
    grey = oracle.image_load({"type": "image_default", "channel": 1, "is_to_linear": False,
                              "is_flip_y": False}, path)[..., 0]
    luma = 0.299 * rgb[..., 0] + 0.587 * rgb[..., 1] + 0.114 * rgb[..., 2]
    assert np.abs(grey - luma).mean() < 2.0 / 255
