"""Image decoders behind the bitmap texture's assets (PNG / PNM through
image_default, Radiance .hdr through image_hdr, OpenEXR through image_exr),
checked against images encoded in Python from the format specifications
(tests/imgenc.py) and against the conversions of rad.core asset/image_stb.cpp,
image_hdr.cpp and image_exr.cpp."""
import numpy as np
import pytest

import imgenc


def _srgb_to_linear(v):
    v = np.asarray(v, np.float32)
    return np.where(v <= np.float32(0.04045), v * np.float32(1.0 / 12.92),
                    np.power((v + np.float32(0.055)) * np.float32(1.0 / 1.055), np.float32(2.4)))


def _load(oracle, tmp_path, name, data, asset):
    path = tmp_path / name
    path.write_bytes(data)
    return oracle.image_load(asset, path)


def _luma(rgb):
    rgb = rgb.astype(np.int64)
    return (rgb[..., 0] * 77 + rgb[..., 1] * 150 + 29 * rgb[..., 2]) >> 8


CASES = [  # (colour type, bit depth, channels in the file)
    (0, 8, 1), (0, 16, 1), (0, 1, 1), (0, 2, 1), (0, 4, 1), (2, 8, 3), (2, 16, 3), (4, 8, 2), (6, 8, 4),
    (6, 16, 4), (3, 8, 1), (3, 4, 1), (3, 1, 1)]


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("colour,depth,c", CASES, ids=lambda v: str(v))
def test_png_decode(oracle, tmp_path, colour, depth, c, interlace):
    rng = np.random.default_rng(colour * 100 + depth)
    h, w = 13, 21  # odd sizes exercise partial Adam7 passes and row padding
    top = (1 << depth) - 1
    samples = rng.integers(0, top + 1, size=(h, w, c))
    palette = None
    if colour == 3:
        palette = rng.integers(0, 256, size=(1 << depth, 3))
        samples = rng.integers(0, 1 << depth, size=(h, w, 1))
    data = imgenc.png(samples, depth, colour, palette, interlace=interlace)
    # 8-bit samples as stbi_load returns them
    if colour == 3:
        rgb8 = palette[samples[..., 0]]
    elif depth == 16:
        rgb8 = samples >> 8
    elif depth < 8:
        rgb8 = samples * {1: 255, 2: 85, 4: 17}[depth]
    else:
        rgb8 = samples
    if rgb8.shape[2] in (1, 2):
        want3 = np.repeat(rgb8[..., :1], 3, axis=2)
        want1 = rgb8[..., 0]
    else:
        want3 = rgb8[..., :3]
        want1 = _luma(rgb8[..., :3])
    got3 = _load(oracle, tmp_path, "a.png", data, {"type": "image_default", "is_to_linear": False})
    assert np.array_equal(got3, (want3[::-1] / np.float32(255)).astype(np.float32))
    got1 = _load(oracle, tmp_path, "b.png", data, {"type": "image_default", "channel": 1, "is_flip_y": False})
    assert np.array_equal(got1[..., 0], (want1 / np.float32(255)).astype(np.float32))


def test_png_srgb_to_linear(oracle, tmp_path):
    img = np.arange(256, dtype=np.int64).reshape(16, 16, 1).repeat(3, axis=2)
    got = _load(oracle, tmp_path, "g.png", imgenc.png(img), {"type": "image_default"})
    want = _srgb_to_linear(img[::-1] / np.float32(255))
    assert np.allclose(got, want, rtol=1e-6, atol=0)  # powf vs numpy: a few ulp


def test_pnm_decode(oracle, tmp_path):
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, size=(9, 7, 3))
    got = _load(oracle, tmp_path, "a.ppm", imgenc.pnm(img), {"type": "image_default", "is_to_linear": False,
                                                              "is_flip_y": False})
    assert np.array_equal(got, (img / np.float32(255)).astype(np.float32))


@pytest.mark.parametrize("rle", [False, True])
def test_hdr_decode(oracle, tmp_path, rle):
    rng = np.random.default_rng(5)
    rgb = rng.lognormal(0, 2, size=(11, 40, 3))
    rgb[3, 5:30] = 0.25  # runs for the run-length coder
    q = imgenc.rgbe(rgb)
    e = q[..., 3:].astype(np.int64)
    want = np.where(e > 0, q[..., :3] * np.ldexp(np.float32(1), e - 136).astype(np.float32), 0).astype(np.float32)
    got = _load(oracle, tmp_path, "a.hdr", imgenc.hdr(rgb, rle), {"type": "image_hdr"})
    assert np.array_equal(got, want)
    got = _load(oracle, tmp_path, "b.hdr", imgenc.hdr(rgb, rle), {"type": "image_hdr", "is_flip_y": True})
    assert np.array_equal(got, want[::-1])


@pytest.mark.parametrize("compression", [0, 1, 2, 3], ids=["none", "rle", "zips", "zip"])
@pytest.mark.parametrize("dtype", [np.float16, np.float32], ids=["half", "float"])
def test_exr_decode(oracle, tmp_path, compression, dtype):
    rng = np.random.default_rng(6)
    h, w = 37, 19
    chans = {k: rng.lognormal(0, 1, size=(h, w)).astype(dtype) for k in "RGB"}
    chans["R"][4:9] = 1.5  # compressible rows
    chans["A"] = np.ones((h, w), dtype)  # ignored channel, sorted first
    data = imgenc.exr(chans, compression, ymin=-3, xmin=2)
    got = _load(oracle, tmp_path, "a.exr", data, {"type": "image_exr"})
    want = np.stack([chans[k].astype(np.float32) for k in "RGB"], axis=2)
    assert got.shape == (h, w, 3) and np.array_equal(got, want)


def test_exr_layers_and_missing_channels(oracle, tmp_path):
    """Channels are matched by the name after the last '.' (image_reader.cpp:133-160);
    a missing one reads 0."""
    h, w = 5, 6
    r = np.full((h, w), 2.0, np.float32)
    b = np.full((h, w), 3.0, np.float32)
    got = _load(oracle, tmp_path, "l.exr", imgenc.exr({"diffuse.R": r, "diffuse.B": b}, 3), {"type": "image_exr"})
    assert (got[..., 0] == 2).all() and (got[..., 1] == 0).all() and (got[..., 2] == 3).all()


def test_exr_writer_round_trip(oracle, tmp_path):
    """The film writer's output reads back through the EXR asset path."""
    from radiantiumplusplus_gb300 import exr as exr_out
    rng = np.random.default_rng(7)
    img = rng.random((8, 12, 3)).astype(np.float32)
    exr_out.write_exr(tmp_path / "f.exr", img)
    assert np.array_equal(oracle.image_load({"type": "image_exr"}, tmp_path / "f.exr"), img)


def test_bad_files_are_reported(oracle, tmp_path):
    (tmp_path / "x.png").write_bytes(b"\x89PNG\r\n\x1a\nnot a png")
    with pytest.raises(RuntimeError):
        oracle.image_load({"type": "image_default"}, tmp_path / "x.png")
    (tmp_path / "y.jpg").write_bytes(b"\xff\xd8\xff\xe0garbage")
    with pytest.raises(RuntimeError, match="jpeg"):
        oracle.image_load({"type": "image_default"}, tmp_path / "y.jpg")
    (tmp_path / "z.gif").write_bytes(b"GIF89a\x01\x00\x01\x00")
    with pytest.raises(RuntimeError, match="unsupported image format"):
        oracle.image_load({"type": "image_default"}, tmp_path / "z.gif")


def _widen(v, bits):
    """An n-bit field widened to 8 bits by repeating its bits (stbi__shiftsigned)."""
    v = np.asarray(v, np.int64)
    if bits >= 8:
        return v & 255
    r, got = np.zeros_like(v), 0
    while got < 8:
        r, got = (r << bits) | v, got + bits
    return r >> (got - 8)


def _expect8(rgb, req):
    rgb = np.asarray(rgb, np.int64)
    if rgb.shape[-1] == 1:
        return np.repeat(rgb, 3, axis=-1) if req == 3 else rgb
    return rgb[..., :3] if req == 3 else _luma(rgb[..., :3])[..., None]


def _check8(oracle, tmp_path, name, data, rgb):
    for req in (3, 1):
        got = _load(oracle, tmp_path, name, data, {"type": "image_default", "channel": req, "is_to_linear": False,
                                                   "is_flip_y": False})
        want = _expect8(rgb, req)
        assert got.shape == want.shape and np.array_equal(got, (want / np.float32(255)).astype(np.float32)), req


BMP_CASES = ["pal1", "pal4", "pal8", "rgb24", "os2_24", "os2_pal8", "rgb555", "rgb565", "argb32", "rgb32_no_alpha",
             "v4_abgr32", "top_down24"]


@pytest.mark.parametrize("case", BMP_CASES)
def test_bmp_decode(oracle, tmp_path, case):
    """BMP through stbi_load: palettes, BGR, masked 16 / 32-bit pixels widened by
    bit replication, OS/2 core headers, bottom-up and top-down rows, 4-byte row
    padding (odd widths)."""
    rng = np.random.default_rng(len(case))
    h, w = 7, 13
    if case.startswith("pal") or case == "os2_pal8":
        bpp = 8 if case == "os2_pal8" else int(case[3:])
        pal = rng.integers(0, 256, size=(1 << bpp, 3))
        idx = rng.integers(0, 1 << bpp, size=(h, w))
        data = imgenc.bmp(idx, bpp, hsz=12 if case.startswith("os2") else 40, palette=pal)
        want = pal[idx]
    elif case in ("rgb24", "os2_24", "top_down24"):
        want = rng.integers(0, 256, size=(h, w, 3))
        data = imgenc.bmp(want, 24, hsz=12 if case == "os2_24" else 40, top_down=case == "top_down24")
    elif case in ("rgb555", "rgb565"):
        g6 = case == "rgb565"
        f = np.stack([rng.integers(0, 32, (h, w)), rng.integers(0, 64 if g6 else 32, (h, w)),
                      rng.integers(0, 32, (h, w))], axis=-1)
        words = (f[..., 0] << (11 if g6 else 10)) | (f[..., 1] << 5) | f[..., 2]
        masks = (0xF800, 0x07E0, 0x001F) if g6 else None
        data = imgenc.bmp(words, 16, masks=masks)
        want = np.stack([_widen(f[..., 0], 5), _widen(f[..., 1], 6 if g6 else 5), _widen(f[..., 2], 5)], axis=-1)
    else:
        c = rng.integers(0, 256, size=(h, w, 4))
        if case == "rgb32_no_alpha":
            c[..., 3] = 0
        if case == "v4_abgr32":
            words = c[..., 0] | (c[..., 1] << 8) | (c[..., 2] << 16) | (c[..., 3] << 24)
            data = imgenc.bmp(words, 32, hsz=108, masks=(0xFF, 0xFF00, 0xFF0000, 0xFF000000))
        else:
            words = (c[..., 3] << 24) | (c[..., 0] << 16) | (c[..., 1] << 8) | c[..., 2]
            data = imgenc.bmp(words, 32)
        want = c[..., :3]
    _check8(oracle, tmp_path, case + ".bmp", data, want)


TGA_CASES = [(2, 24, False), (2, 32, False), (2, 16, False), (3, 8, False), (1, 8, False), (2, 24, True),
             (2, 32, True), (3, 8, True), (1, 8, True)]


@pytest.mark.parametrize("top_down", [False, True])
@pytest.mark.parametrize("kind,bits,rle", TGA_CASES, ids=lambda v: str(v))
def test_tga_decode(oracle, tmp_path, kind, bits, rle, top_down):
    """TGA through stbi_load: true colour (BGR, BGRA, 5-5-5 scaled by 255 / 31),
    grey, colour-mapped, each raw and run-length coded, both row orders."""
    rng = np.random.default_rng(kind * 100 + bits + rle)
    h, w = 6, 11
    runs = rng.integers(0, 3, size=(h, w))  # few distinct values: long runs for the RLE packets
    if kind == 1:
        cmap = rng.integers(0, 256, size=(40, 3))
        idx = (runs * 7 + rng.integers(0, 2, size=(h, w))) % 40
        data = imgenc.tga(idx, 1, 8, rle, top_down, cmap=cmap)
        want = cmap[idx]
    elif kind == 3:
        grey = runs * 60 + 10
        data = imgenc.tga(grey, 3, 8, rle, top_down)
        want = grey[..., None]
    elif bits == 16:
        f = rng.integers(0, 32, size=(h, w, 3))
        words = (f[..., 0] << 10) | (f[..., 1] << 5) | f[..., 2]
        data = imgenc.tga(words, 2, 16, rle, top_down)
        want = f * 255 // 31
    else:
        pal = rng.integers(0, 256, size=(3, bits // 8))
        img = pal[runs]
        data = imgenc.tga(img, 2, bits, rle, top_down)
        want = img[..., :3]
    _check8(oracle, tmp_path, "t.tga", data, want)


@pytest.mark.parametrize("case", ["empty", "truncated"])
def test_tga_bad_colour_map(oracle, tmp_path, case):
    """A colour-mapped TGA whose palette is empty, or cut short by the end of
    the file, is refused with an error instead of read past its end."""
    idx = np.zeros((2, 3), np.int64)
    if case == "empty":
        data = bytearray(imgenc.tga(idx, 1, 8, cmap=np.zeros((0, 3), np.int64)))
    else:
        data = bytearray(imgenc.tga(idx, 1, 8, cmap=np.full((40, 3), 7)))
        data = data[:18 + 10 * 3]  # header, then 10 of the 40 palette entries
    with pytest.raises(RuntimeError, match="colour map"):
        _load(oracle, tmp_path, "bad.tga", bytes(data), {"type": "image_default", "channel": 3,
                                                         "is_to_linear": False, "is_flip_y": False})


def test_hdr_through_image_default(oracle, tmp_path):
    """stbi_load of a Radiance file: (v ^ (1 / 2.2)) * 255 + 0.5 truncated, the grey
    request averaging the three decoded channels first."""
    rng = np.random.default_rng(12)
    rgb = rng.uniform(0.0, 1.5, size=(5, 9, 3))
    data = imgenc.hdr(rgb, rle=False)
    q = imgenc.rgbe(rgb)
    dec = (q[..., :3] * np.ldexp(1.0, q[..., 3:4].astype(int) - 136)).astype(np.float32)
    for req in (3, 1):
        v = dec if req == 3 else ((dec[..., 0] + dec[..., 1] + dec[..., 2]) / np.float32(3))[..., None]
        z = (np.power(v.astype(np.float64), np.float64(np.float32(1.0) / np.float32(2.2))).astype(np.float32) *
             np.float32(255) + np.float32(0.5))
        want = np.clip(z, 0, 255).astype(np.uint8)
        got = _load(oracle, tmp_path, "h.hdr", data, {"type": "image_default", "channel": req, "is_to_linear": False,
                                                      "is_flip_y": False})
        assert np.array_equal(got, (want / np.float32(255)).astype(np.float32)), req
