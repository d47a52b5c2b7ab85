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
