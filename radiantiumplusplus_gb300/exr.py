"""Film output: uncompressed scanline OpenEXR (RGB fp32) and sRGB PNG.

SampleRenderer::SaveResult writes the film as an RGB fp32 EXR through
ImageReader::WriteExr (rad.offline/src/renderer/sample_renderer.cpp:34-46,
rad.core/src/image_reader.cpp:230-255). OpenEXR is not available here, so this
writes the format directly: single-part scanline file, NO_COMPRESSION, channels
B, G, R as FLOAT. The PNG preview applies Color24f::ToSRGB
(rad.core/include/rad/core/color.h:47-52).
"""

from __future__ import annotations

import struct
import zlib

import numpy as np

__all__ = ["write_exr", "read_exr", "to_srgb", "write_png"]


def _attr(name, typ, data):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data


def write_exr(path, rgb):
    """Write an (H, W, 3) float32 image as an uncompressed scanline EXR."""
    img = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w, _ = img.shape
    chl = b""
    for c in (b"B", b"G", b"R"):
        chl += c + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1)
    chl += b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (
        b"\x76\x2f\x31\x01" + struct.pack("<I", 2)
        + _attr("channels", "chlist", chl)
        + _attr("compression", "compression", b"\0")
        + _attr("dataWindow", "box2i", box)
        + _attr("displayWindow", "box2i", box)
        + _attr("lineOrder", "lineOrder", b"\0")
        + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
        + _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
        + _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
        + b"\0"
    )
    line_bytes = w * 4 * 3
    block = 8 + line_bytes
    first = len(header) + 8 * h
    offsets = struct.pack("<%dQ" % h, *[first + y * block for y in range(h)])
    with open(path, "wb") as fh:
        fh.write(header)
        fh.write(offsets)
        for y in range(h):
            fh.write(struct.pack("<ii", y, line_bytes))
            row = img[y]
            fh.write(row[:, 2].astype("<f4").tobytes())
            fh.write(row[:, 1].astype("<f4").tobytes())
            fh.write(row[:, 0].astype("<f4").tobytes())
    return path


def read_exr(path):
    """Read back a file written by :func:`write_exr` -> (H, W, 3) float32."""
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:4] != b"\x76\x2f\x31\x01":
        raise ValueError("not an OpenEXR file")
    pos = 8
    w = h = None
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        size = struct.unpack("<i", data[tend + 1:tend + 5])[0]
        val = data[tend + 5:tend + 5 + size]
        if name == "dataWindow":
            x0, y0, x1, y1 = struct.unpack("<iiii", val)
            w, h = x1 - x0 + 1, y1 - y0 + 1
        pos = tend + 5 + size
    pos += 1 + 8 * h
    img = np.empty((h, w, 3), dtype=np.float32)
    for _ in range(h):
        y, n = struct.unpack("<ii", data[pos:pos + 8])
        pos += 8
        row = np.frombuffer(data[pos:pos + n], dtype="<f4").reshape(3, w)
        img[y, :, 2], img[y, :, 1], img[y, :, 0] = row[0], row[1], row[2]
        pos += n
    return img


def to_srgb(rgb):
    """Color24f::ToSRGB: 12.92 v below 0.0031308, else 1.055 v^(1/2.4) - 0.055."""
    v = np.asarray(rgb, dtype=np.float32)
    return np.where(v <= 0.0031308, 12.92 * v, (1.0 + 0.055) * np.power(np.maximum(v, 0), 1.0 / 2.4) - 0.055)


def write_png(path, rgb):
    a = (np.clip(to_srgb(rgb), 0, 1) * 255 + 0.5).astype(np.uint8)
    h, w, _ = a.shape
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                 + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
    return path
