"""Image encoders for the decoder tests and textured test scenes, written from the
format specifications with Python's zlib: PNG (every colour type and bit depth,
the five row filters, Adam7 interlacing), binary PNM, Radiance RGBE (flat and
run-length) and OpenEXR scanline files (NONE / RLE / ZIPS / ZIP; HALF / FLOAT).
"""
import struct
import zlib

import numpy as np

_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(t, d):
    return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_rows(rows, bpp, filters):
    out = b""
    prev = bytes(len(rows[0])) if rows else b""
    for y, row in enumerate(rows):
        f = filters[y % len(filters)]
        enc = bytearray(len(row))
        for i in range(len(row)):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
            enc[i] = (row[i] - pred) & 0xFF
        out += bytes([f]) + bytes(enc)
        prev = row
    return out


def _pack_row(samples, depth):
    """samples: 1-D int array of one row's samples -> bytes at `depth` bits each."""
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    if depth == 16:
        return samples.astype(">u2").tobytes()
    bits = "".join(format(int(v), "0%db" % depth) for v in samples)
    bits += "0" * (-len(bits) % 8)
    return bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))


def png(img, depth=8, colour=None, palette=None, filters=(0, 1, 2, 3, 4), interlace=False, level=6):
    """img: (h, w, c) integer samples (c = 1, 2, 3, 4; palette indices for colour 3)."""
    img = np.asarray(img)
    h, w, c = img.shape
    if colour is None:
        colour = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    bpp = max(1, c * depth // 8)

    def image_bytes(sub):
        sh, sw = sub.shape[:2]
        rows = [_pack_row(sub[y].reshape(-1), depth) for y in range(sh)]
        return _filter_rows(rows, bpp, filters)

    if not interlace:
        raw = image_bytes(img)
    else:
        raw = b""
        for x0, y0, dx, dy in _ADAM7:
            sub = img[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += image_bytes(sub)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, colour, 0, 0, int(interlace)))
    if palette is not None:
        data += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    return data + _chunk(b"IDAT", zlib.compress(raw, level)) + _chunk(b"IEND", b"")


def pnm(img):
    img = np.asarray(img, np.uint8)
    h, w, c = img.shape
    return (b"P6" if c == 3 else b"P5") + b"\n# test image\n%d %d\n255\n" % (w, h) + img.tobytes()


def rgbe(rgb):
    """float (h, w, 3) -> RGBE bytes (h, w, 4), the Radiance mantissa / exponent split."""
    rgb = np.asarray(rgb, np.float64)
    m = rgb.max(axis=2)
    out = np.zeros(rgb.shape[:2] + (4,), np.uint8)
    nz = m >= 1e-32
    e = np.zeros_like(m, dtype=np.int64)
    frac, ex = np.frexp(m[nz])
    e[nz] = ex
    scale = np.zeros_like(m)
    scale[nz] = frac * 256.0 / m[nz]
    out[..., :3] = np.where(nz[..., None], np.floor(rgb * scale[..., None]), 0).astype(np.uint8)
    out[..., 3] = np.where(nz, e + 128, 0).astype(np.uint8)
    return out


def hdr(rgb, rle=True):
    q = rgbe(rgb)
    h, w, _ = q.shape
    data = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (h, w)
    if not rle:
        return data + q.tobytes()
    for y in range(h):
        data += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            ch = q[y, :, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and ch[x + run] == ch[x]:
                    run += 1
                if run >= 3:
                    data += bytes([128 + run, int(ch[x])])
                    x += run
                else:
                    n = 1
                    while x + n < w and n < 128 and not (x + n + 2 < w and ch[x + n] == ch[x + n + 1] == ch[x + n + 2]):
                        n += 1
                    data += bytes([n]) + ch[x:x + n].tobytes()
                    x += n
    return data


def _exr_attr(name, typ, data):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data


def _exr_predict(raw):
    """OpenEXR ZIP / RLE preprocessing: interleave halves, then byte deltas + 128."""
    n = len(raw)
    t = bytearray(n)
    t[0:(n + 1) // 2] = raw[0::2]
    t[(n + 1) // 2:] = raw[1::2]
    out = bytearray(n)
    if n:
        out[0] = t[0]
    for i in range(1, n):
        out[i] = (t[i] - t[i - 1] + 128 + 256) & 0xFF
    return bytes(out)


def _exr_rle(data):
    out = b""
    i, n = 0, len(data)
    while i < n:
        run = 1
        while i + run < n and run < 128 and data[i + run] == data[i]:
            run += 1
        if run >= 3:
            out += struct.pack("b", run - 1) + data[i:i + 1]
            i += run
        else:
            j = i
            while j < n and j - i < 127 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
                j += 1
            j = max(j, i + 1)
            out += struct.pack("b", -(j - i)) + data[i:j]
            i = j
    return out


def exr(channels, compression=0, ymin=0, xmin=0):
    """channels: dict name -> (h, w) array, float16 or float32; compression 0 NONE,
    1 RLE, 2 ZIPS, 3 ZIP. Channels are stored sorted by name, as OpenEXR does."""
    names = sorted(channels)
    h, w = channels[names[0]].shape
    chl = b""
    for nme in names:
        typ = 1 if channels[nme].dtype == np.float16 else 2
        chl += nme.encode() + b"\0" + struct.pack("<iB3xii", typ, 0, 1, 1)
    chl += b"\0"
    box = struct.pack("<iiii", xmin, ymin, xmin + w - 1, ymin + h - 1)
    header = (b"\x76\x2f\x31\x01" + struct.pack("<I", 2) + _exr_attr("channels", "chlist", chl)
              + _exr_attr("compression", "compression", bytes([compression]))
              + _exr_attr("dataWindow", "box2i", box) + _exr_attr("displayWindow", "box2i", box)
              + _exr_attr("lineOrder", "lineOrder", b"\0")
              + _exr_attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + _exr_attr("screenWindowCenter", "v2f", struct.pack("<ff", 0, 0))
              + _exr_attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    lines = 16 if compression == 3 else 1
    chunks = []
    for y0 in range(0, h, lines):
        raw = b""
        for y in range(y0, min(h, y0 + lines)):
            for nme in names:
                a = channels[nme]
                raw += a[y].astype("<f2" if a.dtype == np.float16 else "<f4").tobytes()
        if compression == 0:
            data = raw
        else:
            pre = _exr_predict(raw)
            data = _exr_rle(pre) if compression == 1 else zlib.compress(pre)
            if len(data) >= len(raw):
                data = raw
        chunks.append(struct.pack("<ii", ymin + y0, len(data)) + data)
    offs, pos = [], len(header) + 8 * len(chunks)
    for c in chunks:
        offs.append(pos)
        pos += len(c)
    return header + b"".join(struct.pack("<Q", o) for o in offs) + b"".join(chunks)
