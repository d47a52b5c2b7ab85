"""Image encoders for the decoder tests and textured test scenes, written from the
format specifications with Python's zlib: PNG (every colour type and bit depth,
the five row filters, Adam7 interlacing), binary PNM, Radiance RGBE (flat and
run-length), OpenEXR scanline files (NONE / RLE / ZIPS / ZIP; HALF / FLOAT) and
Huffman JPEG (sequential and progressive, any sampling factors, restart
intervals).
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


# ------------------------------------------------------------------- JPEG
# ITU-T T.81 encoder (Huffman; sequential or progressive): the component planes
# are given (already in the colour space to store), transformed by a float DCT,
# quantised and entropy coded with Huffman tables built from the symbol counts
# (T.81 K.2). jpeg() returns the file and the quantised coefficients, so a test
# can reconstruct the samples without entropy decoding.

def _zigzag():
    out = []
    for s in range(15):
        rows = range(max(0, s - 7), min(s, 7) + 1)
        for r in (rows if s % 2 else reversed(rows)):
            out.append(r * 8 + (s - r))
    return np.array(out)


ZIGZAG = _zigzag()  # zigzag index -> row-major index
_DCT = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16)
                  for x in range(8)] for u in range(8)])


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def bits(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):  # pad with 1 bits
        if self.n:
            self.bits((1 << (8 - self.n)) - 1, 8 - self.n)


def _huff_table(freq):
    """Code lengths limited to 16 bits (T.81 K.2) -> (counts[16], symbols, {sym: (code, len)})."""
    import heapq
    syms = [s for s in range(256) if freq[s]]
    if not syms:
        syms = [0]
    # Huffman code lengths with a reserved symbol (frequency 1) that takes the all-ones code
    heap = [(int(freq[s]), i, [s]) for i, s in enumerate(syms)] + [(1, 10 ** 6, [256])]
    heapq.heapify(heap)
    size = {s: 0 for s in syms + [256]}
    tie = 10 ** 6 + 1
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            size[s] += 1
        heapq.heappush(heap, (f1 + f2, tie, a + b))
        tie += 1
    bits = [0] * 40
    for s, l in size.items():
        bits[l] += 1
    i = 39
    while i > 16:
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
        i -= 1
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # the reserved symbol, last of the longest codes
    order = sorted(syms, key=lambda s: (-int(freq[s]), s))
    lens = []
    for l in range(1, 17):
        lens += [l] * bits[l]
    codes, code, k = {}, 0, 0
    for l in range(1, 17):
        for _ in range(bits[l]):
            codes[order[k]] = (code, l)
            code += 1
            k += 1
        code <<= 1
    return bits[1:17], order[:k], codes


def _nbits(a):
    return int(a).bit_length()


def _magnitude_bits(v, s):
    return v if v > 0 else (v - 1) & ((1 << s) - 1)


class _ScanCoder:
    """Emits one scan twice: a counting pass (symbol frequencies) and a writing pass."""

    def __init__(self, dc, ac, w):
        self.dc, self.ac, self.w = dc, ac, w  # dc / ac: {table: codes} or {table: freq array}

    def sym(self, kind, t, s):
        tab = (self.dc if kind == 0 else self.ac)[t]
        if self.w is None:
            tab[s] += 1
        else:
            code, l = tab[s]
            self.w.bits(code, l)

    def raw(self, v, n):
        if self.w is not None and n:
            self.w.bits(v, n)


def _encode_scan(sc, comps, coef, scan, mcux, mcuy, X, Y, hmax, vmax, restart, rst):
    """One scan of the coefficients through coder sc (T.81 G.1.2 for the progressive cases)."""
    ids, ss, se, ah, al, prog = scan
    members = [c for c in comps if c["id"] in ids]
    st = {"eobrun": 0, "be": [], "pred": {c["id"]: 0 for c in members}}

    def flush_eob(t):
        if st["eobrun"]:
            n = _nbits(st["eobrun"]) - 1
            sc.sym(1, t, n << 4)
            sc.raw(st["eobrun"] - (1 << n), n)
            for b in st["be"]:
                sc.raw(b, 1)
            st["eobrun"], st["be"] = 0, []

    def block(c, blk):
        d = coef[c["id"]][blk]
        if not prog:  # sequential
            diff = int(d[0]) - st["pred"][c["id"]]
            st["pred"][c["id"]] = int(d[0])
            s = _nbits(abs(diff))
            sc.sym(0, c["td"], s)
            sc.raw(_magnitude_bits(diff, s), s)
            r = 0
            for k in range(1, 64):
                v = int(d[ZIGZAG[k]])
                if v == 0:
                    r += 1
                    continue
                while r > 15:
                    sc.sym(1, c["ta"], 0xF0)
                    r -= 16
                s = _nbits(abs(v))
                sc.sym(1, c["ta"], (r << 4) | s)
                sc.raw(_magnitude_bits(v, s), s)
                r = 0
            if r:
                sc.sym(1, c["ta"], 0)
            return
        if ss == 0:  # DC scans
            v = int(d[0]) >> al
            if ah == 0:
                diff = v - st["pred"][c["id"]]
                st["pred"][c["id"]] = v
                s = _nbits(abs(diff))
                sc.sym(0, c["td"], s)
                sc.raw(_magnitude_bits(diff, s), s)
            else:
                sc.raw(v & 1, 1)
            return
        t = c["ta"]
        if ah == 0:  # first AC scan of the band
            r = 0
            for k in range(ss, se + 1):
                v = int(d[ZIGZAG[k]])
                a = abs(v) >> al
                if a == 0:
                    r += 1
                    continue
                flush_eob(t)
                while r > 15:
                    sc.sym(1, t, 0xF0)
                    r -= 16
                s = _nbits(a)
                sc.sym(1, t, (r << 4) | s)
                sc.raw(_magnitude_bits(a if v > 0 else -a, s), s)
                r = 0
            if r:
                st["eobrun"] += 1
                if st["eobrun"] == 0x7FFF:
                    flush_eob(t)
            return
        absv = [abs(int(d[ZIGZAG[k]])) >> al for k in range(ss, se + 1)]
        eob = max([i for i, a in enumerate(absv) if a == 1], default=-1)
        r, br = 0, []
        for i, a in enumerate(absv):
            if a == 0:
                r += 1
                continue
            while r > 15 and i <= eob:
                flush_eob(t)
                sc.sym(1, t, 0xF0)
                r -= 16
                for b in br:
                    sc.raw(b, 1)
                br = []
            if a > 1:
                br.append(a & 1)
                continue
            flush_eob(t)
            sc.sym(1, t, (r << 4) | 1)
            sc.raw(1 if int(d[ZIGZAG[ss + i]]) > 0 else 0, 1)
            for b in br:
                sc.raw(b, 1)
            br, r = [], 0
        if r or br:
            st["eobrun"] += 1
            st["be"] += br
            if st["eobrun"] == 0x7FFF or len(st["be"]) > 900:
                flush_eob(t)

    units = []
    if len(members) == 1:
        c = members[0]
        cx, cy = -(-X * c["h"] // hmax), -(-Y * c["v"] // vmax)
        for j in range(-(-cy // 8)):
            for i in range(-(-cx // 8)):
                units.append([(c, (j, i))])
    else:
        for j in range(mcuy):
            for i in range(mcux):
                units.append([(c, (j * c["v"] + y, i * c["h"] + x)) for c in members
                              for y in range(c["v"]) for x in range(c["h"])])
    ac_t = members[0]["ta"]
    for u, unit in enumerate(units):
        if restart and u and u % restart == 0:
            flush_eob(ac_t)
            rst(u // restart - 1)
            st["pred"] = {c["id"]: 0 for c in members}
        for c, blk in unit:
            block(c, blk)
    flush_eob(ac_t)


def jpeg(planes, sampling, quant, X, Y, ids=None, scans=None, restart=0, app=(), qtab=None, seed=0):
    """planes: per component a float array (Y x X, 0..255 samples at full
    resolution; subsampled components are box-averaged). sampling: (h, v) per
    component. quant: per component a 64-entry table (row-major). scans: None for
    one interleaved sequential scan, a list of component-id tuples for
    sequential scans of those components, or progressive scans
    (ids, Ss, Se, Ah, Al). Returns (file bytes, {component id: coefficient
    blocks (by, bx, 64) row-major int}, component records)."""
    nc = len(planes)
    ids = ids or list(range(1, nc + 1))
    hmax = max(h for h, _ in sampling)
    vmax = max(v for _, v in sampling)
    mcux, mcuy = -(-X // (8 * hmax)), -(-Y // (8 * vmax))
    comps, coef = [], {}
    qtables = []
    for k in range(nc):
        h, v = sampling[k]
        q = np.asarray(quant[k], dtype=np.int64).reshape(64)
        tq = next((i for i, t in enumerate(qtables) if np.array_equal(t, q)), None)
        if tq is None:
            tq = len(qtables)
            qtables.append(q)
        c = {"id": ids[k], "h": h, "v": v, "tq": tq, "td": min(k, 1), "ta": min(k, 1)}
        comps.append(c)
        fx, fy = hmax // h, vmax // v
        pw, ph = mcux * 8 * hmax, mcuy * 8 * vmax
        full = np.pad(np.asarray(planes[k], np.float64), ((0, ph - Y), (0, pw - X)), mode="edge")
        sub = full.reshape(ph // fy, fy, pw // fx, fx).mean(axis=(1, 3))
        cx, cy = -(-X * h // hmax), -(-Y * v // vmax)
        # samples past the component's own size repeat its edge (as encoders pad)
        sub[:, cx:] = sub[:, cx - 1:cx]
        sub[cy:, :] = sub[cy - 1:cy, :]
        blocks = sub.reshape(ph // fy // 8, 8, pw // fx // 8, 8).transpose(0, 2, 1, 3) - 128.0
        f = np.einsum("ux,abxy,vy->abuv", _DCT, blocks, _DCT)  # [by, bx, vertical u, horizontal v]
        coef[c["id"]] = np.round(f.reshape(f.shape[0], f.shape[1], 64) / q).astype(np.int64)
    progressive = scans is not None and len(scans[0]) == 5
    if scans is None:
        scans = [tuple(ids)]
    full_scans = []
    for s in scans:
        if progressive:
            full_scans.append((tuple(s[0]), s[1], s[2], s[3], s[4], True))
        else:
            full_scans.append((tuple(s), 0, 63, 0, 0, False))
    out = bytearray(b"\xff\xd8")
    for a in app:
        out += a
    for t, q in enumerate(qtables):
        sixteen = int(q.max() > 255)
        body = bytes([(sixteen << 4) | t]) + b"".join(
            (int(q[ZIGZAG[i]]).to_bytes(2, "big") if sixteen else bytes([int(q[ZIGZAG[i]])])) for i in range(64))
        out += b"\xff\xdb" + struct.pack(">H", 2 + len(body)) + body
    sof = bytes([8]) + struct.pack(">HHB", Y, X, nc) + b"".join(
        bytes([c["id"], (c["h"] << 4) | c["v"], c["tq"]]) for c in comps)
    out += (b"\xff\xc2" if progressive else b"\xff\xc0") + struct.pack(">H", 2 + len(sof)) + sof
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    for scan in full_scans:
        sid = scan[0]
        members = [c for c in comps if c["id"] in sid]
        # counting pass: symbol frequencies per table
        fdc = {c["td"]: np.zeros(257, np.int64) for c in members}
        fac = {c["ta"]: np.zeros(257, np.int64) for c in members}
        _encode_scan(_ScanCoder(fdc, fac, None), comps, coef, scan, mcux, mcuy, X, Y, hmax, vmax, restart,
                     lambda m: None)
        need_dc = scan[1] == 0 and scan[3] == 0
        need_ac = scan[2] > 0
        dht = b""
        cdc, cac = {}, {}
        for t, fr in fdc.items():
            if need_dc:
                counts, order, cdc[t] = _huff_table(fr)
                dht += bytes([t]) + bytes(counts) + bytes(order)
        for t, fr in fac.items():
            if need_ac:
                counts, order, cac[t] = _huff_table(fr)
                dht += bytes([0x10 | t]) + bytes(counts) + bytes(order)
        if dht:
            out += b"\xff\xc4" + struct.pack(">H", 2 + len(dht)) + dht
        sos = bytes([len(members)]) + b"".join(bytes([c["id"], (c["td"] << 4) | c["ta"]]) for c in members)
        sos += bytes([scan[1], scan[2], (scan[3] << 4) | scan[4]])
        out += b"\xff\xda" + struct.pack(">H", 2 + len(sos)) + sos
        w = _BitWriter()

        def rst(m, w=w):
            w.flush()
            w.out += bytes([0xFF, 0xD0 + (m & 7)])

        _encode_scan(_ScanCoder(cdc, cac, w), comps, coef, scan, mcux, mcuy, X, Y, hmax, vmax, restart, rst)
        w.flush()
        out += w.out
    out += b"\xff\xd9"
    qt = {c["id"]: qtables[c["tq"]] for c in comps}
    return bytes(out), coef, comps, qt


# -------------------------------------------------------------- BMP / TGA
def bmp(img, bpp=24, hsz=40, masks=None, palette=None, top_down=False, compress=None):
    """img: (h, w) palette indices for bpp <= 8, else (h, w, 3|4) raw field values
    for 16 / 32 bits (packed with `masks` (r, g, b[, a]) or the defaults) or RGB
    bytes for 24. hsz 12 writes the OS/2 core header (3-byte palette entries)."""
    h, w = img.shape[:2]
    rows = []
    for y in (range(h) if top_down else range(h - 1, -1, -1)):
        r = img[y]
        if bpp <= 8:
            bits = "".join(format(int(v), "0%db" % bpp) for v in r)
            bits += "0" * (-len(bits) % 8)
            row = bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))
        elif bpp == 24:
            row = bytes(int(c) for px in r for c in (px[2], px[1], px[0]))
        else:
            row = b"".join(int(v).to_bytes(bpp // 8, "little") for v in r)
        rows.append(row + b"\0" * (-len(row) % 4))
    pix = b"".join(rows)
    pal = b""
    if palette is not None:
        pal = b"".join(bytes([int(c[2]), int(c[1]), int(c[0])]) + (b"" if hsz == 12 else b"\0") for c in palette)
    if compress is None:
        compress = 3 if masks is not None else 0
    if hsz == 12:
        hdr = struct.pack("<IHHHH", 12, w, h, 1, bpp)
    else:
        hdr = struct.pack("<IiiHHIIiiII", hsz, w, -h if top_down else h, 1, bpp, compress, len(pix), 2835, 2835, 0, 0)
        m = list(masks or (0, 0, 0)) + [0] * 4
        if hsz >= 56:
            hdr += struct.pack("<IIII", *m[:4])
        hdr += b"\0" * (hsz - len(hdr))
    extra = struct.pack("<III", *m[:3]) if (hsz == 40 and compress == 3) else b""
    off = 14 + len(hdr) + len(extra) + len(pal)
    return b"BM" + struct.pack("<IHHI", off + len(pix), 0, 0, off) + hdr + extra + pal + pix


def tga(img, kind, bits, rle=False, top_down=False, cmap=None, cmap_bits=24, first=0):
    """kind 1 (colour-mapped: img = (h, w) indices), 2 (true colour: img = (h, w,
    3|4) RGB(A) bytes, or (h, w) 16-bit 5-5-5 words for bits 15 / 16), 3 (grey)."""
    h, w = img.shape[:2]

    def px(v):
        if kind == 1:
            return int(v).to_bytes(bits // 8, "little")
        if kind == 3:
            return bytes([int(v)])
        if bits in (15, 16):
            return int(v).to_bytes(2, "little")
        c = [int(x) for x in v]
        return bytes([c[2], c[1], c[0]] + c[3:])

    order = range(h) if top_down else range(h - 1, -1, -1)
    flat = [px(img[y][x]) for y in order for x in range(w)]
    if rle:  # alternate repeat and raw packets of up to 128 pixels
        out, i = [], 0
        while i < len(flat):
            j = i
            while j + 1 < len(flat) and flat[j + 1] == flat[i] and j - i < 127:
                j += 1
            if j > i:
                out.append(bytes([0x80 | (j - i)]) + flat[i])
                i = j + 1
            else:
                k = i
                while k + 1 < len(flat) and flat[k + 1] != flat[k] and k - i < 127:
                    k += 1
                out.append(bytes([k - i]) + b"".join(flat[i:k + 1]))
                i = k + 1
        data = b"".join(out)
    else:
        data = b"".join(flat)
    cm = b""
    if cmap is not None:
        for c in cmap:
            cm += (int(c).to_bytes(2, "little") if cmap_bits in (15, 16) else
                   bytes([int(c[2]), int(c[1]), int(c[0])] + [int(x) for x in c[3:]]))
    typ = kind + (8 if rle else 0)
    hdr = struct.pack("<BBBHHBHHHHBB", 0, 1 if cmap is not None else 0, typ, first,
                      len(cmap) if cmap is not None else 0, cmap_bits if cmap is not None else 0, 0, 0, w, h, bits,
                      0x20 if top_down else 0)
    return hdr + cm + data
