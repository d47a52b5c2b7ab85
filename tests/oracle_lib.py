"""ctypes loader for the CPU oracle (oracle/liboracle.so) -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_scene_load.restype = P
        L.orc_scene_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.orc_scene_free.argtypes = [P]
        L.orc_scene_info.argtypes = [P, P]
        L.orc_trace.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int]
        L.orc_camera_rays.argtypes = [P, P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, P]
        L.orc_render.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, P, P]
        L.orc_render_samples.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_uint32, P]
        L.orc_bsdf_eval.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64, P, P]
        L.orc_texture_eval.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_int64, P]
        L.orc_render_particle.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_int, P]
        L.orc_render_bdpt.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_uint32, ctypes.c_int, P]
        L.orc_render_bdpt.restype = ctypes.c_int64
        L.orc_texture_count.argtypes = [P]
        L.orc_image_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P, P, ctypes.c_int64]
        L.orc_bsdf_sample.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64, P, P, P, P, P]
        L.orc_fresnel_dielectric.argtypes = [ctypes.c_float, ctypes.c_float, P]
        L.orc_fresnel_conductor.argtypes = [ctypes.c_float, P, P, P]
        L.orc_microfacet_d.restype = ctypes.c_float
        L.orc_microfacet_d.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, P]
        L.orc_pcg_u32.restype = ctypes.c_uint32
        L.orc_pcg_u32.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        L.orc_guide_level_res.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P]
        L.orc_guide_forward.argtypes = [ctypes.c_uint32, P, P, P, ctypes.c_float, ctypes.c_float, P, P,
                                        ctypes.c_int64, P, P, ctypes.c_int]
        L.orc_guide_grad.restype = ctypes.c_double
        L.orc_guide_grad.argtypes = [ctypes.c_uint32, P, P, P, ctypes.c_float, ctypes.c_float, P, P,
                                     ctypes.c_int64, P, ctypes.c_int]
        L.orc_guide_mix_pdf.argtypes = [P, P, ctypes.c_int64, P]
        L.orc_half_round.restype = ctypes.c_float
        L.orc_half_round.argtypes = [ctypes.c_float]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleScene:
    def __init__(self, json_text, base_dir=""):
        L = lib()
        self.json_text, self.base_dir = json_text, base_dir
        self.h = L.orc_scene_load(json_text.encode(), base_dir.encode())
        if not self.h:
            raise RuntimeError(L.orc_last_error().decode())
        info = np.zeros(10, dtype=np.int64)
        L.orc_scene_info(self.h, _p(info))
        (self.width, self.height, self.spp, self.seed, self.max_depth, self.rr_depth,
         self.n_shapes, self.n_prims, self.n_lights, self.is_vol) = [int(x) for x in info]

    @classmethod
    def from_file(cls, path):
        with open(path) as fh:
            return cls(fh.read(), os.path.dirname(os.path.abspath(path)))

    def close(self):
        if self.h:
            lib().orc_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, rays, any_hit=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        hits = np.zeros((n, 5), dtype=np.float32)
        lib().orc_trace(self.h, _p(rays), n, _p(hits), 1 if any_hit else 0)
        return hits

    def camera_rays(self, pixels, sample=0, seed=None):
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        out = np.zeros((pixels.shape[0], 8), dtype=np.float32)
        lib().orc_camera_rays(self.h, _p(pixels), pixels.shape[0], sample, self.seed if seed is None else seed,
                              _p(out))
        return out

    def render(self, rows=None, samples=None, seed=None, threads=0):
        W, H = self.width, self.height
        r0, r1, rs = rows if rows is not None else (0, H, 1)
        s0, s1 = samples if samples is not None else (0, self.spp)
        film = np.zeros((H, W, 3), dtype=np.float32)
        stats = np.zeros(4, dtype=np.uint64)
        rc = lib().orc_render(self.h, r0, r1, rs, s0, s1, -1 if seed is None else seed, threads, _p(film),
                              _p(stats))
        if rc != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return film, stats

    def render_particle(self, spp=None, first=0, count=None, seed=None, threads=1):
        """particle_tracer film: light paths [first, first + count) of a job of `spp` light paths
        (threads 0: all host threads; the sum order then depends on the split)."""
        spp = self.spp if spp is None else spp
        count = spp - first if count is None else count
        film = np.zeros((self.height, self.width, 3), np.float32)
        if lib().orc_render_particle(self.h, first, count, spp, self.seed if seed is None else seed, threads,
                                     _p(film)) != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return film

    def render_bdpt(self, samples=None, seed=None, threads=0, rows=None, count=False):
        """bdpt film: per pixel (valid camera-side samples + t = 1 splats landing there) / spp.
        rows = (row0, row1, step) renders a subset of the pixels; count=True also returns the samples run."""
        s0, s1 = samples if samples is not None else (0, self.spp)
        r0, r1, rs = rows if rows is not None else (0, self.height, 1)
        film = np.zeros((self.height, self.width, 3), np.float32)
        n = lib().orc_render_bdpt(self.h, r0, r1, rs, s0, s1, self.seed if seed is None else seed, threads, _p(film))
        if n < 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return (film, n) if count else film

    def texture_count(self):
        return lib().orc_texture_count(self.h)

    def texture_eval(self, texture, uv, duv=None):
        uv = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
        n = uv.shape[0]
        duv = np.zeros((n, 4), np.float32) if duv is None else np.ascontiguousarray(duv, dtype=np.float32)
        out = np.zeros((n, 3), dtype=np.float32)
        if lib().orc_texture_eval(self.h, texture, _p(uv), _p(duv), n, _p(out)) != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return out

    def render_samples(self, pixels, samples, seed=None):
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        samples = np.ascontiguousarray(samples, dtype=np.uint32)
        out = np.zeros((pixels.shape[0], 3), dtype=np.float32)
        rc = lib().orc_render_samples(self.h, _p(pixels), _p(samples), pixels.shape[0],
                                      self.seed if seed is None else seed, _p(out))
        if rc != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return out


def bsdf_eval(bsdf_json, wi, wo):
    wi = np.ascontiguousarray(wi, dtype=np.float32)
    wo = np.ascontiguousarray(wo, dtype=np.float32)
    n = wi.shape[0]
    f = np.zeros((n, 3), dtype=np.float32)
    pdf = np.zeros(n, dtype=np.float32)
    if lib().orc_bsdf_eval(bsdf_json.encode(), _p(wi), _p(wo), n, _p(f), _p(pdf)) != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return f, pdf


def bsdf_sample(bsdf_json, wi, u):
    wi = np.ascontiguousarray(wi, dtype=np.float32)
    u = np.ascontiguousarray(u, dtype=np.float32)
    n = wi.shape[0]
    wo = np.zeros((n, 3), dtype=np.float32)
    pdf = np.zeros(n, dtype=np.float32)
    f = np.zeros((n, 3), dtype=np.float32)
    eta = np.zeros(n, dtype=np.float32)
    typ = np.zeros(n, dtype=np.uint32)
    if lib().orc_bsdf_sample(bsdf_json.encode(), _p(wi), _p(u), n, _p(wo), _p(pdf), _p(f), _p(eta), _p(typ)) != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return wo, pdf, f, eta, typ


# ---------------------------------------------------------------- guide network
GUIDE_LEVELS = 16
GUIDE_NW = 64 * 48 + 64 * 64 * 2 + 48 * 64


class OracleGuide:
    """CPU guide network with the GPU library's layout (table then MLP weights)."""

    def __init__(self, log2t, lo, hi, params, min_res=16, max_res=512, log_kappa_max=5.0, c_max=0.6):
        self.log2t = int(log2t)
        self.log_kappa_max = float(log_kappa_max)
        self.c_max = float(c_max)
        self.res = np.zeros(GUIDE_LEVELS, dtype=np.uint32)
        lib().orc_guide_level_res(min_res, max_res, _p(self.res))
        self.lo = np.asarray(lo, dtype=np.float32)
        hi = np.asarray(hi, dtype=np.float32)
        ext = hi - self.lo
        self.inv = np.where(ext > 1e-6, np.float32(1.0) / np.maximum(ext, np.float32(1e-30)), 1.0).astype(np.float32)
        self.params = np.ascontiguousarray(params, dtype=np.float32)
        self.n_table = GUIDE_LEVELS * (1 << self.log2t) * 2
        assert self.params.size == self.n_table + GUIDE_NW

    def forward(self, queries, exact=False):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        raw = np.zeros((q.shape[0], 48), dtype=np.float32)
        mix = np.zeros((q.shape[0], 44), dtype=np.float32)
        lib().orc_guide_forward(self.log2t, _p(self.res), _p(self.lo), _p(self.inv), self.log_kappa_max,
                                self.c_max, _p(self.params), _p(q),
                                q.shape[0], _p(raw), _p(mix), 1 if exact else 0)
        return raw, mix

    def grad(self, records, exact=False):
        r = np.ascontiguousarray(records, dtype=np.float32)
        g = np.zeros(self.params.size, dtype=np.float64)
        loss = lib().orc_guide_grad(self.log2t, _p(self.res), _p(self.lo), _p(self.inv), self.log_kappa_max,
                                    self.c_max, _p(self.params), _p(r),
                                    r.shape[0], _p(g), 1 if exact else 0)
        return g, loss


def guide_mix_pdf(mix, dirs):
    m = np.ascontiguousarray(mix, dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.zeros(m.shape[0], dtype=np.float64)
    lib().orc_guide_mix_pdf(_p(m), _p(d), m.shape[0], _p(out))
    return out


def guide_checkpoint(log2t, lo, hi, params, min_res=16, max_res=512, step=0):
    """Bytes of a version-1 guide checkpoint holding `params` and zero Adam moments."""
    import struct
    res = np.zeros(GUIDE_LEVELS, dtype=np.uint32)
    lib().orc_guide_level_res(min_res, max_res, _p(res))
    n = int(np.asarray(params).size)
    hd = b"RADGUID1" + struct.pack("<6I", 1, log2t, GUIDE_LEVELS, min_res, max_res, step)
    hd += struct.pack("<Q", n) + struct.pack("<3f", *lo) + struct.pack("<3f", *hi) + res.astype("<u4").tobytes()
    assert len(hd) == 128
    p = np.ascontiguousarray(params, dtype="<f4").tobytes()
    return hd + p + bytes(2 * len(p))


def guide_random_params(log2t, seed, table_scale=0.5, weight_scale=1.0):
    """Seeded parameters with non-trivial hash-grid features (unlike the +-1e-4 initialisation)."""
    rng = np.random.default_rng(seed)
    n_table = GUIDE_LEVELS * (1 << log2t) * 2
    table = rng.uniform(-table_scale, table_scale, n_table)
    w = np.concatenate([
        rng.uniform(-1, 1, 64 * 48) * np.sqrt(6 / 48),
        rng.uniform(-1, 1, 64 * 64) * np.sqrt(6 / 64),
        rng.uniform(-1, 1, 64 * 64) * np.sqrt(6 / 64),
        rng.uniform(-1, 1, 48 * 64) * np.sqrt(6 / 64) * 0.5,
    ]) * weight_scale
    w[64 * 48 + 2 * 64 * 64 + 41 * 64:] = 0.0  # unused output rows
    return np.concatenate([table, w]).astype(np.float32)


def guide_random_queries(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    P = rng.uniform(lo, hi, size=(n, 3))
    N = rng.normal(size=(n, 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    return np.concatenate([P, N, wo], axis=1).astype(np.float32)


def guide_random_records(n, lo, hi, seed, w_max=2.0):
    """Records (n, 16): P, p_bsdf | N, 0 | wo, 0 | wi, weight."""
    rng = np.random.default_rng(seed + 1)
    q = guide_random_queries(n, lo, hi, seed)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    b = rng.uniform(0.01, 1.0, n)
    w = rng.uniform(0.0, w_max, n)
    rec = np.zeros((n, 16), dtype=np.float32)
    rec[:, 0:3], rec[:, 3] = q[:, 0:3], b
    rec[:, 4:7] = q[:, 3:6]
    rec[:, 8:11] = q[:, 6:9]
    rec[:, 12:15], rec[:, 15] = wi, w
    return rec


def image_load(asset, path):
    """An image asset decoded and converted as the bitmap texture sees it -> (h, w, c) float32."""
    import json as _json
    dims = np.zeros(3, np.int32)
    js = _json.dumps(asset).encode()
    if lib().orc_image_load(js, str(path).encode(), _p(dims), None, 0) != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    w, h, c = (int(x) for x in dims)
    px = np.zeros(w * h * c, np.float32)
    if lib().orc_image_load(js, str(path).encode(), _p(dims), _p(px), px.size) != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return px.reshape(h, w, c)
