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
        L.orc_bsdf_sample.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64, P, P, P, P, P]
        L.orc_fresnel_dielectric.argtypes = [ctypes.c_float, ctypes.c_float, P]
        L.orc_fresnel_conductor.argtypes = [ctypes.c_float, P, P, P]
        L.orc_microfacet_d.restype = ctypes.c_float
        L.orc_microfacet_d.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, P]
        L.orc_pcg_u32.restype = ctypes.c_uint32
        L.orc_pcg_u32.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleScene:
    def __init__(self, json_text, base_dir=""):
        L = lib()
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
