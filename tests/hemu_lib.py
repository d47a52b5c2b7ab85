"""ctypes binding of the host-emulation harness (tests/hostemu/libhemu.so):
the renderer's device code and kernels compiled for the host. Test
infrastructure only: it lets the CPU tests compare the device algorithm with
the oracle bit for bit, with the same libm on both sides."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DIR = os.path.join(HERE, "hostemu")
PATH = os.path.join(DIR, "libhemu.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", DIR], check=True)
        L = ctypes.CDLL(PATH)
        P = ctypes.c_void_p
        L.hemu_last_error.restype = ctypes.c_char_p
        L.hemu_scene_load.restype = P
        L.hemu_scene_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.hemu_scene_free.argtypes = [P]
        L.hemu_camera_rays.argtypes = [P, P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, P]
        L.hemu_trace.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int, ctypes.c_int]
        L.hemu_bsdf_eval.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64, P, P]
        L.hemu_bsdf_sample.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64, P, P, P, P, P]
        L.hemu_render_samples.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, P]
        L.hemu_render_mixed.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, P, P]
        L.hemu_set_nudge.argtypes = [ctypes.c_uint64]
        L.hemu_set_nudge_config.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.hemu_set_nudge_target.argtypes = [ctypes.c_int64, ctypes.c_int32]
        L.hemu_last_calls.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().hemu_last_error().decode())


class HemuScene:
    """A scene compiled by the product's host code, traced and shaded by the
    device code running on the CPU."""

    def __init__(self, json_text, base_dir=""):
        self.h = lib().hemu_scene_load(json_text.encode(), base_dir.encode())
        if not self.h:
            raise RuntimeError(lib().hemu_last_error().decode())

    @classmethod
    def from_file(cls, path):
        with open(path) as fh:
            return cls(fh.read(), os.path.dirname(os.path.abspath(path)))

    def close(self):
        if self.h:
            lib().hemu_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def camera_rays(self, pixels, sample, seed):
        pixels = np.ascontiguousarray(pixels, np.uint32)
        out = np.zeros((pixels.shape[0], 8), np.float32)
        _check(lib().hemu_camera_rays(self.h, _p(pixels), pixels.shape[0], sample, seed, _p(out)))
        return out

    def trace(self, rays, any_hit=False, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros((rays.shape[0], 5), np.float32)
        _check(lib().hemu_trace(self.h, _p(rays), rays.shape[0], _p(hits), 1 if any_hit else 0, threads))
        return hits

    def render_samples(self, pixels, samples, seed, vol_mode=0):
        pixels = np.ascontiguousarray(pixels, np.uint32)
        samples = np.ascontiguousarray(samples, np.uint32)
        out = np.zeros((pixels.shape[0], 3), np.float32)
        _check(lib().hemu_render_samples(self.h, _p(pixels), _p(samples), pixels.shape[0], seed, vol_mode, _p(out)))
        return out


def render_mixed(scenes, npix, spw, sample0, seeds):
    """One mixed wave of the given scenes' jobs (all npix[k] pixels, spw samples
    from sample0, each with its seed); returns per job its (spw * npix, 3)
    radiance, path s * npix + j being pixel j, sample sample0 + s."""
    n = len(scenes)
    arr = (ctypes.c_void_p * n)(*[sc.h for sc in scenes])
    outs = [np.zeros((spw * npx, 3), np.float32) for npx in npix]
    optr = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
    sd = np.ascontiguousarray(seeds, np.uint32)
    _check(lib().hemu_render_mixed(arr, n, spw, sample0, _p(sd), optr))
    return outs


def set_nudge(seed):
    """0: exact host libm; else, from a stream with this seed, each nudged
    transcendental result moves (probability 1/2) by 1 .. max_ulps ulps up or
    down (set_nudge_config)."""
    lib().hemu_set_nudge(seed)


NUDGE_FUNCTIONS = ["sinf", "cosf", "tanf", "expf", "logf", "log2f", "powf", "atan2f", "acosf", "asinf", "erff"]


def set_nudge_target(index=-1, ulps=0):
    """Move only call number `index` of each render by `ulps` (signed); -1 ends it."""
    lib().hemu_set_nudge_target(index, ulps)


def last_calls():
    """Transcendental calls made by the last render."""
    return lib().hemu_last_calls()


def set_nudge_config(mask=0x7FF, max_ulps=2):
    """Bit i of mask: NUDGE_FUNCTIONS[i] is nudged; results move by at most max_ulps."""
    lib().hemu_set_nudge_config(mask, max_ulps)


def bsdf_eval(bsdf_json, wi, wo):
    wi = np.ascontiguousarray(wi, np.float32)
    wo = np.ascontiguousarray(wo, np.float32)
    n = wi.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    _check(lib().hemu_bsdf_eval(bsdf_json.encode(), _p(wi), _p(wo), n, _p(f), _p(pdf)))
    return f, pdf


def bsdf_sample(bsdf_json, wi, u):
    wi = np.ascontiguousarray(wi, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    n = wi.shape[0]
    wo = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    f = np.zeros((n, 3), np.float32)
    eta = np.zeros(n, np.float32)
    typ = np.zeros(n, np.uint32)
    _check(lib().hemu_bsdf_sample(bsdf_json.encode(), _p(wi), _p(u), n, _p(wo), _p(pdf), _p(f), _p(eta), _p(typ)))
    return wo, pdf, f, eta, typ
