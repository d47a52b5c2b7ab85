"""radiantiumplusplus_gb300 -- GB300-native drop-in for RadiantiumPlusPlus' offline hot path.

The `path` / `vol_path` renderers of module/rad.offline run as sm_103a
wavefront kernels behind the C ABI in include/radgpu.h (librad_gpu.so). This
package is the Python host mirror of the reference's interface:

* :class:`Scene` -- BuildContext::SetFromJson + Build (build_context.cpp:47-321):
  loads the reference's JSON scene format with the same factory names.
* :class:`Renderer` -- Renderer::Start / Wait / Stop / SaveResult / IsComplete /
  AllTaskCount / CompletedTaskCount / ElapsedTime (renderer.h:19-48).
* :func:`bsdf_eval` / :func:`bsdf_sample` -- Bsdf::Eval / Pdf / Sample batches.
* :meth:`Scene.trace` -- Accel::RayIntersectPreliminary / RayIntersect batches.

There is no CPU fallback: every call goes through librad_gpu.so and raises
:class:`RadError` when the library or the device is missing.
"""

from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import _capi
from ._capi import RadError, check

__all__ = ["Scene", "Job", "Renderer", "RadError", "init", "shutdown", "device_usage", "bsdf_eval", "bsdf_sample",
           "lib"]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lib():
    return _capi.load()


_atexit_registered = False


def init(config=None):
    """rad_init: select the device and set the admission budget (bytes)."""
    global _atexit_registered
    cfg = json.dumps(config) if isinstance(config, dict) else config
    check(lib().rad_init(cfg.encode() if cfg else None))
    if not _atexit_registered:
        import atexit
        atexit.register(lambda: lib().rad_shutdown())
        _atexit_registered = True


def shutdown():
    check(lib().rad_shutdown())


def device_usage():
    """rad_device_usage: (bytes counted against the admission budget, budget)."""
    u, b = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().rad_device_usage(ctypes.byref(u), ctypes.byref(b)))
    return u.value, b.value


class Scene:
    """A resident scene (BVH8 + materials + lights + media) on the device."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)
        info = _capi.SceneInfo()
        check(lib().rad_scene_info_get(self._h, ctypes.byref(info)))
        self.info = info
        self.width, self.height = info.width, info.height
        self.spp, self.seed = info.spp, info.seed

    @classmethod
    def from_json(cls, scene, base_dir=""):
        text = scene if isinstance(scene, str) else json.dumps(scene)
        h = ctypes.c_void_p()
        check(lib().rad_scene_load_json(text.encode(), base_dir.encode(), ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def from_file(cls, path):
        h = ctypes.c_void_p()
        check(lib().rad_scene_load_file(os.fspath(path).encode(), ctypes.byref(h)))
        return cls(h.value)

    @property
    def handle(self):
        return self._h

    def footprint(self):
        v = ctypes.c_uint64()
        check(lib().rad_scene_footprint(self._h, ctypes.byref(v)))
        return v.value

    def close(self):
        if self._h is not None and self._h.value:
            check(lib().rad_scene_destroy(self._h))
        self._h = None

    def trace(self, rays, any_hit=False):
        """rays: (n, 8) float32 (ox, oy, oz, tmin, dx, dy, dz, tmax) -> (n, 5) float32 hit words."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.zeros((rays.shape[0], 5), dtype=np.float32)
        check(lib().rad_trace_batch(self._h, _p(rays), rays.shape[0], _p(hits), 1 if any_hit else 0))
        return hits

    def camera_rays(self, pixels, sample=0, seed=None):
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        out = np.zeros((pixels.shape[0], 8), dtype=np.float32)
        check(lib().rad_camera_rays(self._h, _p(pixels), pixels.shape[0], sample,
                                    self.seed if seed is None else seed, _p(out)))
        return out

    def texture_eval(self, texture, uv, duv=None):
        """Texture number `texture` (creation order) at uv (n, 2) with uv derivatives
        duv (n, 4: du/dx, dv/dx, du/dy, dv/dy; default 0) -> (n, 3)."""
        uv = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
        n = uv.shape[0]
        duv = np.zeros((n, 4), np.float32) if duv is None else np.ascontiguousarray(duv, dtype=np.float32)
        out = np.zeros((n, 3), dtype=np.float32)
        check(lib().rad_scene_texture_eval(self._h, texture, _p(uv), _p(duv), n, _p(out)))
        return out

    def render_samples(self, pixels, samples, seed=None):
        """Li of individual (pixel, sample) pairs through the job kernels -> (n, 3)."""
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        samples = np.ascontiguousarray(samples, dtype=np.uint32)
        out = np.zeros((pixels.shape[0], 3), dtype=np.float32)
        check(lib().rad_render_samples(self._h, _p(pixels), _p(samples), pixels.shape[0],
                                       self.seed if seed is None else seed, _p(out)))
        return out

    def submit(self, spp=0, seed=None, first_sample=0, profile=False, sync=False, count_traversal=False,
               guide=False, vol_bricks=False, vol_fp16=False, vol_real_depth=False, vol_persistent=False):
        return Job(self, spp, seed, first_sample, profile, sync, count_traversal, guide, vol_bricks, vol_fp16,
                   vol_real_depth, vol_persistent)

    def autotune(self, config=None):
        """Pick this scene's launch parameters by timing waves (rad_autotune): for `path` the traversal kernels'
        refill threshold, blocks per SM and leaf vote and the shade-class block size; for `vol_path` the wavefront
        part kernels' top-up threshold, blocks per SM and chunk. config: dict of candidate lists and "reps"."""
        r = _capi.TuneResult()
        text = None if config is None else json.dumps(config).encode()
        check(lib().rad_autotune(self._h, text, ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in r._fields_}

    # ---- learned path guiding (no counterpart in the reference)
    def guide_enable(self, config=None):
        """Create (re-seed) the scene's guide network; config: dict of rad_guide_enable keys."""
        text = None if config is None else json.dumps(config).encode()
        check(lib().rad_guide_enable(self._h, text))

    def guide_info(self):
        gi = _capi.GuideInfo()
        check(lib().rad_guide_info(self._h, ctypes.byref(gi)))
        return {"n_params": gi.n_params, "n_table": gi.n_table, "log2_table": gi.log2_table,
                "levels": gi.levels, "level_res": list(gi.level_res), "lo": list(gi.lo), "hi": list(gi.hi),
                "adam_steps": gi.adam_steps, "device_bytes": gi.device_bytes}

    def guide_checkpoint(self):
        """Parameters and Adam moments as bytes (see rad_guide_checkpoint)."""
        need = ctypes.c_size_t()
        check(lib().rad_guide_checkpoint(self._h, None, 0, ctypes.byref(need)))
        buf = np.empty(need.value, dtype=np.uint8)
        check(lib().rad_guide_checkpoint(self._h, _p(buf), buf.size, ctypes.byref(need)))
        return buf.tobytes()

    def guide_load(self, blob):
        buf = np.frombuffer(blob, dtype=np.uint8)
        check(lib().rad_guide_load(self._h, _p(buf), buf.size))

    def guide_forward(self, queries):
        """queries (n, 9): position, shading normal, wo -> (raw (n, 48), mixture (n, 44))."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        raw = np.zeros((q.shape[0], 48), dtype=np.float32)
        mix = np.zeros((q.shape[0], 44), dtype=np.float32)
        check(lib().rad_guide_forward(self._h, _p(q), q.shape[0], _p(raw), _p(mix)))
        return raw, mix

    def guide_grad(self, records):
        """records (n, 16) -> (gradient over all parameters, summed loss)."""
        r = np.ascontiguousarray(records, dtype=np.float32)
        n_params = self.guide_info()["n_params"]
        g = np.zeros(n_params, dtype=np.float32)
        loss = ctypes.c_float()
        check(lib().rad_guide_grad(self._h, _p(r), r.shape[0], _p(g), ctypes.byref(loss)))
        return g, loss.value

    def render(self, spp=0, seed=None, first_sample=0):
        """Submit, wait and return the film (H, W, 3) float32."""
        job = self.submit(spp, seed, first_sample)
        try:
            job.wait()
            return job.film()
        finally:
            job.close()


class Job:
    """One render job (rad_job_*)."""

    def __init__(self, scene, spp=0, seed=None, first_sample=0, profile=False, sync=False, count_traversal=False,
                 guide=False, vol_bricks=False, vol_fp16=False, vol_real_depth=False, vol_persistent=False):
        self.scene = scene
        flags = (_capi.RAD_JOB_PROFILE_KERNELS if profile else 0) | (_capi.RAD_JOB_SYNC if sync else 0)
        flags |= _capi.RAD_JOB_COUNT_TRAVERSAL if count_traversal else 0
        flags |= _capi.RAD_JOB_GUIDE if guide else 0
        flags |= _capi.RAD_JOB_VOL_BRICKS if vol_bricks else 0
        flags |= _capi.RAD_JOB_VOL_FP16 if vol_fp16 else 0
        flags |= _capi.RAD_JOB_VOL_REAL_DEPTH if vol_real_depth else 0
        flags |= _capi.RAD_JOB_VOL_PERSISTENT if vol_persistent else 0
        d = _capi.JobDesc(spp, 0xFFFFFFFF if seed is None else seed, first_sample, flags)
        h = ctypes.c_void_p()
        check(lib().rad_job_submit(scene.handle, ctypes.byref(d), ctypes.byref(h)))
        self._h = h

    def wait(self, timeout_ms=-1):
        check(lib().rad_job_wait(self._h, timeout_ms))

    def cancel(self):
        check(lib().rad_job_cancel(self._h))

    def progress(self):
        d, t = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().rad_job_progress(self._h, ctypes.byref(d), ctypes.byref(t)))
        return d.value, t.value

    def film(self, out=None):
        W, H = self.scene.width, self.scene.height
        if out is None:
            out = np.empty((H, W, 3), dtype=np.float32)
        check(lib().rad_job_film(self._h, _p(out), W, H))
        return out

    def stats(self):
        s = _capi.Stats()
        check(lib().rad_job_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if self._h is not None and self._h.value:
            check(lib().rad_job_destroy(self._h))
        self._h = None


class Renderer:
    """Mirror of the reference's Renderer / SampleRenderer (renderer.h:19-62).

    ``Renderer(scene_json_path)`` builds the scene (RendererFactory "path" /
    "vol_path" is chosen by the JSON), ``start()`` submits the whole sample
    budget asynchronously, ``wait()`` joins, ``stop()`` cancels (the film keeps
    the samples already accumulated), ``save_result(path)`` writes the film as
    an RGB fp32 OpenEXR file like SampleRenderer::SaveResult.
    """

    def __init__(self, scene, base_dir=""):
        if isinstance(scene, Scene):
            self.scene = scene
        elif isinstance(scene, (str, os.PathLike)) and os.path.exists(scene):
            self.scene = Scene.from_file(scene)
        else:
            self.scene = Scene.from_json(scene, base_dir)
        self._job = None
        self._t0 = None
        self._t1 = None

    def start(self):
        if self._job is None:
            self._t0 = time.perf_counter()
            self._job = self.scene.submit()

    def wait(self):
        if self._job is not None:
            try:
                self._job.wait()
            except RadError as e:
                if e.code != _capi.RAD_ERR_CANCELLED:
                    raise
            self._t1 = time.perf_counter()

    def stop(self):
        if self._job is not None:
            self._job.cancel()

    def is_complete(self):
        if self._job is None:
            return False
        done, total = self._job.progress()
        return done >= total and self._t1 is not None

    def all_task_count(self):
        return self.scene.width * self.scene.height

    def completed_task_count(self):
        if self._job is None:
            return 0
        done, total = self._job.progress()
        return done // max(1, self.scene.spp) if total else 0

    def elapsed_time(self):
        if self._t0 is None:
            return 0
        end = self._t1 if self._t1 is not None else time.perf_counter()
        return int((end - self._t0) * 1000)

    def film(self):
        return self._job.film()

    def save_result(self, path):
        from .exr import write_exr
        write_exr(path, self.film())
        return path

    def close(self):
        if self._job is not None:
            self._job.close()
            self._job = None


def _bsdf_json(bsdf):
    return (bsdf if isinstance(bsdf, str) else json.dumps(bsdf)).encode()


def bsdf_eval(bsdf, wi, wo):
    """Bsdf::Eval and Bsdf::Pdf on the device -> (f (n,3), pdf (n,))."""
    wi = np.ascontiguousarray(wi, dtype=np.float32)
    wo = np.ascontiguousarray(wo, dtype=np.float32)
    n = wi.shape[0]
    f = np.zeros((n, 3), dtype=np.float32)
    pdf = np.zeros(n, dtype=np.float32)
    check(lib().rad_bsdf_eval_batch(_bsdf_json(bsdf), _p(wi), _p(wo), n, _p(f), _p(pdf)))
    return f, pdf


def bsdf_sample(bsdf, wi, u):
    """Bsdf::Sample on the device -> (wo, pdf, f, eta, type)."""
    wi = np.ascontiguousarray(wi, dtype=np.float32)
    u = np.ascontiguousarray(u, dtype=np.float32)
    n = wi.shape[0]
    wo = np.zeros((n, 3), dtype=np.float32)
    pdf = np.zeros(n, dtype=np.float32)
    f = np.zeros((n, 3), dtype=np.float32)
    eta = np.zeros(n, dtype=np.float32)
    typ = np.zeros(n, dtype=np.uint32)
    check(lib().rad_bsdf_sample_batch(_bsdf_json(bsdf), _p(wi), _p(u), n, _p(wo), _p(pdf), _p(f), _p(eta), _p(typ)))
    return wo, pdf, f, eta, typ


def guide_mix_eval(mix, dirs=None, u=None):
    """Packed guide mixtures (n, 44): pdf at dirs (n, 3), or (directions, pdf) sampled from u (n, 3)."""
    mix = np.ascontiguousarray(mix, dtype=np.float32)
    n = mix.shape[0]
    pdf = np.zeros(n, dtype=np.float32)
    if dirs is not None:
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        check(lib().rad_guide_mix_eval(_p(mix), _p(d), None, n, _p(pdf), None))
        return pdf
    uu = np.ascontiguousarray(u, dtype=np.float32)
    out = np.zeros((n, 3), dtype=np.float32)
    check(lib().rad_guide_mix_eval(_p(mix), None, _p(uu), n, _p(pdf), _p(out)))
    return out, pdf
