"""ctypes binding of include/radgpu.h (the C ABI of librad_gpu.so).

The library is the product: there is no Python or CPU fallback. Loading fails
with an ImportError-style RuntimeError when librad_gpu.so is missing.
"""

from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "librad_gpu.so")

RAD_OK = 0
RAD_ERR_INVALID_ARG = 1
RAD_ERR_JSON = 2
RAD_ERR_UNKNOWN_FACTORY = 3
RAD_ERR_IO = 4
RAD_ERR_CUDA = 5
RAD_ERR_OUT_OF_MEMORY = 6
RAD_ERR_ADMISSION = 7
RAD_ERR_TIMEOUT = 8
RAD_ERR_CANCELLED = 9
RAD_ERR_NOT_READY = 10
RAD_ERR_NO_DEVICE = 11
RAD_ERR_DEVICE_CHECK = 12
RAD_ERR_UNSUPPORTED = 13

RAD_JOB_PROFILE_KERNELS = 1
RAD_JOB_SYNC = 2
RAD_JOB_COUNT_TRAVERSAL = 4
RAD_JOB_GUIDE = 8
RAD_JOB_VOL_BRICKS = 16
RAD_JOB_VOL_FP16 = 32
RAD_JOB_VOL_REAL_DEPTH = 64
RAD_JOB_VOL_PERSISTENT = 128

# Every symbol the header declares (the export test checks this list).
EXPORTS = [
    "rad_init", "rad_shutdown", "rad_last_error", "rad_version", "rad_device_usage",
    "rad_scene_load_json", "rad_scene_load_file", "rad_scene_destroy", "rad_scene_info_get",
    "rad_scene_footprint", "rad_job_submit", "rad_job_wait", "rad_job_cancel", "rad_job_progress",
    "rad_job_film", "rad_job_stats", "rad_job_destroy", "rad_trace_batch", "rad_trace_batch_device",
    "rad_bsdf_eval_batch", "rad_bsdf_sample_batch", "rad_camera_rays", "rad_scene_texture_eval", "rad_render_samples",
    "rad_render_samples_noalloc", "rad_guide_enable", "rad_guide_info", "rad_guide_checkpoint",
    "rad_guide_load", "rad_guide_forward", "rad_guide_mix_eval", "rad_guide_grad", "rad_autotune",
]


class RadError(RuntimeError):
    """A non-zero status from the C ABI; `.code` is the RAD_ERR_* value."""

    def __init__(self, code, message):
        super().__init__("radgpu error %d: %s" % (code, message))
        self.code = code


class SceneInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("seed", ctypes.c_uint32), ("max_depth", ctypes.c_int32), ("rr_depth", ctypes.c_int32),
                ("is_vol_path", ctypes.c_int32), ("n_shapes", ctypes.c_int32), ("n_lights", ctypes.c_int32),
                ("n_media", ctypes.c_int32), ("n_materials", ctypes.c_int32), ("n_prims", ctypes.c_uint64),
                ("n_bvh_nodes", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64)]


class JobDesc(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("seed", ctypes.c_uint32), ("first_sample", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_uint64), ("invalid_samples", ctypes.c_uint64),
                ("rays_closest", ctypes.c_uint64), ("rays_shadow", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("gpu_ms", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("ms_generate", ctypes.c_double), ("ms_extend", ctypes.c_double),
                ("ms_shade", ctypes.c_double), ("ms_shadow", ctypes.c_double), ("ms_accumulate", ctypes.c_double),
                ("ms_volpath", ctypes.c_double), ("n_extend", ctypes.c_uint64), ("n_shade", ctypes.c_uint64),
                ("n_shadow", ctypes.c_uint64), ("trav_nodes_closest", ctypes.c_uint64),
                ("trav_prims_closest", ctypes.c_uint64), ("trav_nodes_shadow", ctypes.c_uint64),
                ("trav_prims_shadow", ctypes.c_uint64), ("guide_records", ctypes.c_uint64),
                ("guide_train_steps", ctypes.c_uint64), ("ms_guide_infer", ctypes.c_double),
                ("ms_guide_train", ctypes.c_double), ("mixed_waves", ctypes.c_uint64)]


class TuneResult(ctypes.Structure):
    _fields_ = [("refill_busy", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double), ("leaf_frac8", ctypes.c_int32),
                ("shade_block", ctypes.c_int32),
                ("vol_chunk", ctypes.c_int32)]


class GuideInfo(ctypes.Structure):
    _fields_ = [("n_params", ctypes.c_uint64), ("n_table", ctypes.c_uint64), ("log2_table", ctypes.c_uint32),
                ("levels", ctypes.c_uint32), ("level_res", ctypes.c_uint32 * 16), ("lo", ctypes.c_float * 3),
                ("hi", ctypes.c_float * 3), ("adam_steps", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64)]


_lib = None


def load(path=LIB_PATH):
    """Load librad_gpu.so (built by radiantiumplusplus_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("librad_gpu.so is not built (%s); run radiantiumplusplus_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I64 = ctypes.c_int64
    sig = {
        "rad_init": [ctypes.c_char_p],
        "rad_shutdown": [],
        "rad_last_error": [ctypes.c_char_p, ctypes.c_size_t],
        "rad_version": [P, P],
        "rad_device_usage": [P, P],
        "rad_scene_load_json": [ctypes.c_char_p, ctypes.c_char_p, P],
        "rad_scene_load_file": [ctypes.c_char_p, P],
        "rad_scene_destroy": [P],
        "rad_scene_info_get": [P, P],
        "rad_scene_footprint": [P, P],
        "rad_job_submit": [P, P, P],
        "rad_job_wait": [P, I64],
        "rad_job_cancel": [P],
        "rad_job_progress": [P, P, P],
        "rad_job_film": [P, P, ctypes.c_int32, ctypes.c_int32],
        "rad_job_stats": [P, P],
        "rad_job_destroy": [P],
        "rad_trace_batch": [P, P, I64, P, ctypes.c_int32],
        "rad_trace_batch_device": [P, P, I64, P, ctypes.c_int32],
        "rad_bsdf_eval_batch": [ctypes.c_char_p, P, P, I64, P, P],
        "rad_bsdf_sample_batch": [ctypes.c_char_p, P, P, I64, P, P, P, P, P],
        "rad_camera_rays": [P, P, I64, ctypes.c_uint32, ctypes.c_uint32, P],
        "rad_scene_texture_eval": [P, ctypes.c_uint32, P, P, I64, P],
        "rad_render_samples": [P, P, P, I64, ctypes.c_uint32, P],
        "rad_render_samples_noalloc": [P, P, P, I64, ctypes.c_uint32, P, P],
        "rad_guide_enable": [P, ctypes.c_char_p],
        "rad_guide_info": [P, P],
        "rad_guide_checkpoint": [P, P, ctypes.c_size_t, P],
        "rad_guide_load": [P, P, ctypes.c_size_t],
        "rad_guide_forward": [P, P, I64, P, P],
        "rad_guide_mix_eval": [P, P, P, I64, P, P],
        "rad_guide_grad": [P, P, I64, P, P],
        "rad_autotune": [P, ctypes.c_char_p, P],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(4096)
    load().rad_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status):
    if status != RAD_OK:
        raise RadError(status, last_error())
    return status
