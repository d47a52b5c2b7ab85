"""rad_render_samples_noalloc: the allocation-free variant of rad_render_samples.

Callers that cannot call cudaMalloc pass device buffers they own; the path
state lives in a fixed device array inside the library. Its output must equal
rad_render_samples' (same kernels, same PCG streams) on two calls in a row.
This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from helpers import box, spheres

pytestmark = pytest.mark.gpu


def _noalloc(rad, scene, pixels, samples, seed):
    import torch
    dp = torch.from_numpy(pixels.astype(np.int32)).cuda()
    ds = torch.from_numpy(samples.astype(np.int32)).cuda()
    out = torch.zeros((pixels.shape[0], 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rad.check(rad.lib().rad_render_samples_noalloc(scene.handle, ctypes.c_void_p(dp.data_ptr()),
                                                   ctypes.c_void_p(ds.data_ptr()), pixels.shape[0], seed,
                                                   ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)))
    return out.cpu().numpy()


@pytest.mark.parametrize("which", ["box", "spheres"])
def test_noalloc_matches_render_samples_twice(rad, scene_dir, which):
    path = box(scene_dir, 40, 30, 4)[0] if which == "box" else spheres(scene_dir, 300, 4, 48, 32, 4)[0]
    scene = rad.Scene.from_file(path)
    rng = np.random.default_rng(4)
    for call in range(2):
        n = 16384 if call == 0 else 5000
        pix = rng.integers(0, scene.width * scene.height, n).astype(np.uint32)
        smp = rng.integers(0, 64, n).astype(np.uint32)
        ref = scene.render_samples(pix, smp)
        got = _noalloc(rad, scene, pix, smp, scene.seed)
        close = np.abs(got - ref) <= 1e-3 * np.maximum(np.abs(ref), 1e-1)
        assert close.all(), "call %d: %d samples differ" % (call, (~close.all(1)).sum())
    scene.close()


def test_noalloc_rejects_oversize(rad, scene_dir):
    scene = rad.Scene.from_file(box(scene_dir, 8, 8, 1)[0])
    n = 16385
    st = rad.lib().rad_render_samples_noalloc(scene.handle, ctypes.c_void_p(1), ctypes.c_void_p(1), n, 0,
                                              ctypes.c_void_p(1), None)
    assert st == 1 and "16384" in rad._capi.last_error()
    scene.close()


@pytest.mark.parametrize("renderer", ["particle_tracer", "bdpt"])
def test_noalloc_refuses_splatting_renderers(rad, scene_dir, renderer):
    """particle_tracer has no per-pixel samples and bdpt needs its allocated
    subpath scratch: both answer RAD_ERR_UNSUPPORTED before touching the buffers."""
    from helpers import write
    from radiantiumplusplus_gb300 import scenes
    sc = scenes.box_room(8, 8, 1)
    sc["renderer"] = {"type": renderer}
    scene = rad.Scene.from_file(write(scene_dir, "noalloc_" + renderer, sc)[0])
    st = rad.lib().rad_render_samples_noalloc(scene.handle, ctypes.c_void_p(1), ctypes.c_void_p(1), 1, 0,
                                              ctypes.c_void_p(1), None)
    assert st == rad._capi.RAD_ERR_UNSUPPORTED
    scene.close()
