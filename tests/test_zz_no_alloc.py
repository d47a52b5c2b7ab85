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


def _scene_path(scene_dir, which):
    from helpers import volume, write
    from radiantiumplusplus_gb300 import scenes
    if which == "box":
        return box(scene_dir, 40, 30, 4)[0]
    if which == "spheres":
        return spheres(scene_dir, 300, 4, 48, 32, 4)[0]
    if which == "vol_path":
        return volume(scene_dir, 32, 32, 4, grid=24)[0]
    sc = scenes.box_room(40, 30, 4)
    sc["renderer"] = {"type": "ao"}
    return write(scene_dir, "noalloc_ao", sc)[0]


@pytest.mark.parametrize("which", ["box", "spheres", "vol_path", "ao"])
def test_noalloc_matches_render_samples_twice(rad, scene_dir, which):
    """The same kernels on the same per-sample PCG streams: every sample's
    radiance is bit-identical to rad_render_samples', on two calls in a row
    (the second smaller, over the first call's leftover scratch contents)."""
    scene = rad.Scene.from_file(_scene_path(scene_dir, which))
    rng = np.random.default_rng(4)
    for call in range(2):
        n = 16384 if call == 0 else 5000
        pix = rng.integers(0, scene.width * scene.height, n).astype(np.uint32)
        smp = rng.integers(0, 64, n).astype(np.uint32)
        ref = scene.render_samples(pix, smp)
        got = _noalloc(rad, scene, pix, smp, scene.seed)
        same = (got == ref) | (np.isnan(got) & np.isnan(ref))
        assert same.all(), "call %d: %d samples differ" % (call, (~same.all(1)).sum())
        assert np.abs(ref).sum() > 0
    scene.close()


def test_noalloc_reports_pixels_beyond_the_film(rad, scene_dir):
    """Pixel indices sit in device memory, so the check is on the device: an
    index past the film gives RAD_ERR_DEVICE_CHECK, and the next call is clean."""
    scene = rad.Scene.from_file(box(scene_dir, 8, 8, 1)[0])
    pix = np.array([0, 5, 64, 3], np.uint32)
    smp = np.zeros(4, np.uint32)
    with pytest.raises(rad.RadError) as e:
        _noalloc(rad, scene, pix, smp, 0)
    assert e.value.code == rad._capi.RAD_ERR_DEVICE_CHECK
    pix[2] = 63
    got = _noalloc(rad, scene, pix, smp, 0)
    assert np.array_equal(got, scene.render_samples(pix, smp, seed=0))
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
