"""Serving loop: jobs of different scenes submitted together are admitted,
interleaved on the device, and each result is identical to rendering it alone."""
import time

import numpy as np
import pytest

from helpers import box, spheres

pytestmark = pytest.mark.gpu


def test_mix_equals_alone(rad, scene_dir):
    a = rad.Scene.from_file(box(scene_dir, 40, 40, 6)[0])
    b = rad.Scene.from_file(spheres(scene_dir, 300, 4, 48, 32, 5)[0])
    c = rad.Scene.from_file(box(scene_dir, 24, 56, 3, seed=9)[0])
    alone = [s.render() for s in (a, b, c)]
    jobs = [s.submit() for s in (a, b, c, a)]
    for j in jobs:
        j.wait()
    mixed = [j.film() for j in jobs]
    for k, ref in enumerate(alone + [alone[0]]):
        assert np.array_equal(mixed[k], ref)
    st = jobs[0].stats()
    assert st["samples"] == 40 * 40 * 6
    assert st["rays_closest"] >= st["samples"]
    for j in jobs:
        j.close()
    for s in (a, b, c):
        s.close()


def test_progress_and_cancel(rad, scene_dir):
    # long enough (seconds, even with many samples per wave) to be cancelled while running
    s = rad.Scene.from_file(box(scene_dir, 256, 256, 4)[0])
    j = s.submit(spp=20000)
    time.sleep(0.05)
    j.cancel()
    with pytest.raises(rad.RadError) as e:
        j.wait()
    assert e.value.code == 9  # RAD_ERR_CANCELLED
    done, total = j.progress()
    assert total == 256 * 256 * 20000 and done < total
    j.close()
    j2 = s.submit(spp=2)
    j2.wait()
    assert j2.progress() == (256 * 256 * 2, 256 * 256 * 2)
    j2.close()
    s.close()


def test_resume_disjoint_samples(rad, scene_dir):
    """Two halves with disjoint sample indices sum to the full render (resumable accumulation)."""
    s = rad.Scene.from_file(box(scene_dir, 32, 32, 8)[0])
    full = s.render(spp=8)
    h1 = s.render(spp=4, first_sample=0)
    h2 = s.render(spp=4, first_sample=4)
    assert np.allclose((h1 + h2) * 0.5, full, rtol=1e-5, atol=1e-6)
    s.close()


def test_errors_are_status_codes(rad, scene_dir):
    with pytest.raises(rad.RadError) as e:
        rad.Scene.from_json('{"camera": ')
    assert e.value.code == 2  # RAD_ERR_JSON
    with pytest.raises(rad.RadError) as e:
        rad.Scene.from_json({"camera": {"type": "orthographic"}, "scene": [], "renderer": {"type": "path"}})
    assert e.value.code == 3  # RAD_ERR_UNKNOWN_FACTORY
    with pytest.raises(rad.RadError) as e:
        rad.bsdf_eval({"type": "plastic_x"}, np.zeros((1, 3)), np.zeros((1, 3)))
    assert e.value.code == 3


def test_graph_replay_equals_direct_launches(rad, scene_dir):
    """Jobs replay one captured CUDA graph per wave; a profiled job launches kernels directly. Same film."""
    s = rad.Scene.from_file(spheres(scene_dir, 200, 3, 40, 24, 5)[0])
    g = s.submit(spp=5)
    g.wait()
    d = s.submit(spp=5, profile=True)
    d.wait()
    assert np.array_equal(g.film(), d.film())
    assert g.stats()["samples"] == d.stats()["samples"] == 40 * 24 * 5
    g.close()
    d.close()
    s.close()


def test_autotune_picks_parameters_and_keeps_results(rad, scene_dir):
    """The tuner only changes launch shapes: the film is bit-identical before and after."""
    s = rad.Scene.from_file(spheres(scene_dir, 200, 3, 40, 24, 5)[0])
    before = s.render(spp=3, seed=7)
    r = s.autotune({"reps": 1})
    assert r["candidates"] == 11 and r["refill_busy"] in (16, 20, 24, 28, 32) and r["blocks_per_sm"] in (4, 6, 8)
    assert r["leaf_frac8"] in (2, 3, 4, 5, 6)
    assert r["best_ms"] > 0 and r["best_ms"] <= r["default_ms"]
    assert np.array_equal(before, s.render(spp=3, seed=7))
    r2 = s.autotune({"refill_busy": [1, 32], "blocks_per_sm": [2], "leaf_frac8": [8], "reps": 1})
    assert r2["candidates"] == 2 and r2["blocks_per_sm"] == 2 and r2["leaf_frac8"] == 8
    assert np.array_equal(before, s.render(spp=3, seed=7))
    with pytest.raises(rad.RadError):
        s.autotune({"refill_busy": [40]})
    s.close()


def test_cli_renders_and_saves(rad, scene_dir):
    """python -m radiantiumplusplus_gb300 --scene x.json writes <dir>/<stem>.exr equal to the job film."""
    import os
    import subprocess
    import sys
    from radiantiumplusplus_gb300.exr import read_exr
    path = box(scene_dir, 32, 24, 4)[0]
    r = subprocess.run([sys.executable, "-m", "radiantiumplusplus_gb300", "--scene", path], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = os.path.join(os.path.dirname(path), "scene.exr")
    assert os.path.exists(out) and "save result to" in r.stdout
    s = rad.Scene.from_file(path)
    assert np.allclose(read_exr(out), s.render(), rtol=0, atol=0)
    s.close()
