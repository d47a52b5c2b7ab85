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


def _film_bytes(scene):
    return scene.width * scene.height * 16 + 64  # float4 per pixel + stats tail (rad_job_submit)


def test_parked_film_stays_counted(rad, scene_dir):
    """A destroyed job's film is parked with its scene for the next job: it is
    still counted against the budget until the scene (or admission) frees it."""
    used0, _ = rad.device_usage()
    s = rad.Scene.from_file(box(scene_dir, 36, 20, 2)[0])
    used1, _ = rad.device_usage()
    assert used1 == used0 + s.footprint()
    j = s.submit(spp=2)
    j.wait()
    assert rad.device_usage()[0] == used1 + _film_bytes(s)
    j.close()
    assert rad.device_usage()[0] == used1 + _film_bytes(s)  # parked, still counted
    j2 = s.submit(spp=1)  # takes the parked film over: counted once
    j2.wait()
    assert rad.device_usage()[0] == used1 + _film_bytes(s)
    j2.close()
    s.close()
    assert rad.device_usage()[0] == used0


def test_admission_refusals_and_parked_film_release(rad, scene_dir):
    """Against a small budget: a scene that does not fit and a job whose film
    does not fit are refused with RAD_ERR_ADMISSION; a job that fits only once
    another scene's parked film is freed is admitted (the film is released)."""
    used0, budget0 = rad.device_usage()
    try:
        a = rad.Scene.from_file(box(scene_dir, 64, 64, 1)[0])
        j = a.submit(spp=1)
        j.wait()
        j.close()  # a's film is now parked
        b = rad.Scene.from_file(box(scene_dir, 48, 48, 1, seed=3)[0])
        used = rad.device_usage()[0]
        # room for b's film only if a's parked film is released
        rad.init({"budget_bytes": used - _film_bytes(a) + _film_bytes(b)})
        jb = b.submit(spp=1)
        jb.wait()
        assert rad.device_usage()[0] == used - _film_bytes(a) + _film_bytes(b)
        jb.close()
        # a film larger than the whole remaining budget: refused, async and sync
        rad.init({"budget_bytes": rad.device_usage()[0] + 100})
        for sync in (False, True):
            jc = a.submit(spp=1, sync=sync)
            with pytest.raises(rad.RadError) as e:
                jc.wait()
            assert e.value.code == 7  # RAD_ERR_ADMISSION
            jc.close()
        assert rad.device_usage()[0] == used - _film_bytes(a)  # both films freed: nothing parked
        rad.init({"budget_bytes": rad.device_usage()[0] + 100})
        with pytest.raises(rad.RadError) as e:
            rad.Scene.from_file(box(scene_dir, 16, 16, 1, seed=5)[0])
        assert e.value.code == 7
        b.close()
        a.close()
    finally:
        rad.init({"budget_bytes": budget0})
    assert rad.device_usage()[0] == used0


def test_wait_times_out(rad, scene_dir):
    """rad_job_wait returns RAD_ERR_TIMEOUT while the job runs on; the job still finishes."""
    s = rad.Scene.from_file(box(scene_dir, 256, 256, 4)[0])
    j = s.submit(spp=4000)
    with pytest.raises(rad.RadError) as e:
        j.wait(timeout_ms=1)
    assert e.value.code == 8  # RAD_ERR_TIMEOUT
    j.cancel()
    with pytest.raises(rad.RadError) as e:
        j.wait()
    assert e.value.code == 9
    j.close()
    s.close()
