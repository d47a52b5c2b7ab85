"""Serving loop: jobs of different scenes submitted together are admitted,
interleaved on the device, and each result is identical to rendering it alone."""
import os
import time

import numpy as np
import pytest

from helpers import box, spheres

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


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


def test_init_refuses_path_buffers_larger_than_the_device(scene_dir):
    """A first rad_init whose path buffers cannot fit (max_paths 4e9, ~1 TB) fails
    with an error before allocating, leaves nothing behind, and a second
    rad_init with the defaults brings the library up; a render then works."""
    import subprocess
    import sys
    import textwrap
    path = box(scene_dir, 24, 16, 2)[0]
    script = textwrap.dedent("""
        import sys
        sys.path.insert(0, {root!r})
        import numpy as np
        import radiantiumplusplus_gb300 as rad
        try:
            rad.init({{"device": 0, "max_paths": 4000000000}})
            print("NO ERROR")
        except rad.RadError as e:
            print("REFUSED", e.code)
        rad.init({{"device": 0}})
        s = rad.Scene.from_file({path!r})
        f = s.render(spp=2)
        print("RENDER", float(f.mean()) > 0)
        s.close()
    """).format(root=os.path.dirname(HERE), path=path)
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "REFUSED" in r.stdout and "RENDER True" in r.stdout, r.stdout


def test_autotune_picks_parameters_and_keeps_results(rad, scene_dir):
    """The tuner only changes launch shapes: the film is bit-identical before and after."""
    s = rad.Scene.from_file(spheres(scene_dir, 200, 3, 40, 24, 5)[0])
    before = s.render(spp=3, seed=7)
    r = s.autotune({"reps": 1})
    assert r["candidates"] == 13 and r["refill_busy"] in (16, 20, 24, 28, 32) and r["blocks_per_sm"] in (4, 6, 8)
    assert r["leaf_frac8"] in (2, 3, 4, 5, 6) and r["shade_block"] in (64, 128, 256)
    assert r["best_ms"] > 0 and r["best_ms"] <= r["default_ms"]
    assert np.array_equal(before, s.render(spp=3, seed=7))
    r2 = s.autotune({"refill_busy": [1, 32], "blocks_per_sm": [2], "leaf_frac8": [8], "shade_block": [256], "reps": 1})
    assert r2["candidates"] == 2 and r2["blocks_per_sm"] == 2 and r2["leaf_frac8"] == 8 and r2["shade_block"] == 256
    assert np.array_equal(before, s.render(spp=3, seed=7))
    r3 = s.autotune({"refill_busy": [24], "blocks_per_sm": [8], "leaf_frac8": [3], "shade_block": [64], "reps": 1})
    assert r3["shade_block"] == 64
    assert np.array_equal(before, s.render(spp=3, seed=7))
    for bad in ({"refill_busy": [40]}, {"shade_block": [96]}):
        with pytest.raises(rad.RadError):
            s.autotune(bad)
    s.close()


def test_autotune_volume_wavefront(rad, scene_dir):
    """On a vol_path scene the tuner times the wavefront's part kernels (lane
    top-up threshold, blocks per SM); the film is bit-identical before and after."""
    from helpers import volume
    path, _, _ = volume(scene_dir, 40, 32, 3, grid=24)
    s = rad.Scene.from_file(path)
    before = s.render(spp=3, seed=5)
    r = s.autotune({"reps": 1})
    assert r["refill_busy"] in (8, 12, 16, 20, 24, 28, 32) and r["blocks_per_sm"] in (2, 3, 4)
    assert r["vol_chunk"] in (4, 8, 16, 32, 64)
    assert r["candidates"] >= 12 and r["best_ms"] > 0 and r["default_ms"] > 0
    assert np.array_equal(before, s.render(spp=3, seed=5))
    r2 = s.autotune({"refill_busy": [1], "blocks_per_sm": [1], "vol_chunk": [1], "reps": 1})
    assert r2["refill_busy"] == 1 and r2["blocks_per_sm"] == 1 and r2["vol_chunk"] == 1
    assert np.array_equal(before, s.render(spp=3, seed=5))
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


def _films_alone(scenes_):
    return [s.render() for s in scenes_]


def test_mixed_waves_equal_alone(rad, scene_dir):
    """Jobs of different scenes running together share the launches of each
    wave (mixed waves); every film is bit-identical to the job rendered alone,
    including a frame larger than its share of a wave (taken in pixel chunks)
    and a job whose spp is not a multiple of its samples per wave."""
    from helpers import materials
    blocker = rad.Scene.from_file(box(scene_dir, 256, 256, 1, seed=21)[0])
    big = rad.Scene.from_file(box(scene_dir, 1280, 1000, 3, seed=22)[0])
    small = [rad.Scene.from_file(box(scene_dir, 40, 40, 6)[0]),
             rad.Scene.from_file(spheres(scene_dir, 300, 4, 48, 32, 5)[0]),
             rad.Scene.from_file(materials(scene_dir, 24, 56, 7)[0])]
    alone = _films_alone([big] + small)
    jb = blocker.submit(spp=20000)  # keeps waves going while the others are submitted
    jobs = [s.submit() for s in [big] + small]
    for j in jobs:
        j.wait()
    films = [j.film() for j in jobs]
    mixed = [j.stats()["mixed_waves"] for j in jobs]
    jb.cancel()
    with pytest.raises(rad.RadError):
        jb.wait()
    jb.close()
    for k, (f, a) in enumerate(zip(films, alone)):
        assert np.array_equal(f, a), k
    assert min(mixed) > 0, mixed
    st = jobs[0].stats()
    assert st["samples"] == 1280 * 1000 * 3
    for j in jobs:
        j.close()
    for s in [blocker, big] + small:
        s.close()


def test_mixed_waves_more_jobs_than_a_wave_holds(rad, scene_dir):
    """More running jobs than one wave's job table (16): every job still runs
    to completion and equals its film alone."""
    blocker = rad.Scene.from_file(box(scene_dir, 256, 256, 1, seed=31)[0])
    ss = [rad.Scene.from_file(box(scene_dir, 16 + 2 * k, 24, 3 + k % 4, seed=40 + k)[0]) for k in range(20)]
    alone = _films_alone(ss)
    jb = blocker.submit(spp=20000)
    jobs = [s.submit() for s in ss]
    for j in jobs:
        j.wait()
    for j, a in zip(jobs, alone):
        assert np.array_equal(j.film(), a)
        j.close()
    jb.cancel()
    with pytest.raises(rad.RadError):
        jb.wait()
    jb.close()
    for s in [blocker] + ss:
        s.close()


def test_mixing_can_be_switched_off(rad, scene_dir):
    """rad_init {"mix_jobs": 0}: jobs take turns wave by wave instead; same films."""
    a = rad.Scene.from_file(box(scene_dir, 32, 32, 4, seed=51)[0])
    b = rad.Scene.from_file(box(scene_dir, 48, 16, 4, seed=52)[0])
    alone = _films_alone([a, b])
    blocker = rad.Scene.from_file(box(scene_dir, 256, 256, 1, seed=53)[0])
    try:
        rad.init({"mix_jobs": 0})
        jb = blocker.submit(spp=20000)
        ja, jbb = a.submit(), b.submit()
        ja.wait()
        jbb.wait()
        assert ja.stats()["mixed_waves"] == 0 and jbb.stats()["mixed_waves"] == 0
        assert np.array_equal(ja.film(), alone[0]) and np.array_equal(jbb.film(), alone[1])
        jb.cancel()
        with pytest.raises(rad.RadError):
            jb.wait()
        for j in (ja, jbb, jb):
            j.close()
    finally:
        rad.init({"mix_jobs": 1})
    for s in (a, b, blocker):
        s.close()
