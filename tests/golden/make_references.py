"""Generates the high-spp reference images the image-level GPU tests compare
against (tests/test_gpu_images.py), with the oracle: the CPU restatement of
the reference's Path::Li / VolPath::Li (path.cpp:131-236, vol_path.cpp:27-349)
over the seeded synthetic scenes of radiantiumplusplus_gb300/scenes.py.

Each reference is the mean of 16,384 samples per pixel (65,536 for the two
noisier scenes, whose per-pixel variance would otherwise leave the
reference's own noise near the relMSE bar the converged GPU renders are held
to), rendered with a seed the GPU tests do not use, and stored as float16 RGB
(row-major, height x width x 3) with its sample count and seed:

* box_room_256.npz       -- the box room, 256x256, depth 8, Russian roulette from 3
* many_spheres_96x54.npz -- the many-spheres field (10,000 icospheres, 3.2 M
  triangles, sky + 20 emitters), depth 16, at a 96x54 frame of the same camera
* fbm_volume_64.npz      -- vol_path over the 256^3 fBm density grid in the
  rough-glass box, depth 32, at a 64x64 frame of the same camera

Run from the repository root:  python tests/golden/make_references.py [name ...]
(about 30 minutes on 8 cores for all three).
"""
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

SPP = {"box_room_256": 16384, "many_spheres_96x54": 65536, "fbm_volume_64": 65536}
REF_SEED = 7777  # the GPU tests render with the scenes' own seeds
NAMES = ["box_room_256", "many_spheres_96x54", "fbm_volume_64"]


def scene_of(name):
    """(scene dict, assets) of a reference; the GPU tests render the same scene."""
    from radiantiumplusplus_gb300 import scenes
    if name == "box_room_256":
        return scenes.box_room(256, 256, 64), None
    if name == "many_spheres_96x54":
        return scenes.many_spheres(n_spheres=10000, width=96, height=54, spp=64, max_depth=16, seed=2)
    if name == "fbm_volume_64":
        return scenes.volume_box(width=64, height=64, spp=64, max_depth=32, grid=256)
    raise KeyError(name)


def make(name, threads=0):
    import oracle_lib
    from radiantiumplusplus_gb300 import scenes
    sc, assets = scene_of(name)
    spp = SPP[name]
    with tempfile.TemporaryDirectory() as d:
        path = scenes.write_scene(d, sc, assets)
        o = oracle_lib.OracleScene.from_file(path)
        acc = np.zeros((o.height, o.width, 3), np.float64)
        chunk = 1024
        t0 = time.time()
        for s0 in range(0, spp, chunk):
            film, _ = o.render(samples=(s0, s0 + chunk), seed=REF_SEED, threads=threads or (os.cpu_count() or 1))
            acc += film.astype(np.float64)  # a partial sample range comes back as the plain sum
            print("%s: %d / %d spp, %.0f s" % (name, s0 + chunk, spp, time.time() - t0), flush=True)
        o.close()
    mean = (acc / spp).astype(np.float16)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), mean=mean, spp=spp, seed=REF_SEED)


if __name__ == "__main__":
    for n in sys.argv[1:] or NAMES:
        make(n)
