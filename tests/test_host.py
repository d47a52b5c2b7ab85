"""Host-side logic that needs no GPU: scene generators, EXR writer, oracle loads."""
import json
import os

import numpy as np

from helpers import box, materials, spheres, volume
from radiantiumplusplus_gb300 import exr, scenes


def test_exr_round_trip(tmp_path):
    img = np.random.default_rng(0).uniform(0, 5, (7, 11, 3)).astype(np.float32)
    p = exr.write_exr(str(tmp_path / "a.exr"), img)
    assert np.array_equal(exr.read_exr(p), img)


def test_srgb_matches_color24f():
    v = np.array([0.0, 0.002, 0.0031308, 0.5, 1.0], np.float32)
    s = exr.to_srgb(v)
    assert abs(s[1] - 12.92 * 0.002) < 1e-7 and abs(s[4] - 1.0) < 1e-6


def test_icosphere_counts_and_winding():
    v, f = scenes.icosphere(2)
    assert len(v) == 162 and len(f) == 320
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert (np.einsum("ij,ij->i", n, v[f].mean(1)) > 0).all()


def test_generated_scenes_load_in_oracle(oracle, scene_dir):
    for path, text, d in (box(scene_dir), spheres(scene_dir, 50, 3), volume(scene_dir, 16, 16, 1, grid=16),
                          materials(scene_dir, 16, 16, 1)):
        o = oracle.OracleScene(text, d)
        assert o.width > 0 and o.n_prims > 0
        o.close()


def test_unknown_factory_is_reported(oracle):
    import pytest
    sc = scenes.box_room(8, 8, 1)
    sc["renderer"]["type"] = "bdpt_x"
    with pytest.raises(RuntimeError, match="cannot find factory"):
        oracle.OracleScene(json.dumps(sc), "")


def test_cli_argument_errors():
    """The CLI's argument errors (rad.offline.cli/main.cpp:14-33) need no GPU."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-m", "radiantiumplusplus_gb300"], capture_output=True, text=True)
    assert r.returncode == 2 and "--scene <scene.json>" in r.stderr
    r = subprocess.run([sys.executable, "-m", "radiantiumplusplus_gb300", "--scene", "no_such_scene.json"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "cannot open file" in r.stderr
