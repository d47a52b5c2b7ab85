"""Seeded synthetic scenes in the reference's JSON scene format.

Every scene here is plain reference JSON (camera / sampler / scene entity tree /
assets / renderer, rad.offline/src/build/build_context.cpp:47-321) plus the OBJ
and Mitsuba ``.vol`` assets it names, so the same files load in the reference
renderer, in this library and in the CPU oracle.

* :func:`box_room` -- the 256x256 box room (five walls, two rotated boxes, one
  ceiling emitter), ``path`` renderer, max depth 8, Russian roulette from 3.
* :func:`many_spheres` -- the many-spheres stress scene: icospheres
  (subdivision 2, 320 triangles each) with lognormal radii, a 40/30/20/10 mix of
  diffuse / rough_metal / rough_glass / disney, a constant sky and small sphere
  emitters; 1920x1080, depth 16 at full size.
* :func:`volume_box` -- the volumetric scene: an fBm density grid in a
  rough-dielectric box on a diffuse ground, a directional light plus a constant
  sky, ``vol_path`` renderer.
* :func:`guided_room` -- hard indirect transport for path guiding: the
  many-spheres field inside a closed cubic room lit only by a directional light
  through a small square opening in the ceiling.
"""

from __future__ import annotations

import json
import math
import os
import struct

import numpy as np

__all__ = ["box_room", "many_spheres", "volume_box", "guided_room", "icosphere_obj", "write_scene"]


def _rect(translate, rotate=None, scale=(1.0, 1.0, 1.0), **extra):
    tw = {"translate": list(map(float, translate)), "scale": list(map(float, scale))}
    if rotate is not None:
        tw["rotate"] = {"axis": list(map(float, rotate[0])), "angle": float(rotate[1])}
    ent = {"to_world": tw, "shape": {"type": "rectangle"}}
    ent.update(extra)
    return ent


def box_room(width=256, height=256, spp=64, seed=1, max_depth=8, rr_depth=3):
    """Box room: 2x2x2 Lambertian box open towards the camera, two boxes, one emitter."""
    grey = {"type": "diffuse", "reflectance": [0.725, 0.725, 0.725]}
    red = {"type": "diffuse", "reflectance": [0.63, 0.065, 0.05]}
    green = {"type": "diffuse", "reflectance": [0.14, 0.45, 0.091]}
    ents = [
        _rect((0, 0, 0), ((1, 0, 0), -90), bsdf={"ref": "grey"}),            # floor, normal +y
        _rect((0, 2, 0), ((1, 0, 0), 90), bsdf={"ref": "grey"}),             # ceiling, normal -y
        _rect((0, 1, -1), None, bsdf={"ref": "grey"}),                       # back wall, normal +z
        _rect((-1, 1, 0), ((0, 1, 0), 90), bsdf=red),                        # x=-1 wall, normal +x
        _rect((1, 1, 0), ((0, 1, 0), -90), bsdf=green),                      # x=+1 wall, normal -x
        {"to_world": {"translate": [0.35, 0.3, 0.3], "rotate": {"axis": [0, 1, 0], "angle": -17.0},
                      "scale": [0.3, 0.3, 0.3]},
         "shape": {"type": "cube"}, "bsdf": {"ref": "grey"}},                # 0.6 tall box
        {"to_world": {"translate": [-0.35, 0.6, -0.35], "rotate": {"axis": [0, 1, 0], "angle": 17.0},
                      "scale": [0.3, 0.6, 0.3]},
         "shape": {"type": "cube"}, "bsdf": {"ref": "grey"}},                # 1.2 tall box
        _rect((0, 1.98, 0), ((1, 0, 0), 90), (0.25, 0.2, 1.0),
              light={"type": "area", "radiance": [17.0, 12.0, 4.0]}),        # 0.5 x 0.4 emitter
    ]
    return {
        "camera": {"type": "perspective", "fov": 40.0, "resolution": [width, height],
                   "origin": [0.0, 1.0, 3.9], "target": [0.0, 1.0, 0.0], "up": [0.0, 1.0, 0.0]},
        "sampler": {"type": "independent", "sample_count": spp, "seed": seed},
        "bsdf_vars": [{"name": "grey", "bsdf": grey}],
        "scene": ents,
        "accel": {"type": "embree"},
        "renderer": {"type": "path", "max_depth": max_depth, "rr_depth": rr_depth},
    }



def materials_room(width=256, height=256, spp=64, seed=1, max_depth=8, rr_depth=3):
    """Box room with the delta and layered BSDFs: plastic floor, rough_plastic back
    wall, a perfect_mirror sphere, a perfect_glass sphere, a masked diffuse box and a
    two-sided plastic / rough_plastic ceiling panel."""
    sc = box_room(width, height, spp, seed, max_depth, rr_depth)
    ents = sc["scene"]
    ents[0]["bsdf"] = {"type": "plastic", "diffuse": [0.55, 0.5, 0.45], "int_ior": 1.5}
    ents[2]["bsdf"] = {"type": "rough_plastic", "diffuse": [0.3, 0.4, 0.6], "alpha": 0.15}
    ents[5]["bsdf"] = {"type": "mask", "opacity": 0.6,
                       "nested": {"type": "diffuse", "reflectance": [0.8, 0.8, 0.8]}}
    ents[6]["bsdf"] = {"type": "two_side", "out_side": {"type": "plastic", "no_linear": True},
                       "in_side": {"type": "rough_plastic", "alpha": 0.3, "distribution": "beckmann"}}
    ents.append({"shape": {"type": "sphere", "center": [0.45, 0.85, 0.35], "radius": 0.25},
                 "bsdf": {"type": "perfect_mirror", "reflectance": [0.95, 0.95, 0.95],
                          "eta": [0.2, 0.92, 1.1], "k": [3.9, 2.45, 2.14]}})
    ents.append({"shape": {"type": "sphere", "center": [-0.4, 0.35, 0.45], "radius": 0.3},
                 "bsdf": {"type": "perfect_glass", "int_ior": 1.5}})
    return sc


def lights_room(width=256, height=256, spp=64, seed=1, max_depth=8, rr_depth=3):
    """Box room lit by a point light, a projection light shining onto the back wall
    and a dimmed area light (delta lights next to an MIS-weighted emitter)."""
    sc = box_room(width, height, spp, seed, max_depth, rr_depth)
    ents = sc["scene"]
    ents[-1]["light"]["radiance"] = [4.0, 3.0, 1.0]
    ents.append({"light": {"type": "point", "position": [0.3, 1.6, 0.2], "intensity": [1.5, 1.3, 1.0]}})
    ents.append({"to_world": {"translate": [0.2, 1.3, 2.2], "rotate": {"axis": [0, 1, 0], "angle": 180.0}},
                 "light": {"type": "projection", "fov": 28.0, "irradiance": [2.0, 1.6, 1.2],
                           "scale": [1.0, 0.8, 1.2]}})
    return sc

def icosphere(subdiv=2):
    """Unit icosphere: (positions, triangles) with outward counter-clockwise winding."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(v), np.array(f, dtype=np.int64)


def icosphere_obj(subdiv=2):
    """OBJ text of a unit icosphere with per-vertex normals (v//vn faces)."""
    v, f = icosphere(subdiv)
    lines = ["o ico"]
    lines += ["v %.9g %.9g %.9g" % tuple(p) for p in v]
    lines += ["vn %.9g %.9g %.9g" % tuple(p) for p in v]
    lines += ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1) for a, b, c in f]
    return "\n".join(lines) + "\n"


def many_spheres(n_spheres=10000, n_emitters=20, width=1920, height=1080, spp=256, max_depth=16,
                 seed=2, sampler_seed=2, extent=100.0):
    """Many-spheres stress scene; returns (scene dict, {asset file name: text})."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, extent, size=(n_spheres, 3))
    radii = rng.lognormal(0.0, 0.5, size=n_spheres)
    kind = rng.uniform(size=n_spheres)
    ents = []
    for i in range(n_spheres):
        k = kind[i]
        if k < 0.4:
            bsdf = {"type": "diffuse", "reflectance": rng.uniform(0.1, 0.9, 3).round(6).tolist()}
        elif k < 0.7:
            bsdf = {"type": "rough_metal", "alpha": round(float(rng.uniform(0.05, 0.5)), 6)}
        elif k < 0.9:
            bsdf = {"type": "rough_glass", "int_ior": 1.5, "ext_ior": 1.0,
                    "alpha": round(float(rng.uniform(0.0, 0.3)), 6)}
        else:
            p = rng.uniform(size=12).round(6)
            bsdf = {"type": "disney", "base_color": p[:3].tolist(), "roughness": float(p[3]),
                    "anisotropic": float(p[4]), "spec_trans": float(p[5]), "sheen": float(p[6]),
                    "sheen_tint": float(p[7]), "flatness": float(p[8]), "spec_tint": float(p[9]),
                    "metallic": float(p[10]), "clearcoat": float(p[11]),
                    "clearcoat_gloss": round(float(rng.uniform()), 6),
                    "specular": round(float(rng.uniform()), 6)}
        ents.append({"to_world": {"translate": centres[i].round(5).tolist(), "scale": round(float(radii[i]), 6)},
                     "shape": {"type": "mesh", "asset_name": "ico"}, "bsdf": bsdf})
    ec = rng.uniform(0.0, extent, size=(n_emitters, 3))
    for i in range(n_emitters):
        ents.append({"shape": {"type": "sphere", "center": ec[i].round(5).tolist(), "radius": 0.5},
                     "light": {"type": "area", "radiance": [50.0, 50.0, 50.0]}})
    ents.append({"light": {"type": "skybox", "radiance": [0.5, 0.5, 0.5]}})
    mid = extent / 2
    scene = {
        "camera": {"type": "perspective", "fov": 55.0, "resolution": [width, height], "far": 10 * extent,
                   "origin": [mid, mid, -0.4 * extent], "target": [mid, mid, mid], "up": [0.0, 1.0, 0.0]},
        "sampler": {"type": "independent", "sample_count": spp, "seed": sampler_seed},
        "assets": [{"name": "ico", "type": "model_obj", "location": "ico.obj"}],
        "scene": ents,
        "accel": {"type": "embree"},
        "renderer": {"type": "path", "max_depth": max_depth, "rr_depth": 3},
    }
    return scene, {"ico.obj": icosphere_obj(2)}


def _sphere_bsdf(rng):
    k = rng.uniform()
    if k < 0.4:
        return {"type": "diffuse", "reflectance": rng.uniform(0.1, 0.9, 3).round(6).tolist()}
    if k < 0.7:
        return {"type": "rough_metal", "alpha": round(float(rng.uniform(0.05, 0.5)), 6)}
    if k < 0.9:
        return {"type": "rough_glass", "int_ior": 1.5, "ext_ior": 1.0, "alpha": round(float(rng.uniform(0.0, 0.3)), 6)}
    p = rng.uniform(size=14).round(6)
    return {"type": "disney", "base_color": p[:3].tolist(), "roughness": float(p[3]), "anisotropic": float(p[4]),
            "spec_trans": float(p[5]), "sheen": float(p[6]), "sheen_tint": float(p[7]), "flatness": float(p[8]),
            "spec_tint": float(p[9]), "metallic": float(p[10]), "clearcoat": float(p[11]),
            "clearcoat_gloss": float(p[12]), "specular": float(p[13])}


def guided_room(n_spheres=10000, width=1920, height=1080, spp=64, max_depth=16, room=200.0, opening=5.0,
                irradiance=1000.0, field=100.0, radius_scale=1.0, seed=5, sampler_seed=5):
    """Closed room [0, room]^3 of grey Lambertian walls with a square `opening` in
    the ceiling centre, the many-spheres field (icospheres with centres uniform in
    a `field`^3 cube at the room centre, lognormal(0, 0.5) radii x radius_scale,
    materials as in many_spheres), lit only by a directional light of the given
    irradiance shining down through the opening. Returns (scene dict, {asset: text})."""
    rng = np.random.default_rng(seed)
    R, c, h = float(room), float(room) / 2.0, float(opening) / 2.0
    wall = {"type": "diffuse", "reflectance": [0.7, 0.7, 0.7]}
    ents = [
        _rect((c, 0, c), ((1, 0, 0), -90), (c, c, 1), bsdf={"ref": "wall"}),          # floor, +y
        _rect((c, c, 0), None, (c, c, 1), bsdf={"ref": "wall"}),                      # z = 0, +z
        _rect((c, c, R), ((0, 1, 0), 180), (c, c, 1), bsdf={"ref": "wall"}),         # z = R, -z
        _rect((0, c, c), ((0, 1, 0), 90), (c, c, 1), bsdf={"ref": "wall"}),           # x = 0, +x
        _rect((R, c, c), ((0, 1, 0), -90), (c, c, 1), bsdf={"ref": "wall"}),          # x = R, -x
        # ceiling (-y) as four strips around the opening
        _rect((c, R, (c - h) / 2), ((1, 0, 0), 90), (c, (c - h) / 2, 1), bsdf={"ref": "wall"}),
        _rect((c, R, (c + h + R) / 2), ((1, 0, 0), 90), (c, (R - c - h) / 2, 1), bsdf={"ref": "wall"}),
        _rect(((c - h) / 2, R, c), ((1, 0, 0), 90), ((c - h) / 2, h, 1), bsdf={"ref": "wall"}),
        _rect(((c + h + R) / 2, R, c), ((1, 0, 0), 90), ((R - c - h) / 2, h, 1), bsdf={"ref": "wall"}),
    ]
    f0 = c - field / 2.0
    centres = rng.uniform(f0, f0 + field, size=(n_spheres, 3))
    radii = rng.lognormal(0.0, 0.5, size=n_spheres) * radius_scale
    for i in range(n_spheres):
        ents.append({"to_world": {"translate": centres[i].round(5).tolist(), "scale": round(float(radii[i]), 6)},
                     "shape": {"type": "mesh", "asset_name": "ico"}, "bsdf": _sphere_bsdf(rng)})
    ents.append({"light": {"type": "directional", "direction": [0.08, -1.0, 0.05],
                           "irradiance": [irradiance, irradiance, irradiance]}})
    scene = {
        "camera": {"type": "perspective", "fov": 70.0, "resolution": [width, height], "far": 10 * R,
                   "origin": [c, 0.35 * R, 0.99 * R], "target": [c, 0.4 * R, 0.0], "up": [0.0, 1.0, 0.0]},
        "sampler": {"type": "independent", "sample_count": spp, "seed": sampler_seed},
        "bsdf_vars": [{"name": "wall", "bsdf": wall}],
        "assets": [{"name": "ico", "type": "model_obj", "location": "ico.obj"}],
        "scene": ents,
        "accel": {"type": "embree"},
        "renderer": {"type": "path", "max_depth": max_depth, "rr_depth": 3},
    }
    return scene, {"ico.obj": icosphere_obj(2)}


def _value_noise(shape, cells, rng):
    """Trilinearly interpolated lattice noise on a grid of `shape` voxels."""
    lat = rng.uniform(-1.0, 1.0, size=(cells + 1,) * 3).astype(np.float32)
    out = np.empty(shape, dtype=np.float32)
    n = shape[0]
    c = (np.arange(n, dtype=np.float32) + 0.5) / n * cells
    i0 = np.minimum(c.astype(np.int64), cells - 1)
    f = c - i0
    f = f * f * (3 - 2 * f)
    for z in range(n):
        z0, fz = i0[z], f[z]
        a = lat[z0] * (1 - fz) + lat[z0 + 1] * fz                 # (cells+1, cells+1) over (y, x)
        b = a[i0][:, i0] * ((1 - f)[:, None] * (1 - f)[None, :])
        b += a[i0 + 1][:, i0] * (f[:, None] * (1 - f)[None, :])
        b += a[i0][:, i0 + 1] * ((1 - f)[:, None] * f[None, :])
        b += a[i0 + 1][:, i0 + 1] * (f[:, None] * f[None, :])
        out[z] = b
    return out


def fbm_density(n=256, octaves=6, threshold=0.3, seed=3):
    """Seeded 6-octave fBm value noise thresholded at `threshold`; float32 (z, y, x) in [0, 1]."""
    rng = np.random.default_rng(seed)
    acc = np.zeros((n, n, n), dtype=np.float32)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = min(4 * (2 ** o), n)
        acc += amp * _value_noise((n, n, n), cells, rng)
        total += amp
        amp *= 0.5
    acc = acc / total * 0.5 + 0.5
    d = np.clip((acc - threshold) / (1.0 - threshold), 0.0, 1.0)
    return d.astype(np.float32)


def write_vol(path, density):
    """Mitsuba .vol v3, float32, one channel (rad.core/src/volume_reader.cpp:65-124)."""
    nz, ny, nx = density.shape
    with open(path, "wb") as fh:
        fh.write(b"VOL" + bytes([3]))
        fh.write(struct.pack("<i", 1))
        fh.write(struct.pack("<iii", nx, ny, nz))
        fh.write(struct.pack("<i", 1))
        fh.write(struct.pack("<6f", 0, 0, 0, 1, 1, 1))
        fh.write(np.ascontiguousarray(density, dtype="<f4").tobytes())


def volume_box(width=1024, height=1024, spp=128, max_depth=32, grid=256, seed=3, sampler_seed=3):
    """Volumetric scene; returns (scene dict, {asset file name: bytes})."""
    dens = fbm_density(grid, seed=seed)
    import io
    buf = io.BytesIO()
    nz, ny, nx = dens.shape
    buf.write(b"VOL" + bytes([3]) + struct.pack("<i", 1) + struct.pack("<iii", nx, ny, nz) + struct.pack("<i", 1))
    buf.write(struct.pack("<6f", 0, 0, 0, 1, 1, 1))
    buf.write(np.ascontiguousarray(dens, dtype="<f4").tobytes())
    medium = {"type": "heterogeneous", "scale": 20.0, "albedo": 0.9,
              "sigma_t": {"type": "volume_grid", "asset_name": "density"},
              "phase": {"type": "hg_phase", "g": 0.6}}
    ents = [
        {"to_world": {"translate": [0, 1, 0], "scale": [1, 1, 1]}, "shape": {"type": "cube"},
         "bsdf": {"type": "rough_glass", "int_ior": 1.33, "ext_ior": 1.0, "alpha": 0.05},
         "in_medium": medium},
        _rect((0, 0, 0), ((1, 0, 0), -90), (6, 6, 1), bsdf={"type": "diffuse", "reflectance": 0.5}),
        {"light": {"type": "directional", "direction": [-0.4, -1.0, -0.3], "irradiance": [3.0, 3.0, 3.0]}},
        {"light": {"type": "skybox", "radiance": [0.3, 0.35, 0.45]}},
    ]
    scene = {
        "camera": {"type": "perspective", "fov": 40.0, "resolution": [width, height], "far": 100.0,
                   "origin": [0.0, 2.2, 5.5], "target": [0.0, 0.9, 0.0], "up": [0.0, 1.0, 0.0]},
        "sampler": {"type": "independent", "sample_count": spp, "seed": sampler_seed},
        "assets": [{"name": "density", "type": "volume_data_mitsuba_vol", "location": "density.vol"}],
        "scene": ents,
        "accel": {"type": "embree"},
        "renderer": {"type": "vol_path", "max_depth": max_depth, "rr_depth": 5},
    }
    return scene, {"density.vol": buf.getvalue()}


def write_scene(directory, scene, assets=None, name="scene.json"):
    """Write `scene` (and its assets) into `directory`; returns the JSON path."""
    os.makedirs(directory, exist_ok=True)
    for fname, data in (assets or {}).items():
        mode = "wb" if isinstance(data, (bytes, bytearray)) else "w"
        with open(os.path.join(directory, fname), mode) as fh:
            fh.write(data)
    path = os.path.join(directory, name)
    with open(path, "w") as fh:
        json.dump(scene, fh)
    return path
