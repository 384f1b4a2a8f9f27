"""Seeded synthetic workloads of the benchmark configurations.

Each builder returns host-side inputs only (numpy voxel grids, palettes, camera and light
structs, ray arrays); uploading them is the caller's business.  All content is generated by
libvtrace's deterministic host generators; camera and light poses come from numpy's seeded PCG64.

  terrain256   256^3 fBm heightfield (~30% occupancy), 640x480 pinhole camera, 60 deg vertical FOV
  shapes1024   1024^3 with 10,000 boxes and spheres (radius 2-40, ~4-5% occupancy), 1920x1080,
               directional light with one hard-shadow ray per lit hit
  cave512      512^3 3D-noise cave (~45% occupancy), 16,777,216 rays with origins uniform in the
               grid and directions uniform on the sphere
  multiview    8 scenes (128^3-512^3, terrain / shapes / cave) and 64 cameras with resolutions
               log-uniform between 320x240 and 3840x2160 and 1-4 jittered samples per pixel
  serving      32 scenes (128^3-1024^3) and a Poisson stream of render requests (mean rate
               2,000/s) with resolutions log-uniform between 320x240 and 1920x1080, 1-8 spp
"""
import math

import numpy as np

from . import camera_look_at, gen_cave, gen_palette, gen_rays_uniform, gen_shapes, gen_terrain, make_light


def seeded_pose(n, seed, distance, elev=(15.0, 45.0)):
    """Eye on a sphere of `distance` around the grid centre (elevation in degrees), looking at
    the centre with +Y up."""
    rng = np.random.default_rng(seed)
    az = rng.uniform(0.0, 2.0 * math.pi)
    el = math.radians(rng.uniform(*elev))
    c = np.array([n[0] / 2.0, n[1] / 2.0, n[2] / 2.0])
    d = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    eye = c + distance * d
    return tuple(float(x) for x in eye), tuple(float(x) for x in c)


def seeded_light(seed, ambient=0.25, shadows=True):
    rng = np.random.default_rng(seed + 1000)
    az = rng.uniform(0.0, 2.0 * math.pi)
    el = math.radians(rng.uniform(30.0, 60.0))
    d = (math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az))
    return make_light(d, ambient, shadows)


def terrain256(n=256, width=640, height=480, seed=1):
    vox = gen_terrain(n, seed, octaves=5, occupancy=0.3)
    pal = gen_palette(seed)
    eye, target = seeded_pose((n, n, n), seed, 1.1 * n)
    cam = camera_look_at(eye, target, (0.0, 1.0, 0.0), 60.0, width, height)
    return {"name": "terrain%d_%dx%d" % (n, width, height), "voxels": vox, "palette": pal,
            "camera": cam, "light": seeded_light(seed, shadows=False)}


def shapes1024(n=1024, width=1920, height=1080, seed=2, count=10000):
    vox = gen_shapes(n, seed, count=count, rmin=2.0, rmax=40.0)
    pal = gen_palette(seed)
    # just outside the grid (|eye - centre| = 0.9 n > half-diagonal of a face), so the grid
    # fills the frame and every primary ray traverses it
    eye, target = seeded_pose((n, n, n), seed, 0.9 * n)
    cam = camera_look_at(eye, target, (0.0, 1.0, 0.0), 60.0, width, height)
    return {"name": "shapes%d_%dx%d_shadow" % (n, width, height), "voxels": vox, "palette": pal,
            "camera": cam, "light": seeded_light(seed, shadows=True)}


def cave512(n=512, rays=1 << 24, seed=3):
    vox = gen_cave(n, seed, occupancy=0.45)
    pal = gen_palette(seed)
    r = gen_rays_uniform(n, seed + 1, rays)
    return {"name": "cave%d_%drays" % (n, rays), "voxels": vox, "palette": pal, "rays": r}


def multiview(n_scenes=8, n_views=64, seed=4, min_px=320 * 240, max_px=3840 * 2160,
              sizes=(128, 192, 256, 320, 384, 448, 512, 256), max_spp=4):
    """Scenes (voxels, palette, kind) and view specs (scene index, camera, spp, light)."""
    rng = np.random.default_rng(seed)
    kinds = ["terrain", "shapes", "cave"]
    scenes = []
    for i in range(n_scenes):
        n = int(sizes[i % len(sizes)])
        kind = kinds[i % 3]
        if kind == "terrain":
            vox = gen_terrain(n, seed * 100 + i, octaves=5, occupancy=0.3)
        elif kind == "shapes":
            vox = gen_shapes(n, seed * 100 + i, count=max(50, n * n // 100), rmin=2.0,
                             rmax=max(4.0, n / 25.0))
        else:
            vox = gen_cave(n, seed * 100 + i, occupancy=0.45)
        scenes.append({"voxels": vox, "palette": gen_palette(seed * 100 + i), "kind": kind,
                       "n": n})
    views = []
    for v in range(n_views):
        si = v % n_scenes
        n = scenes[si]["n"]
        area = math.exp(rng.uniform(math.log(min_px), math.log(max_px)))
        aspect = 16.0 / 9.0 if rng.random() < 0.5 else 4.0 / 3.0
        h = max(1, int(round(math.sqrt(area / aspect))))
        w = max(1, int(round(h * aspect)))
        spp = int(rng.integers(1, max_spp + 1))
        # caves are viewed from inside, the rest from outside the grid
        if scenes[si]["kind"] == "cave":
            eye = tuple(float(x) for x in rng.uniform(0.3 * n, 0.7 * n, 3))
            target = tuple(float(x) for x in rng.uniform(0.0, n, 3))
        else:
            eye, target = seeded_pose((n, n, n), seed * 1000 + v, float(rng.uniform(0.9, 1.6)) * n)
        cam = camera_look_at(eye, target, (0.0, 1.0, 0.0), 60.0, w, h)
        light = seeded_light(seed * 1000 + v, shadows=bool(rng.random() < 0.5))
        views.append({"scene": si, "camera": cam, "spp": spp, "seed": seed * 7 + v,
                      "view_id": v, "light": light})
    return scenes, views


def serving_scenes(n_scenes=32, seed=5, lo=128, hi=1024):
    """Scene sizes log-uniform in [lo, hi] (multiples of 8); shapes and terrain everywhere, caves
    for the small ones (their noise is the slowest generator)."""
    rng = np.random.default_rng(seed)
    scenes = []
    for i in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))) / 8.0)) * 8
        kind = ["shapes", "terrain", "cave"][i % 3]
        if kind == "cave" and n > 256:
            kind = "shapes"
        if kind == "terrain":
            vox = gen_terrain(n, seed * 1000 + i, octaves=5, occupancy=0.3)
        elif kind == "shapes":
            vox = gen_shapes(n, seed * 1000 + i, count=max(50, n * n // 100), rmin=2.0,
                             rmax=max(4.0, n / 25.0))
        else:
            vox = gen_cave(n, seed * 1000 + i, occupancy=0.45)
        scenes.append({"voxels": vox, "palette": gen_palette(seed * 1000 + i), "kind": kind, "n": n})
    return scenes


def serving_requests(scenes, count, rate=2000.0, seed=6, min_px=320 * 240, max_px=1920 * 1080,
                     max_spp=8):
    """`count` requests with Poisson arrival times (seconds from 0) at mean `rate` per second."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    reqs = []
    for k in range(count):
        si = int(rng.integers(0, len(scenes)))
        n = scenes[si]["n"]
        area = math.exp(rng.uniform(math.log(min_px), math.log(max_px)))
        aspect = 16.0 / 9.0 if rng.random() < 0.5 else 4.0 / 3.0
        h = max(1, int(round(math.sqrt(area / aspect))))
        w = max(1, int(round(h * aspect)))
        if scenes[si]["kind"] == "cave":
            eye = tuple(float(x) for x in rng.uniform(0.3 * n, 0.7 * n, 3))
            target = tuple(float(x) for x in rng.uniform(0.0, n, 3))
        else:
            eye, target = seeded_pose((n, n, n), seed * 100000 + k, float(rng.uniform(0.9, 1.6)) * n)
        reqs.append({"t": float(t[k]), "scene": si,
                     "camera": camera_look_at(eye, target, (0.0, 1.0, 0.0), 60.0, w, h),
                     "spp": int(rng.integers(1, max_spp + 1)), "seed": k, "view_id": k,
                     "light": seeded_light(seed * 100000 + k, shadows=False)})
    return reqs
