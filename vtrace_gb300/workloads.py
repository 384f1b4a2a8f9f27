"""Seeded synthetic workloads of the benchmark configurations.

Each builder returns host-side inputs only (numpy voxel grids, palettes, camera and light
structs, ray arrays); uploading them is the caller's business.  All content is generated by
libvtrace's deterministic host generators; camera and light poses come from numpy's seeded PCG64.

  terrain256   256^3 fBm heightfield (~30% occupancy), 640x480 pinhole camera, 60 deg vertical FOV
  shapes1024   1024^3 with 10,000 boxes and spheres (radius 2-40, ~4-5% occupancy), 1920x1080,
               directional light with one hard-shadow ray per lit hit
  cave512      512^3 3D-noise cave (~45% occupancy), 16,777,216 rays with origins uniform in the
               grid and directions uniform on the sphere
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
