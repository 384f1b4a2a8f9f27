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


def _value_noise2(x, z, seed, cell):
    """Smooth 2D value noise in [0, 1) at integer coordinates (numpy arrays), lattice spacing
    `cell`, from a seeded integer hash."""
    def h(ix, iz):
        v = (ix.astype(np.int64) * 374761393 + iz.astype(np.int64) * 668265263 + seed * 2246822519)
        v = (v ^ (v >> 13)) * 1274126177
        return ((v ^ (v >> 16)) & 0xFFFF).astype(np.float64) / 65536.0
    fx, fz = x / cell, z / cell
    ix, iz = np.floor(fx).astype(np.int64), np.floor(fz).astype(np.int64)
    ux, uz = fx - ix, fz - iz
    ux, uz = ux * ux * (3 - 2 * ux), uz * uz * (3 - 2 * uz)
    a, b = h(ix, iz), h(ix + 1, iz)
    c, d = h(ix, iz + 1), h(ix + 1, iz + 1)
    return (a + (b - a) * ux) + ((c + (d - c) * ux) - (a + (b - a) * ux)) * uz


def pager_world(load_dist=10, chunk=16, seed=7, entity_sizes=(40, 50), width=1000, height=1000):
    """The shape of vtrace's own world (src/world.rs:136-190, src/gen/pager.rs): terrain chunks of
    chunk^3 voxels on a 2-unit lattice within `load_dist` chunks of the camera's chunk, one texture
    and one instance (translate * scale 2) per chunk holding any voxel, and 11 x 11 entity
    instances (unit cubes at (1.5 x, -5, 1.5 z)) alternating two voxel models.  Terrain is a
    seeded value-noise heightfield (the build's own content).  Returns textures (x-fastest RGBA8
    [z, y, x] uint32 arrays), instances (column-major float32 [n, 16] with the texture index in
    the bits of element 15), and the perspective and camera matrices of src/render.rs:190-214."""
    rng = np.random.default_rng(seed)
    pal = gen_palette(seed)
    R = load_dist
    textures, instances = [], []

    def inst(tx, ty, tz, s, tid):
        m = np.zeros(16, np.float32)
        m[0] = m[5] = m[10] = s
        m[12], m[13], m[14] = tx, ty, tz
        m[15] = np.array([tid], np.int32).view(np.float32)[0]
        return m

    # entity models: random blobs of boxes (stand-ins for the .vox assets, 40^3 and 50^3)
    ent = []
    for n in entity_sizes:
        t = np.zeros((n, n, n), np.uint32)
        for _ in range(12):
            lo = rng.integers(0, n - 4, 3)
            hi = np.minimum(lo + rng.integers(3, max(4, n // 3), 3), n)
            t[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = pal[int(rng.integers(1, 256))] | 0xFF000000
        ent.append(len(textures))
        textures.append(t)
    for x in range(-5, 6):
        for z in range(-5, 6):
            instances.append(inst(x * 1.5, -5.0, z * 1.5, 1.0, ent[0] if (x + z + 10) % 2 == 0 else ent[1]))
    # terrain: height in voxels over the world's voxel columns (8 voxels per world unit)
    vox_per_unit = chunk / 2.0
    span = np.arange(-R * chunk, (R + 1) * chunk)
    gx, gz = np.meshgrid(span, span, indexing="xy")  # [z, x]
    hgt = (-8.0 + 40.0 * _value_noise2(gx, gz, seed, 48.0) + 10.0 * _value_noise2(gx, gz, seed + 1, 13.0))
    ys = np.arange(chunk)
    for cz in range(-R, R + 1):
        for cy in range(-R, R + 1):
            for cx in range(-R, R + 1):
                h = hgt[(cz + R) * chunk:(cz + R + 1) * chunk, (cx + R) * chunk:(cx + R + 1) * chunk]
                vy = cy * chunk + ys
                solid = vy[:, None, None] < h[None, :, :]          # [y, z, x]
                if not solid.any():
                    continue
                depth = h[None, :, :] - vy[:, None, None]
                idx = np.clip((depth * 3).astype(np.int64) % 255 + 1, 1, 255)
                t = np.where(solid, pal[idx] | np.uint32(0xFF000000), 0).astype(np.uint32)
                textures.append(np.ascontiguousarray(t.transpose(1, 0, 2)))  # [z, y, x]
                instances.append(inst(cx * 2.0, cy * 2.0, cz * 2.0, 2.0, len(textures) - 1))
    from math import tan
    fov = 80.0 / 180.0 * 3.1415926
    f = 1.0 / tan(fov / 2.0)
    near, far = 0.01, 10000.0
    P = np.zeros(16, np.float32)
    P[0], P[5] = f / (width / height), f
    P[10], P[11], P[14] = (far + near) / (near - far), -1.0, 2.0 * far * near / (near - far)
    eye = np.array([0.3, float(hgt[R * chunk, R * chunk]) / vox_per_unit + 2.5, 0.2])
    d = np.array([0.8, -0.35, 0.45])
    d /= np.linalg.norm(d)
    s = np.cross(d, [0.0, 1.0, 0.0])
    s /= np.linalg.norm(s)
    u = np.cross(s, d)
    C = np.eye(4)
    C[0, :3], C[1, :3], C[2, :3] = s, u, -d
    C[:3, 3] = [-s @ eye, -u @ eye, d @ eye]
    C = np.ascontiguousarray(C.T, np.float32).reshape(16)
    return {"name": "pager_world_r%d" % R, "textures": textures,
            "instances": np.stack(instances).astype(np.float32), "P": P, "C": C,
            "width": width, "height": height}
