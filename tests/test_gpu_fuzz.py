"""Seeded randomized parity sweep: many small scenes of every generator at odd sizes (not multiples
of 8 or of each other), cameras outside and inside the grid in every direction, lights with and
without shadow rays, every render launch form and warp-tile shape, and ray buffers mixing uniform
rays with the DDA's edge cases (axis-parallel and planar directions, zero components, origins on
voxel faces and grid faces, rays from outside that graze or miss the box).  Every record, all 16
bytes, must equal the oracle's."""
import numpy as np
import pytest

import vtrace_gb300 as vt
from vtrace_gb300 import autotune, workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

CASES = 48


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def random_grid(rng):
    dims = tuple(int(x) for x in rng.integers(9, 90, 3))
    kind = int(rng.integers(0, 3))
    seed = int(rng.integers(0, 1 << 30))
    if kind == 0:
        vox = vt.gen_terrain(dims, seed, octaves=4, occupancy=float(rng.uniform(0.1, 0.6)))
    elif kind == 1:
        vox = vt.gen_shapes(dims, seed, count=int(rng.integers(3, 60)), rmin=1.0,
                            rmax=float(rng.uniform(2.0, 12.0)))
    else:
        vox = vt.gen_cave(dims, seed, occupancy=float(rng.uniform(0.2, 0.6)))
    return vox, vt.gen_palette(seed)


def random_camera(rng, dims):
    nx, ny, nz = dims
    c = np.array([nx, ny, nz], np.float64) / 2.0
    if rng.random() < 0.3:  # inside the grid
        eye = rng.uniform(0.1, 0.9, 3) * np.array([nx, ny, nz])
    else:
        d = rng.normal(size=3)
        eye = c + d / np.linalg.norm(d) * float(rng.uniform(0.8, 2.5)) * max(dims)
    target = c + rng.normal(size=3) * max(dims) * 0.2
    w, h = int(rng.integers(5, 70)), int(rng.integers(3, 50))
    return vt.camera_look_at(tuple(eye), tuple(target), (0.0, 1.0, 0.0),
                             float(rng.uniform(30.0, 100.0)), w, h)


def edge_rays(rng, dims, n):
    nx, ny, nz = dims
    size = np.array([nx, ny, nz], np.float32)
    o = (rng.uniform(0, 1, (n, 3)) * size).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    k = rng.integers(0, 8, n)
    # origins snapped onto voxel faces / the grid's faces
    o[k == 1] = np.floor(o[k == 1])
    o[k == 2, 0] = 0.0
    o[k == 3, 1] = size[1]
    # axis-parallel and planar directions, exact diagonals
    d[k == 4] = np.eye(3, dtype=np.float32)[rng.integers(0, 3, int((k == 4).sum()))] * \
        rng.choice([-1.0, 1.0], (int((k == 4).sum()), 1)).astype(np.float32)
    d[k == 5, int(rng.integers(0, 3))] = 0.0
    d[k == 6] = np.sign(rng.normal(size=(int((k == 6).sum()), 3))).astype(np.float32)
    # from outside, aimed at random points of the box or beside it
    m = k == 7
    o[m] = (rng.uniform(-1.0, 2.0, (int(m.sum()), 3)) * size).astype(np.float32)
    d[m] = (rng.uniform(-0.2, 1.2, (int(m.sum()), 3)) * size - o[m]).astype(np.float32)
    return np.concatenate([o, d], 1).astype(np.float32)


def assert_same(got, want, what):
    g = np.ascontiguousarray(got).view(np.uint8).reshape(-1, 16)
    w = np.ascontiguousarray(want).view(np.uint8).reshape(-1, 16)
    bad = np.nonzero((g != w).any(1))[0]
    assert len(bad) == 0, "%s: %d of %d records differ; first %d: got %r want %r" % (
        what, len(bad), len(g), bad[0], got.reshape(-1)[bad[0]], want.reshape(-1)[bad[0]])


FORMS = [autotune.tuning(tile_shape=t, block_warps=w) for t, w in
         [(vt.TILE_8X4, 4), (vt.TILE_4X8, 2), (vt.TILE_16X2, 8), (vt.TILE_32X1, 1)]]
FORMS += [autotune.tuning(wavefront=True), autotune.tuning(refill_min=8, persistent=True),
          autotune.tuning(persistent=True, wavefront=True)]


def test_random_scenes_cameras_and_launch_forms(torch):
    rng = np.random.default_rng(20261204)
    saved = vt.get_tuning(vt.KERNEL_RENDER)
    try:
        for case in range(CASES):
            vox, pal = random_grid(rng)
            dims = vox.shape[::-1]
            g = vt.Grid.from_u8(vox, pal)
            og = po.Grid(vox, pal)
            try:
                cam = random_camera(rng, dims)
                light = workloads.seeded_light(int(rng.integers(0, 1000)),
                                               shadows=bool(rng.random() < 0.7))
                form = FORMS[case % len(FORMS)]
                autotune.install(vt.KERNEL_RENDER, form)
                d = torch.full((cam.width * cam.height * 16,), 0xCD, dtype=torch.uint8,
                               device="cuda")
                vt.render(g, cam, light, d)
                torch.cuda.synchronize()
                want = po.render(og, po.make_camera(cam.as_dict()),
                                 po.make_light(list(light.dir), light.ambient,
                                               bool(light.shadows)))
                assert_same(d.cpu().numpy().view(vt.HIT_DTYPE), want,
                            "case %d %r render %s" % (case, dims,
                                                      autotune.key(vt.KERNEL_RENDER, form)))
                rays = edge_rays(rng, dims, 4000)
                d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
                d_hits = torch.empty(rays.shape[0] * 16, dtype=torch.uint8, device="cuda")
                vt.trace_rays(g, d_rays, rays.shape[0], d_hits)
                torch.cuda.synchronize()
                assert_same(d_hits.cpu().numpy().view(vt.HIT_DTYPE), po.trace_rays(og, rays),
                            "case %d %r rays" % (case, dims))
            finally:
                g.destroy()
    finally:
        vt.set_tuning(vt.KERNEL_RENDER, **saved)
