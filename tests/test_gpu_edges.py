"""Edge cases of the traversal against the oracle: single-voxel and fully solid grids, grids one
brick thick and 65535 voxels long, axis-aligned light (shadow rays with zero components), 1-pixel
images, empty ray buffers, non-finite and far-away rays."""
import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import pyoracle as po
from test_gpu_parity import (assert_hits_equal, device_render, device_trace, oracle_camera,
                             oracle_light, special_rays)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def check_rays(torch, vox, pal, rays, what):
    g = vt.Grid.from_u8(vox, pal)
    try:
        hits, _, _ = device_trace(torch, g, rays)
        assert_hits_equal(hits, po.trace_rays(po.Grid(vox, pal), rays), what)
        return hits
    finally:
        g.destroy()


@pytest.mark.parametrize("solid", [0, 1])
def test_single_voxel_grid(torch, solid):
    vox = np.full((1, 1, 1), 5 * solid, np.uint8)
    rng = np.random.default_rng(solid)
    rays = special_rays(rng, (1, 1, 1), 30000)
    hits = check_rays(torch, vox, vt.gen_palette(2), rays, "1^3 grid solid=%d" % solid)
    assert ((hits["face"] & vt.FLAG_HIT) != 0).any() == bool(solid)


def test_fully_solid_grid(torch):
    vox = np.full((24, 16, 40), 7, np.uint8)
    rng = np.random.default_rng(3)
    rays = np.concatenate([special_rays(rng, (40, 16, 24), 40000),
                           vt.gen_rays_uniform((40, 16, 24), 3, 40000)])
    hits = check_rays(torch, vox, vt.gen_palette(3), rays, "solid grid")
    inside = (hits["face"] & 7) == 0
    assert inside.any() and (~inside & ((hits["face"] & vt.FLAG_HIT) != 0)).any()


@pytest.mark.parametrize("dims", [(65535, 1, 3), (8, 8, 4096), (4096, 9, 8)])
def test_long_thin_grids(torch, dims):
    nx, ny, nz = dims
    rng = np.random.default_rng(nx + nz)
    vox = np.zeros((nz, ny, nx), np.uint8)
    # sparse solid specks and one wall, so rays cross long empty runs between them
    n = max(8, nx * ny * nz // 4000)
    vox[rng.integers(0, nz, n), rng.integers(0, ny, n), rng.integers(0, nx, n)] = 9
    vox[nz // 2:, :, nx // 3] = 3
    rays = np.concatenate([special_rays(rng, dims, 40000), vt.gen_rays_uniform(dims, 5, 40000)])
    # and rays along the long axis from one end
    long_axis = int(np.argmax(dims))
    o = rng.random((2000, 3)).astype(np.float32) * np.array(dims, np.float32)
    o[:, long_axis] = -3.0
    d = np.zeros((2000, 3), np.float32)
    d[:, long_axis] = 1.0
    d[1000:] += rng.normal(scale=1e-3, size=(1000, 3)).astype(np.float32)
    rays = np.concatenate([rays, np.concatenate([o, d], 1)]).astype(np.float32)
    check_rays(torch, vox, vt.gen_palette(4), rays, "thin grid %r" % (dims,))


def test_axis_aligned_light_and_one_pixel_images(torch):
    w = vt.gen_terrain(64, 8, occupancy=0.35)
    pal = vt.gen_palette(8)
    g = vt.Grid.from_u8(w, pal)
    og = po.Grid(w, pal)
    try:
        light = vt.make_light((0.0, 1.0, 0.0), 0.25, True)  # shadow rays straight up
        for (W, H) in ((1, 1), (1, 37), (53, 1), (80, 60)):
            cam = vt.camera_look_at((-20.0, 90.0, -30.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0, W, H)
            img, _ = device_render(torch, g, cam, light)
            assert_hits_equal(img, po.render(og, oracle_camera(cam), oracle_light(light)),
                              "%dx%d axis light" % (W, H))
        assert ((img["face"] & vt.FLAG_SHADOW_RAY) != 0).any()
    finally:
        g.destroy()


def test_empty_and_degenerate_ray_buffers(torch):
    vox = vt.gen_shapes(48, 2, count=20, rmin=2.0, rmax=8.0)
    pal = vt.gen_palette(2)
    g = vt.Grid.from_u8(vox, pal)
    try:
        buf = torch.empty(16, dtype=torch.uint8, device="cuda")
        vt.trace_rays(g, buf, 0, buf)  # n = 0: nothing to do
        torch.cuda.synchronize()
        rays = np.array([
            [np.nan, 1, 1, 1, 0, 0], [1, 1, 1, np.inf, 0, 0], [1, 1, 1, 0, 0, 0],
            [1e30, 1e30, 1e30, -1, -1, -1], [-1e30, 24, 24, 1, 0, 0], [24, 24, 24, 1e-30, 1e-30, 1],
            [0, 0, 0, 1, 1, 1], [48, 48, 48, -1, -1, -1], [24, 48, 24, 0, -1, 0],
        ], np.float32)
        hits, _, _ = device_trace(torch, g, rays)
        assert_hits_equal(hits, po.trace_rays(po.Grid(vox, pal), rays), "degenerate rays")
        assert hits["face"][0] & vt.FLAG_INVALID and hits["face"][1] & vt.FLAG_INVALID
    finally:
        g.destroy()
