"""Dense-input orders and .vox models on the device: z-fastest chunks (src/voxel/rawchunk.rs:292)
give the same bricks as the x-fastest array they transpose to, and a .vox model passed through
add_texture renders as the oracle's restatement of the reference frame."""
import ctypes

import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import pyoracle as po
from oracle import vox as ovox
from test_gpu_compat import instance, look_at, perspective
from test_gpu_parity import assert_hits_equal, device_render, oracle_camera

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def same_grid(a, b):
    assert a.info() == b.info()
    da, ma = a.bricks()
    db, mb = b.bricks()
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ma, mb)
    np.testing.assert_array_equal(a.octants(), b.octants())


@pytest.mark.parametrize("dims", [(64, 64, 64), (37, 20, 45), (100, 3, 9), (8, 70, 33)])
def test_z_fastest_u8_chunk_matches_x_fastest(torch, dims):
    nx, ny, nz = dims
    rng = np.random.default_rng(nx * 7 + ny)
    vox = np.where(rng.random((nz, ny, nx)) < 0.07, rng.integers(1, 256, (nz, ny, nx)), 0)
    vox = vox.astype(np.uint8)
    pal = vt.gen_palette(5)
    chunk = np.ascontiguousarray(vox.transpose(2, 1, 0))  # [x, y, z], z fastest
    ga, gb = vt.Grid.from_u8(vox, pal), vt.Grid.from_chunk(chunk, pal)
    try:
        same_grid(ga, gb)
        cam = vt.camera_look_at((-0.6 * nx, 1.3 * ny + 5, -0.4 * nz), (nx / 2, ny / 2, nz / 2),
                                (0, 1, 0), 60.0, 96, 64)
        img, _ = device_render(torch, gb, cam, None)
        assert_hits_equal(img, po.render(po.Grid(vox, pal), oracle_camera(cam)), "chunk %r" % (dims,))
        assert ((img["face"] & vt.FLAG_HIT) != 0).any()
    finally:
        ga.destroy()
        gb.destroy()


def test_z_fastest_rgba8_chunk_matches_x_fastest(torch):
    rng = np.random.default_rng(11)
    nx, ny, nz = 50, 33, 41
    tex = rng.integers(0, 2**32, (nz, ny, nx), dtype=np.uint64).astype(np.uint32)
    tex[rng.random((nz, ny, nx)) < 0.9] &= np.uint32(0x00FFFFFF)  # alpha 0: empty
    ga = vt.Grid.from_rgba8(tex)
    gb = vt.Grid.from_chunk(np.ascontiguousarray(tex.transpose(2, 1, 0)))
    try:
        same_grid(ga, gb)
    finally:
        ga.destroy()
        gb.destroy()


def test_vox_model_through_add_texture(torch):
    """world.rs:65-70 + render.rs:246-261: the first model of a .vox file becomes a texture via
    add_texture (which reads the z-fastest chunk x-fastest), drawn by render_tick."""
    rng = np.random.default_rng(4)
    n = 24
    cells = rng.choice(n ** 3, 1500, replace=False)
    vox = np.stack([cells // (n * n), (cells // n) % n, cells % n, rng.integers(1, 256, 1500)], 1)
    pal = rng.integers(0, 2**32, 256, dtype=np.uint64).astype(np.uint32) | np.uint32(0xFF000000)
    buf = ovox.write([((n, n, n), vox.astype(np.uint8))], pal)
    chunk = vt.vox_model_chunk(buf)  # [x, y, z, 4]
    L = vt.lib()
    assert L.entry() == 0
    try:
        tid = L.add_texture(chunk.ctypes.data, n, n, n)
        assert tid >= 0
        insts = np.stack([instance(25, (0, 1, 0), (3, 3, 3), (0, -0.5, -6), tid),
                          instance(-40, (1, 0, 1), (2, 2, 2), (2.5, 1.0, -8), tid)])
        ptr = L.start_update_instances(len(insts))
        ctypes.memmove(ptr, insts.ctypes.data, insts.nbytes)
        assert L.end_update_instances(len(insts)) == 0
        P = perspective(80.0 / 180.0 * 3.1415926, 1.0, 0.01, 10000.0)
        C = look_at((0.3, 1.2, 1.5), (0.5, 0.0, -7.0), (0.0, 1.0, 0.0))
        info = vt.RenderTickInfo(P.ctypes.data, C.ctypes.data)
        w, h = ctypes.c_int32(0), ctypes.c_int32(0)
        assert L.render_tick(ctypes.byref(w), ctypes.byref(h), ctypes.byref(info)) == 0
        fb = np.zeros((h.value, w.value, 4), np.uint8)
        assert L.vt_framebuffer_download(fb.ctypes.data, fb.nbytes) == 0
        # the GPU image the copy makes: the chunk's bytes read x-fastest with (w, h, d) = size
        texels = chunk.view(np.uint32).reshape(-1).reshape(n, n, n)
        want = po.compat_render([po.Grid(texels=texels)], insts, P, C, w.value, h.value)
        assert (fb != want).any(-1).sum() == 0
        assert (fb != np.array([0xC0, 0xE8, 0xF6, 0xFF], np.uint8)).any(-1).mean() > 0.02
    finally:
        L.cleanup()
