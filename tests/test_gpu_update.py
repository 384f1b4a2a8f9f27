"""Chunk paging (vt_grid_update): after any sequence of box writes the grid holds exactly what a
fresh build of the updated dense array holds — occupancy, payloads (through the directory's
slots), distances, octant words — and traces bit-identically to the oracle."""
import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import pyoracle as po
from test_gpu_parity import assert_hits_equal, device_render, device_trace, oracle_camera

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def same_as_fresh(g, fresh):
    a, b = g.info(), fresh.info()
    for k in ("nx", "ny", "nz", "bricks_total", "bricks_nonempty", "voxels_occupied", "payload_format"):
        assert a[k] == b[k], k
    da, ma = g.bricks()
    db, mb = fresh.bricks()
    empty_a, empty_b = (da & 0x80000000) != 0, (db & 0x80000000) != 0
    np.testing.assert_array_equal(empty_a, empty_b)
    np.testing.assert_array_equal(da[empty_a], db[empty_b])  # distances
    full = np.nonzero(~empty_a)[0]
    # the update's slots are not the fresh build's: compare masks through the directory
    np.testing.assert_array_equal(ma[da[full]], mb[db[full]])
    assert len(np.unique(da[full])) == len(full)  # no slot shared by two bricks
    np.testing.assert_array_equal(g.octants(), fresh.octants())
    np.testing.assert_array_equal(g.long_boxes(), fresh.long_boxes())


def random_box(rng, dims, max_edge):
    nx, ny, nz = dims
    w, h, d = (int(rng.integers(1, min(max_edge, n) + 1)) for n in (nx, ny, nz))
    x0, y0, z0 = int(rng.integers(0, nx - w + 1)), int(rng.integers(0, ny - h + 1)), int(rng.integers(0, nz - d + 1))
    return (x0, y0, z0), (w, h, d)


def test_update_sequence_matches_fresh_builds(torch):
    rng = np.random.default_rng(21)
    nx, ny, nz = 100, 70, 90
    vox = vt.gen_terrain((nx, ny, nz), 3, occupancy=0.25)
    pal = vt.gen_palette(3)
    pal[7] &= 0x00FFFFFF  # an index whose colour is transparent: stored, not occupied
    g = vt.Grid.from_u8(vox, pal)
    cam = vt.camera_look_at((-40.0, 120.0, -50.0), (50.0, 20.0, 45.0), (0, 1, 0), 60.0, 120, 90)
    try:
        for step in range(14):
            kind = step % 4
            if kind == 0:    # a 16^3 chunk on the chunk lattice
                org = tuple(int(rng.integers(0, n // 16)) * 16 for n in (nx, ny, nz))
                size = tuple(min(16, n - o) for n, o in zip((nx, ny, nz), org))
            else:
                org, size = random_box(rng, (nx, ny, nz), 40)
            w, h, d = size
            if kind == 1:    # clear
                box = np.zeros((d, h, w), np.uint8)
            else:
                box = np.where(rng.random((d, h, w)) < 0.3, rng.integers(1, 256, (d, h, w)), 0).astype(np.uint8)
            x0, y0, z0 = org
            vox[z0:z0 + d, y0:y0 + h, x0:x0 + w] = box
            if kind == 3:    # a z-fastest chunk, as the Rust host stores them
                g.update(org, np.ascontiguousarray(box.transpose(2, 1, 0)), vt.ORDER_Z_FASTEST)
            else:
                g.update(org, box)
            fresh = vt.Grid.from_u8(vox, pal)
            try:
                same_as_fresh(g, fresh)
            finally:
                fresh.destroy()
            if step % 5 == 4:
                og = po.Grid(vox, pal)
                img, _ = device_render(torch, g, cam, None)
                assert_hits_equal(img, po.render(og, oracle_camera(cam)), "render after step %d" % step)
                rays = vt.gen_rays_uniform((nx, ny, nz), step, 50000)
                hits, _, _ = device_trace(torch, g, rays)
                assert_hits_equal(hits, po.trace_rays(og, rays), "rays after step %d" % step)
        # the whole grid at once, then all empty
        vox[:] = np.where(rng.random(vox.shape) < 0.05, 9, 0)
        g.update((0, 0, 0), vox)
        fresh = vt.Grid.from_u8(vox, pal)
        same_as_fresh(g, fresh)
        fresh.destroy()
        vox[:] = 0
        g.update((0, 0, 0), vox)
        assert g.info()["bricks_nonempty"] == 0 and g.info()["voxels_occupied"] == 0
    finally:
        g.destroy()


def test_paging_into_an_empty_rgba8_world_grows_slots(torch):
    rng = np.random.default_rng(5)
    n = 64
    world = np.zeros((n, n, n), np.uint32)
    g = vt.Grid.from_rgba8(world)
    try:
        assert g.info()["bricks_nonempty"] == 0
        for cz in range(0, n, 16):
            for cx in range(0, n, 16):
                chunk = np.where(rng.random((16, 16, 16)) < 0.2,
                                 rng.integers(0, 2**32, (16, 16, 16), dtype=np.uint64).astype(np.uint32) | np.uint32(0x01000000),
                                 0).astype(np.uint32)
                world[cz:cz + 16, 8:24, cx:cx + 16] = chunk
                g.update((cx, 8, cz), chunk)
        fresh = vt.Grid.from_rgba8(world)
        try:
            same_as_fresh(g, fresh)
        finally:
            fresh.destroy()
        rays = vt.gen_rays_uniform((n, n, n), 2, 40000)
        hits, _, _ = device_trace(torch, g, rays)
        assert_hits_equal(hits, po.trace_rays(po.Grid(texels=world), rays), "paged rgba8 world")
    finally:
        g.destroy()


def test_update_errors(torch):
    g = vt.Grid.from_u8(np.zeros((16, 16, 16), np.uint8), vt.gen_palette(1))
    try:
        with pytest.raises(vt.VtError) as e:
            g.update((10, 0, 0), np.ones((4, 4, 8), np.uint8))  # x0 + w = 18 > 16
        assert e.value.code == -1
        import torch as t
        buf = t.zeros(8 * 8 * 16, dtype=t.uint8, device="cuda")
        b = vt.Batch([vt.make_view(g, vt.camera_look_at((-8, 20, -8), (8, 8, 8), (0, 1, 0), 60.0, 8, 8), buf, 1, 0, 0, None)])
        with pytest.raises(vt.VtError) as e:
            g.update((0, 0, 0), np.ones((4, 4, 4), np.uint8))
        assert e.value.code == -6  # VT_EBUSY
        b.destroy()
        g.update((0, 0, 0), np.ones((4, 4, 4), np.uint8))
    finally:
        g.destroy()
