"""The reference-compatible C entry points (entry, add_texture, start/end_update_instances,
render_tick, get_input_data_pointer, cleanup) driven in the order vtrace's Rust host calls them
(src/render.rs:184-320), with the headless framebuffer checked against the oracle."""
import ctypes
import math
import struct

import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def perspective(fov, aspect, near, far):
    """glm::perspective (OpenGL clip conventions), column-major, as src/render.rs:208-210."""
    f = 1.0 / math.tan(fov / 2.0)
    m = np.zeros((4, 4), np.float32)  # m[col][row]
    m[0][0] = f / aspect
    m[1][1] = f
    m[2][2] = (far + near) / (near - far)
    m[2][3] = -1.0
    m[3][2] = 2.0 * far * near / (near - far)
    return m


def look_at(eye, center, up):
    """glm::look_at, column-major, as src/render.rs:212-214."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[:3, 3] = [-s @ eye, -u @ eye, f @ eye]
    return np.ascontiguousarray(m.T, np.float32)  # column-major storage


def instance(rot_deg, axis, scale, translate, texture_id):
    a = math.radians(rot_deg)
    ax = np.asarray(axis, np.float64)
    ax /= np.linalg.norm(ax)
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + math.sin(a) * K + (1 - math.cos(a)) * (K @ K)
    M = np.eye(4)
    M[:3, :3] = R @ np.diag(scale)
    M[:3, 3] = translate
    cm = np.ascontiguousarray(M.T, np.float32).reshape(16)
    cm[15] = struct.unpack("<f", struct.pack("<i", texture_id))[0]  # trace.vert:38
    return cm


@pytest.fixture(scope="module")
def lib():
    import torch
    assert torch.cuda.is_available()
    return vt.lib()


def test_reference_call_sequence(lib):
    L = lib
    assert L.entry() == 0
    rng = np.random.default_rng(3)
    # two textures: x-fastest RGBA8, some translucent texels
    t0 = np.zeros((16, 16, 16, 4), np.uint8)
    solid = rng.random((16, 16, 16)) < 0.08
    t0[solid] = rng.integers(0, 256, (int(solid.sum()), 4), dtype=np.uint8)
    t0[solid, 3] = rng.choice([255, 255, 128, 40], int(solid.sum()))
    t1 = np.zeros((10, 12, 8, 4), np.uint8)  # (z, y, x): 8 x 12 x 10
    t1[2:8, 3:9, 1:7] = (200, 60, 30, 255)
    id0 = L.add_texture(t0.ctypes.data, 16, 16, 16)
    id1 = L.add_texture(t1.ctypes.data, 8, 12, 10)
    assert (id0, id1) == (0, 1)
    insts = np.stack([
        instance(0, (0, 1, 0), (4, 4, 4), (0, 0, -6), 0),
        instance(30, (1, 1, 0), (3, 5, 3), (2.5, -1, -9), 1),
        instance(-20, (0, 0, 1), (6, 6, 6), (-3, 1, -12), 0),
        instance(0, (0, 1, 0), (1, 1, 1), (0, 0, -3), 7),        # unbound texture: not drawn
        instance(0, (0, 1, 0), (50, 50, 50), (0, 0, 0), 1),      # camera inside: culled
        instance(0, (0, 1, 0), (0, 4, 4), (1, 0, -5), 0),         # singular matrix: not drawn
    ])
    ptr = L.start_update_instances(len(insts))
    assert ptr
    ctypes.memmove(ptr, insts.ctypes.data, insts.nbytes)
    assert L.end_update_instances(len(insts)) == 0
    P = perspective(80.0 / 180.0 * 3.1415926, 1.0, 0.01, 10000.0)  # src/render.rs:190,199
    C = look_at((0.5, 0.8, 2.0), (0.0, 0.0, -8.0), (0.0, 1.0, 0.0))
    info = vt.RenderTickInfo(P.ctypes.data, C.ctypes.data)
    w, h = ctypes.c_int32(0), ctypes.c_int32(0)
    assert L.render_tick(ctypes.byref(w), ctypes.byref(h), ctypes.byref(info)) == 0
    assert (w.value, h.value) == (1000, 1000)
    fb = np.zeros((1000, 1000, 4), np.uint8)
    assert L.vt_framebuffer_download(fb.ctypes.data, fb.nbytes) == 0
    grids = [po.Grid(texels=t0.view(np.uint32)[..., 0]), po.Grid(texels=t1.view(np.uint32)[..., 0])]
    want = po.compat_render(grids, insts, P, C, 1000, 1000)
    diff = np.nonzero((fb != want).any(-1))
    assert len(diff[0]) == 0, (len(diff[0]), fb[diff][:3], want[diff][:3])
    sky = np.array([0xC0, 0xE8, 0xF6, 0xFF], np.uint8)
    covered = (fb != sky).any(-1).mean()
    assert 0.01 < covered < 0.9
    inp = L.get_input_data_pointer()
    assert bytes(inp.contents.keys) == b"\0" * 6
    # zero instances are treated as one (lib/memory.c:236,251)
    assert L.start_update_instances(0)
    assert L.end_update_instances(0) == 0
    assert L.render_tick(ctypes.byref(w), ctypes.byref(h), ctypes.byref(info)) == 0
    L.cleanup()
    assert L.render_tick(ctypes.byref(w), ctypes.byref(h), ctypes.byref(info)) == -1
    assert L.add_texture(t0.ctypes.data, 16, 16, 16) == -1


@pytest.mark.parametrize("load_dist,size", [(3, (320, 240)), (5, (256, 320)), (4, (203, 117))])
def test_pager_world_with_instance_culling(lib, monkeypatch, load_dist, size):
    """vtrace's own world shape (src/world.rs:136-190): hundreds of 16^3 terrain chunks around
    the camera, some straddling it, and 121 entities, drawn through the per-tile instance bins;
    the frame equals the oracle's loop over every instance (203 x 117: warps that straddle the
    frame's right and bottom edges)."""
    from vtrace_gb300 import workloads
    w, h = size
    world = workloads.pager_world(load_dist=load_dist, width=w, height=h)
    monkeypatch.setenv("VTRACE_WIDTH", str(w))
    monkeypatch.setenv("VTRACE_HEIGHT", str(h))
    L = lib
    assert L.entry() == 0
    try:
        for t in world["textures"]:
            nz, ny, nx = t.shape
            assert L.add_texture(t.ctypes.data, nx, ny, nz) >= 0
        insts = world["instances"]
        ptr = L.start_update_instances(len(insts))
        ctypes.memmove(ptr, insts.ctypes.data, insts.nbytes)
        assert L.end_update_instances(len(insts)) == 0
        info = vt.RenderTickInfo(world["P"].ctypes.data, world["C"].ctypes.data)
        ww, hh = ctypes.c_int32(0), ctypes.c_int32(0)
        assert L.render_tick(ctypes.byref(ww), ctypes.byref(hh), ctypes.byref(info)) == 0
        assert (ww.value, hh.value) == (w, h)
        fb = np.zeros((h, w, 4), np.uint8)
        assert L.vt_framebuffer_download(fb.ctypes.data, fb.nbytes) == 0
    finally:
        L.cleanup()
    grids = [po.Grid(texels=t) for t in world["textures"]]
    want = po.compat_render(grids, insts, world["P"], world["C"], w, h)
    diff = np.nonzero((fb != want).any(-1))
    assert len(diff[0]) == 0, (len(diff[0]), diff[0][:5], diff[1][:5])
    sky = np.array([0xC0, 0xE8, 0xF6, 0xFF], np.uint8)
    assert 0.05 < (fb != sky).any(-1).mean() < 0.99


def test_random_affine_instances_in_shuffled_order(lib, monkeypatch):
    """Overlapping instances with rotations, non-uniform scales and shears (condition numbers from
    1 to about 4000, so that the per-instance depth bound is both used and switched off), some
    close to the camera, in shuffled draw order so that nearer and farther cubes alternate: every
    pixel (blending and the depth test included) equals the oracle's loop over every instance."""
    rng = np.random.default_rng(31)
    w, h = 160, 120
    monkeypatch.setenv("VTRACE_WIDTH", str(w))
    monkeypatch.setenv("VTRACE_HEIGHT", str(h))
    texs = []
    for k in range(6):
        n = int(rng.integers(6, 20))
        t = np.where(rng.random((n, n, n)) < 0.35,
                     vt.gen_palette(k)[rng.integers(1, 256, (n, n, n))] | 0xFF000000, 0)
        t[rng.random((n, n, n)) < 0.1] &= 0x7FFFFFFF  # half-transparent texels blend
        texs.append(np.ascontiguousarray(t.astype(np.uint32)))
    insts = []
    for i in range(160):
        M = np.eye(4)
        A = rng.normal(size=(3, 3))
        A = np.linalg.qr(A)[0] @ np.diag(rng.uniform(0.3, 3.0, 3))
        if i % 5 == 0:
            A = A @ np.array([[1, rng.uniform(-8, 8), 0], [0, 1, 0], [0, 0, 1]])  # shear
        if i % 17 == 0:
            A = A @ np.diag([1, 1, rng.uniform(0.002, 0.01)])  # nearly flat: large condition
        M[:3, :3] = A
        M[:3, 3] = rng.uniform(-6, 6, 3) + (0.0, 0.0, -8.0 if i % 9 else -1.0)
        cm = np.ascontiguousarray(M.T, np.float32).reshape(16)
        cm[15] = struct.unpack("<f", struct.pack("<i", int(rng.integers(0, len(texs)))))[0]
        insts.append(cm)
    insts = np.ascontiguousarray(np.stack(insts))
    P = perspective(math.radians(80.0), w / h, 0.01, 200.0)
    C = look_at((0.5, 0.8, 4.0), (0.0, 0.0, -8.0), (0.0, 1.0, 0.0))
    L = lib
    assert L.entry() == 0
    try:
        for t in texs:
            nz, ny, nx = t.shape
            assert L.add_texture(t.ctypes.data, nx, ny, nz) >= 0
        ptr = L.start_update_instances(len(insts))
        ctypes.memmove(ptr, insts.ctypes.data, insts.nbytes)
        assert L.end_update_instances(len(insts)) == 0
        info = vt.RenderTickInfo(P.ctypes.data, C.ctypes.data)
        ww, hh = ctypes.c_int32(0), ctypes.c_int32(0)
        assert L.render_tick(ctypes.byref(ww), ctypes.byref(hh), ctypes.byref(info)) == 0
        fb = np.zeros((h, w, 4), np.uint8)
        assert L.vt_framebuffer_download(fb.ctypes.data, fb.nbytes) == 0
    finally:
        L.cleanup()
    grids = [po.Grid(texels=t) for t in texs]
    want = po.compat_render(grids, insts, P.reshape(16), C.reshape(16), w, h)
    diff = np.nonzero((fb != want).any(-1))
    assert len(diff[0]) == 0, (len(diff[0]), diff[0][:5], diff[1][:5])
    assert (fb != np.array([0xC0, 0xE8, 0xF6, 0xFF], np.uint8)).any(-1).mean() > 0.2
