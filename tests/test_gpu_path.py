"""Path tracing on the device against the oracle's restatement of the estimator: bit-identical
float radiance and RGBA8, the same ray count, on u8 and RGBA8 grids."""
import ctypes

import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import pyoracle as po
from vtrace_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def oracle_params(p):
    return po.make_path_params(p.spp, p.max_bounces, p.seed, list(p.sky), list(p.sun_dir),
                               list(p.sun))


@pytest.fixture(params=[(1, 32, 0), (1, 4, 0), (0, 32, 0), (1, 8, 1)],
                ids=["persistent", "refill4", "per_pixel", "wavefront"])
def form(request, torch):
    saved = vt.get_tuning(vt.KERNEL_PATH)
    vt.set_tuning(vt.KERNEL_PATH, request.param[1], 0, bool(request.param[0]), bool(request.param[2]))
    yield request.param
    vt.set_tuning(vt.KERNEL_PATH, **saved)


@pytest.mark.parametrize("case", ["terrain", "shapes", "nosun", "deep"])
def test_path_trace_matches_oracle(torch, form, case):
    if case == "shapes":
        w = workloads.shapes1024(n=128, width=80, height=60, count=60)
        p = vt.make_path_params(spp=3, max_bounces=3, seed=5)
    elif case == "nosun":
        w = workloads.terrain256(n=64, width=64, height=48)
        p = vt.make_path_params(spp=2, max_bounces=2, seed=2, sun=(0.0, 0.0, 0.0))
    elif case == "deep":
        w = workloads.cave512(n=64, rays=1)
        w["camera"] = vt.camera_look_at((20.0, 30.0, 24.0), (40.0, 28.0, 50.0), (0, 1, 0), 70.0, 48, 40)
        p = vt.make_path_params(spp=2, max_bounces=8, seed=11)
    else:
        w = workloads.terrain256(n=64, width=72, height=54)
        p = vt.make_path_params(spp=4, max_bounces=3, seed=9)
    cam = w["camera"]
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    try:
        d_out = torch.zeros(cam.width * cam.height * 16, dtype=torch.uint8, device="cuda")
        d_rays = torch.zeros(1, dtype=torch.int64, device="cuda")
        vt.path_trace(g, cam, p, d_out, d_rays)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.float32).reshape(cam.height, cam.width, 4)
        want, rays = po.path_trace(po.Grid(w["voxels"], w["palette"]),
                                   po.make_camera(cam.as_dict()), oracle_params(p))
        bad = np.nonzero((got != want).any(-1))
        assert len(bad[0]) == 0, (case, len(bad[0]), got[bad][:2], want[bad][:2])
        assert int(d_rays.item()) == rays
        assert rays > cam.width * cam.height * p.spp
        # RGBA8 output and the synchronous host form
        p.out_format = vt.PATH_OUT_RGBA8
        img8, rays8 = vt.path_trace_host(g, cam, p)
        np.testing.assert_array_equal(img8, po.path_rgba8(want))
        assert rays8 == rays
    finally:
        g.destroy()


def test_path_trace_rgba8_grid_and_determinism(torch, form):
    rng = np.random.default_rng(8)
    n = 40
    tex = np.zeros((n, n, n), np.uint32)
    tex[:10] = 0xFF3080C0
    solid = rng.random((n, n, n)) < 0.03
    tex[solid] = rng.integers(0, 2**24, int(solid.sum()), dtype=np.uint64).astype(np.uint32) | np.uint32(0xFF000000)
    cam = vt.camera_look_at((-20.0, 45.0, -25.0), (20.0, 10.0, 20.0), (0, 1, 0), 60.0, 56, 42)
    p = vt.make_path_params(spp=2, max_bounces=4, seed=1)
    g = vt.Grid.from_rgba8(tex)
    try:
        a, ra = vt.path_trace_host(g, cam, p)
        b, rb = vt.path_trace_host(g, cam, p)
        np.testing.assert_array_equal(a, b)
        assert ra == rb
        want, rays = po.path_trace(po.Grid(texels=tex), po.make_camera(cam.as_dict()), oracle_params(p))
        np.testing.assert_array_equal(a, want)
        assert ra == rays
        p.seed = 2
        c, _ = vt.path_trace_host(g, cam, p)
        assert (c != a).any()
        # more samples than one chunk of the persistent form's sample buffer holds per pixel
        p.seed, p.spp, p.max_bounces = 3, 37, 1
        big, rb = vt.path_trace_host(g, cam, p)
        want, rays = po.path_trace(po.Grid(texels=tex), po.make_camera(cam.as_dict()), oracle_params(p))
        np.testing.assert_array_equal(big, want)
        assert rb == rays
        with pytest.raises(vt.VtError):
            p.spp = 0
            vt.path_trace_host(g, cam, p)
        # 2^32 pixels: refused before any buffer is touched (here an output far too small)
        p.spp = 1
        huge = vt.camera_look_at((-20.0, 45.0, -25.0), (20.0, 10.0, 20.0), (0, 1, 0), 60.0, 65536, 65536)
        tiny = torch.zeros(256, dtype=torch.uint8, device="cuda")
        assert vt.lib().vt_path_trace(g.id, ctypes.byref(huge), ctypes.byref(p), tiny.data_ptr(),
                                      None, None) == -9  # VT_ELIMIT
    finally:
        g.destroy()
