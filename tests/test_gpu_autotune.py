"""The autotuner's search space and the autotuner itself, on the GPU: every warp-tile shape and
block size of the render launch gives the oracle's records, and autotune() picks and installs a
tuning of each entry point after which the records are still the oracle's."""
import numpy as np
import pytest

import vtrace_gb300 as vt
from vtrace_gb300 import autotune, workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def assert_same(got, want, what):
    g = np.ascontiguousarray(got).view(np.uint8).reshape(-1, 16)
    w = np.ascontiguousarray(want).view(np.uint8).reshape(-1, 16)
    bad = int((g != w).any(1).sum())
    assert bad == 0, "%s: %d of %d records differ from the oracle" % (what, bad, len(g))


def oracle_frame(w, light):
    og = po.Grid(w["voxels"], w["palette"])
    return og, po.render(og, po.make_camera(w["camera"].as_dict()),
                         po.make_light(list(light.dir), light.ambient, bool(light.shadows)))


@pytest.fixture(scope="module")
def frame_case(torch):
    # odd image size: partial warp tiles and blocks on both edges for every shape
    w = workloads.terrain256(n=96, width=333, height=203)
    light = workloads.seeded_light(1, shadows=True)
    og, want = oracle_frame(w, light)
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    yield w, light, g, want
    g.destroy()


@pytest.mark.parametrize("tile", [vt.TILE_8X4, vt.TILE_4X8, vt.TILE_16X2, vt.TILE_32X1])
@pytest.mark.parametrize("warps", [1, 2, 4, 8])
def test_render_tile_shapes_agree(torch, frame_case, tile, warps):
    w, light, g, want = frame_case
    saved = vt.get_tuning(vt.KERNEL_RENDER)
    try:
        vt.set_tuning(vt.KERNEL_RENDER, 16, 0, False, False, tile, warps)
        cam = w["camera"]
        d = torch.full((cam.width * cam.height * 16,), 0xAB, dtype=torch.uint8, device="cuda")
        vt.render(g, cam, light, d)
        torch.cuda.synchronize()
        assert_same(d.cpu().numpy().view(vt.HIT_DTYPE), want,
                    "tile %s, %d warps" % (vt.TILE_NAMES[tile], warps))
    finally:
        vt.set_tuning(vt.KERNEL_RENDER, **saved)


@pytest.mark.parametrize("tile", [vt.TILE_8X4, vt.TILE_4X8, vt.TILE_16X2, vt.TILE_32X1])
def test_batch_tile_shapes_agree(torch, tile):
    """Batch work units of every pixel-tile shape give the oracle's sample records (odd view
    sizes: partial tiles on both edges)."""
    scenes, views = workloads.multiview(n_scenes=2, n_views=4, sizes=(64, 48), min_px=37 * 23,
                                        max_px=141 * 77, seed=9)
    grids = [vt.Grid.from_u8(s["voxels"], s["palette"]) for s in scenes]
    saved = vt.get_tuning(vt.KERNEL_BATCH)
    try:
        vt.set_tuning(vt.KERNEL_BATCH, 32, 0, True, False, tile, 4)
        outs, specs = [], []
        for v in views:
            c = v["camera"]
            buf = torch.zeros(c.width * c.height * v["spp"] * 16, dtype=torch.uint8, device="cuda")
            outs.append(buf)
            specs.append(vt.make_view(grids[v["scene"]], c, buf, v["spp"], v["seed"],
                                      v["view_id"], v["light"]))
        b = vt.Batch(specs)
        b.run()
        torch.cuda.synchronize()
        ogrids = [po.Grid(s["voxels"], s["palette"]) for s in scenes]
        for v, o in zip(views, outs):
            L = v["light"]
            want = po.render_view(ogrids[v["scene"]], po.make_camera(v["camera"].as_dict()),
                                  po.make_light(list(L.dir), L.ambient, bool(L.shadows)),
                                  v["spp"], v["seed"], v["view_id"])
            assert_same(o.cpu().numpy().view(vt.HIT_DTYPE), want,
                        "batch tile %s view %d" % (vt.TILE_NAMES[tile], v["view_id"]))
        b.destroy()
    finally:
        vt.set_tuning(vt.KERNEL_BATCH, **saved)
        for g in grids:
            g.destroy()


def test_set_tuning_rejects_bad_shapes(torch):
    with pytest.raises(vt.VtError):
        vt.set_tuning(vt.KERNEL_RENDER, 16, 0, False, False, 4, 4)
    with pytest.raises(vt.VtError):
        vt.set_tuning(vt.KERNEL_RENDER, 16, 0, False, False, vt.TILE_8X4, 3)


def test_autotune_render_installs_an_exact_choice(torch, frame_case):
    w, light, g, want = frame_case
    cam = w["camera"]
    saved = vt.get_tuning(vt.KERNEL_RENDER)
    stream = torch.cuda.Stream()
    d = torch.empty(cam.width * cam.height * 16, dtype=torch.uint8, device="cuda")
    try:
        best, table = autotune.autotune(vt.KERNEL_RENDER, lambda: vt.render(g, cam, light, d, stream),
                                        stream, repeats=2)
        assert len(table) == len(autotune.render_candidates())
        assert all(ms > 0 for ms in table.values())
        got = vt.get_tuning(vt.KERNEL_RENDER)
        assert autotune.key(vt.KERNEL_RENDER, got) == autotune.key(vt.KERNEL_RENDER, best)
        assert table[autotune.key(vt.KERNEL_RENDER, best)] == min(table.values())
        d.fill_(0)
        vt.render(g, cam, light, d, stream)
        torch.cuda.synchronize()
        assert_same(d.cpu().numpy().view(vt.HIT_DTYPE), want, "tuned render")
    finally:
        vt.set_tuning(vt.KERNEL_RENDER, **saved)


def test_autotune_trace_rays_installs_an_exact_choice(torch):
    w = workloads.cave512(n=64, rays=1 << 16)
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    saved = vt.get_tuning(vt.KERNEL_TRACE_RAYS)
    stream = torch.cuda.Stream()
    n = w["rays"].shape[0]
    d_rays = torch.from_numpy(w["rays"].view(np.uint8).reshape(-1)).cuda()
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    try:
        best, table = autotune.autotune(vt.KERNEL_TRACE_RAYS,
                                        lambda: vt.trace_rays(g, d_rays, n, d_hits, stream),
                                        stream, repeats=2)
        assert len(table) == len(autotune.rays_candidates())
        d_hits.fill_(0)
        vt.trace_rays(g, d_rays, n, d_hits, stream)
        torch.cuda.synchronize()
        want = po.trace_rays(po.Grid(w["voxels"], w["palette"]), w["rays"])
        assert_same(d_hits.cpu().numpy().view(vt.HIT_DTYPE), want, "tuned trace_rays")
    finally:
        vt.set_tuning(vt.KERNEL_TRACE_RAYS, **saved)
        g.destroy()


def test_autotune_batch_installs_an_exact_choice(torch):
    scenes, views = workloads.multiview(n_scenes=2, n_views=5, sizes=(64, 48),
                                        min_px=40 * 30, max_px=160 * 120)
    grids = [vt.Grid.from_u8(s["voxels"], s["palette"]) for s in scenes]
    saved = vt.get_tuning(vt.KERNEL_BATCH)
    stream = torch.cuda.Stream()
    outs, specs = [], []
    for v in views:
        c = v["camera"]
        buf = torch.zeros(c.width * c.height * v["spp"] * 16, dtype=torch.uint8, device="cuda")
        outs.append(buf)
        specs.append(vt.make_view(grids[v["scene"]], c, buf, v["spp"], v["seed"], v["view_id"],
                                  v["light"]))
    holder = {"b": vt.Batch(specs)}

    def prepare():  # a batch's launch shape is fixed when it is created
        holder["b"].destroy()
        holder["b"] = vt.Batch(specs)

    try:
        best, table = autotune.autotune(vt.KERNEL_BATCH, lambda: holder["b"].run(stream), stream,
                                        repeats=2, prepare=prepare)
        assert len(table) == len(autotune.batch_candidates())
        for o in outs:
            o.zero_()
        holder["b"].run(stream)
        torch.cuda.synchronize()
        ogrids = [po.Grid(s["voxels"], s["palette"]) for s in scenes]
        for v, o in zip(views, outs):
            L = v["light"]
            want = po.render_view(ogrids[v["scene"]], po.make_camera(v["camera"].as_dict()),
                                  po.make_light(list(L.dir), L.ambient, bool(L.shadows)),
                                  v["spp"], v["seed"], v["view_id"])
            assert_same(o.cpu().numpy().view(vt.HIT_DTYPE), want, "tuned batch view %d" % v["view_id"])
        # the counting run of the same batch gives the same records and counts its rays
        st = holder["b"].stats()
        assert st["rays"] >= holder["b"].primary_rays
    finally:
        holder["b"].destroy()
        vt.set_tuning(vt.KERNEL_BATCH, **saved)
        for g in grids:
            g.destroy()
