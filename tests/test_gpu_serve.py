"""The continuous-batching service: every request's image is the same whether it ran alone or
packed with others into shared launches, and equals the oracle's averaged jittered samples; the
grid cache respects its HBM budget; failures are reported per request."""
import ctypes
import numpy as np
import pytest

import vtrace_gb300 as vt
from vtrace_gb300 import workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def oracle_image(scene, v):
    og = po.Grid(scene["voxels"], scene["palette"])
    cam = po.make_camera(v["camera"].as_dict())
    L = v["light"]
    light = po.make_light(list(L.dir), L.ambient, bool(L.shadows))
    hits = po.render_view(og, cam, light, v["spp"], v["seed"], v["view_id"])
    c = hits["rgba"].reshape(-1, v["spp"]).astype(np.uint64)
    out = np.zeros((c.shape[0], 4), np.uint8)
    for k in range(4):
        ch = (c >> np.uint64(8 * k)) & np.uint64(255)
        out[:, k] = ((ch.sum(1) + v["spp"] // 2) // v["spp"]).astype(np.uint8)
    return out.reshape(v["camera"].height, v["camera"].width, 4)


def grid_bound(n):
    """The service's bound of an n^3 u8 scene's device bytes: a grid allocation with every brick
    occupied (directory, octant and long-box words, palette, masks, payloads), each part rounded
    up to 256 bytes."""
    b = ((n + 7) // 8) ** 3
    al = lambda v: (v + 255) // 256 * 256
    return al(4 * b) + al(4 * b) + al(12 * b) + 1024 + al(64 * b) + al(512 * b)


def small_world(n_views=12):
    return workloads.multiview(n_scenes=3, n_views=n_views, sizes=(64, 96, 48), min_px=40 * 30,
                               max_px=160 * 120)


def pinned(torch, cam):
    return torch.zeros(cam.height * cam.width * 4, dtype=torch.uint8, pin_memory=True)


def test_results_same_alone_and_in_the_mix(torch):
    scenes, views = small_world()
    svc = vt.Service(max_inflight=1)
    try:
        sids = [svc.add_scene(s["voxels"], s["palette"]) for s in scenes]
        alone = []
        for v in views:  # one at a time: every launch carries a single request
            buf = pinned(torch, v["camera"])
            svc.wait(svc.submit(sids[v["scene"]], v["camera"], buf, v["spp"], v["seed"],
                                v["view_id"], v["light"]))
            alone.append(buf.numpy().copy())
        # a large request occupies the only slot while the others queue up behind it, so they
        # are packed into shared launches whatever the timing
        big = vt.camera_look_at((-40.0, 80.0, -40.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0, 1920, 1080)
        blocker = svc.submit(sids[0], big, pinned(torch, big), 8)
        bufs = [pinned(torch, v["camera"]) for v in views]
        rids = [svc.submit(sids[v["scene"]], v["camera"], b, v["spp"], v["seed"], v["view_id"],
                           v["light"]) for v, b in zip(views, bufs)]
        svc.wait(blocker)
        launches_blocked = svc.stats()["launches"]
        timings = [svc.wait(r) for r in rids]
        st = svc.stats()
        assert st["launches"] - launches_blocked < len(views)  # requests shared launches
        for a, b, v in zip(alone, bufs, views):
            np.testing.assert_array_equal(a, b.numpy(), err_msg="view %d" % v["view_id"])
        for i in (0, 4, 7, 11):
            img = bufs[i].numpy().reshape(views[i]["camera"].height, views[i]["camera"].width, 4)
            np.testing.assert_array_equal(img, oracle_image(scenes[views[i]["scene"]], views[i]))
        assert all(t["submit_ns"] <= t["launch_ns"] <= t["done_ns"] for t in timings)
    finally:
        svc.stop()


def test_plain_mode_gives_the_same_images(torch):
    scenes, views = small_world(6)
    svc = vt.Service(plain=True)
    try:
        sids = [svc.add_scene(s["voxels"], s["palette"]) for s in scenes]
        bufs = [pinned(torch, v["camera"]) for v in views]
        rids = [svc.submit(sids[v["scene"]], v["camera"], b, v["spp"], v["seed"], v["view_id"],
                           v["light"]) for v, b in zip(views, bufs)]
        for r in rids:
            svc.wait(r)
        assert svc.stats()["launches"] == len(views)
        for b, v in zip(bufs, views):
            img = b.numpy().reshape(v["camera"].height, v["camera"].width, 4)
            np.testing.assert_array_equal(img, oracle_image(scenes[v["scene"]], v))
    finally:
        svc.stop()


def test_split_requests_match_unsplit_ones(torch):
    """A request cut into many 4-row pieces, packed into shared launches with other requests'
    pieces, gives the same image as the same request run whole, and the oracle's."""
    scenes, views = small_world(6)
    v = dict(views[1], spp=3)
    v["camera"] = vt.camera_look_at((-30.0, 70.0, -30.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0,
                                    203, 131)  # 131 rows: the last piece is a partial tile row
    whole = vt.Service(max_inflight=1, max_samples_per_piece=0)
    split = vt.Service(max_inflight=2, max_samples_per_piece=203 * 3 * 8,
                       max_samples_per_launch=203 * 3 * 20)
    try:
        out = []
        for svc in (whole, split):
            sids = [svc.add_scene(s["voxels"], s["palette"]) for s in scenes]
            buf = pinned(torch, v["camera"])
            others = [pinned(torch, w["camera"]) for w in views]
            rids = [svc.submit(sids[w["scene"]], w["camera"], b, w["spp"], w["seed"], w["view_id"],
                               w["light"]) for w, b in zip(views[:3], others)]
            rid = svc.submit(sids[v["scene"]], v["camera"], buf, v["spp"], v["seed"], v["view_id"],
                             v["light"])
            rids += [svc.submit(sids[w["scene"]], w["camera"], b, w["spp"], w["seed"],
                                w["view_id"], w["light"]) for w, b in zip(views[3:], others[3:])]
            t = svc.wait(rid)
            assert t["samples"] == 203 * 131 * 3
            for r in rids:
                svc.wait(r)
            out.append((buf.numpy().copy(), [o.numpy().copy() for o in others]))
        assert split.stats()["views_launched"] >= 131 // 8  # the big request ran as pieces
        np.testing.assert_array_equal(out[0][0], out[1][0])
        for a, b in zip(out[0][1], out[1][1]):
            np.testing.assert_array_equal(a, b)
        img = out[1][0].reshape(131, 203, 4)
        np.testing.assert_array_equal(img, oracle_image(scenes[v["scene"]], v))
    finally:
        whole.stop()
        split.stop()


def test_pageable_outputs_through_the_staging_area(torch):
    """Outputs in ordinary (pageable) host memory: the resolve writes each piece's rows into the
    slot's device staging area and they are copied out; same images as the oracle's, whether
    the request is split into pieces or not."""
    scenes, views = small_world(5)
    svc = vt.Service(max_inflight=2, max_samples_per_piece=1500, max_samples_per_launch=6000)
    try:
        sids = [svc.add_scene(s["voxels"], s["palette"]) for s in scenes]
        outs = [np.zeros(v["camera"].width * v["camera"].height * 4, np.uint8) for v in views]
        rids = [svc.submit(sids[v["scene"]], v["camera"], o, v["spp"], v["seed"], v["view_id"],
                           v["light"]) for v, o in zip(views, outs)]
        for r in rids:
            svc.wait(r)
        for o, v in zip(outs, views):
            img = o.reshape(v["camera"].height, v["camera"].width, 4)
            np.testing.assert_array_equal(img, oracle_image(scenes[v["scene"]], v))
        assert svc.stats()["views_launched"] > len(views)  # some requests ran as pieces
    finally:
        svc.stop()


def test_stop_while_other_threads_submit_and_poll(torch):
    """vt_serve_stop while other threads are inside submit and poll calls on the same service:
    every call returns (a request id, VT_ECANCELED or VT_ENOTFOUND), nothing is left waiting."""
    import threading
    scenes, views = small_world(4)
    for round_ in range(3):
        svc = vt.Service(max_inflight=2)
        sid = svc.add_scene(scenes[0]["voxels"], scenes[0]["palette"])
        v = views[0]
        stop_flag = threading.Event()
        codes = []
        bufs = [pinned(torch, v["camera"]) for _ in range(8)]
        service = svc.id  # the raw id: the workers keep calling after stop() has released it

        def worker(k):
            n = 0
            while not stop_flag.is_set() or n < 4:
                r = vt.ServeRequest()
                r.scene, r.spp, r.seed, r.camera = sid, 1, n, v["camera"]
                r.host_rgba = bufs[(k + n) % len(bufs)].data_ptr()
                rid = ctypes.c_uint64(0)
                rc = vt.lib().vt_serve_submit(service, ctypes.byref(r), ctypes.byref(rid))
                if rc == 0:
                    rc = vt.lib().vt_serve_poll(service, rid.value, 2000, None)
                if rc not in (0, -8):  # VT_ENOTREADY: still running
                    codes.append(rc)
                    if rc in (-4, -7):
                        return
                n += 1

        threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for t in threads:
            t.start()
        import time
        time.sleep(0.05 * (round_ + 1))
        stop_flag.set()
        svc.stop()
        for t in threads:
            t.join(timeout=60)
        assert not any(t.is_alive() for t in threads)
        assert set(codes) <= {-4, -7}, codes  # VT_ENOTFOUND, VT_ECANCELED only


def test_start_refuses_slots_beyond_the_budget(torch):
    with pytest.raises(vt.VtError) as e:
        vt.Service(hbm_budget_bytes=1 << 20, max_samples_per_launch=1 << 20)
    assert e.value.code == -2


def test_cache_evicts_least_recently_used_under_its_budget(torch):
    scenes, views = small_world(8)
    # room for the largest scene's bound only (beside the one slot's sample buffer): alternating
    # scenes force evictions
    bound = max(grid_bound(s["n"]) for s in scenes)
    cap = 160 * 120 * 4
    svc = vt.Service(hbm_budget_bytes=bound + 1024 + cap * 20, max_inflight=1,
                     max_samples_per_launch=cap)
    try:
        sids = [svc.add_scene(s["voxels"], s["palette"]) for s in scenes]
        for v in views:
            buf = pinned(torch, v["camera"])
            svc.wait(svc.submit(sids[v["scene"]], v["camera"], buf, v["spp"], v["seed"],
                                v["view_id"], v["light"]))
            img = buf.numpy().reshape(v["camera"].height, v["camera"].width, 4)
            np.testing.assert_array_equal(img, oracle_image(scenes[v["scene"]], v))
        st = svc.stats()
        assert st["evictions"] > 0 and st["resident_bytes"] <= bound + 1024
    finally:
        svc.stop()


def test_failures_are_reported_per_request(torch):
    scenes, views = small_world(4)
    # 64 KB beside the slot's buffer: smaller than any scene's bound
    svc = vt.Service(hbm_budget_bytes=(64 << 10) + 4096 * 20, max_inflight=1,
                     max_samples_per_launch=4096)
    try:
        sid = svc.add_scene(scenes[1]["voxels"], scenes[1]["palette"])
        v = views[0]
        with pytest.raises(vt.VtError):
            svc.submit(sid + 5, v["camera"], pinned(torch, v["camera"]))
        rid = svc.submit(sid, v["camera"], pinned(torch, v["camera"]), v["spp"])
        with pytest.raises(vt.VtError) as e:
            svc.wait(rid)
        assert e.value.code == -2  # VT_ENOMEM: the scene cannot fit the budget
    finally:
        svc.stop()
    # stopping with requests still queued cancels them; a poller blocked on one returns
    import threading
    svc = vt.Service(max_inflight=1, max_views_per_launch=1)
    sid = svc.add_scene(scenes[0]["voxels"], scenes[0]["palette"])
    big = vt.camera_look_at((-40.0, 80.0, -40.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0, 1280, 720)
    bufs = [pinned(torch, big) for _ in range(40)]
    rids = [svc.submit(sid, big, b, 8, seed=k) for k, b in enumerate(bufs)]
    got = {}

    def waiter():
        try:
            got["timing"] = svc.poll(rids[-1], 30_000_000)
        except vt.VtError as err:
            got["code"] = err.code

    th = threading.Thread(target=waiter)
    th.start()
    svc.stop()
    th.join(timeout=60)
    assert not th.is_alive()
    assert got.get("code") == -7  # VT_ECANCELED


def test_oversized_piece_and_its_scene_must_fit_together(torch):
    """A piece larger than a slot's buffer takes a temporary counted against the budget.  When
    the scene fits alone and the temporary fits alone but not both, the request fails with
    VT_ENOMEM (its scene is never evicted from under it); with room for both it renders."""
    scenes, _ = small_world(2)
    sc = scenes[0]
    n = sc["n"]
    bound = grid_bound(n)
    g = vt.Grid.from_u8(sc["voxels"], sc["palette"])
    actual = g.info()["device_bytes"]
    g.destroy()
    assert actual <= bound  # equal for grids small enough to get a slot for every brick
    cap = 1024  # samples per slot: 20 KiB of slot buffers
    # a request whose temporary (20 B per sample) lies between bound - actual and bound
    width = 64
    height = max(4, int((bound - (bound - actual) // 2) // 20 // width))
    extra = width * height * 20
    assert bound - actual < extra < bound
    cam = vt.camera_look_at((-1.5 * n, 2.0 * n, -1.5 * n), (n / 2, n / 4, n / 2), (0, 1, 0), 60.0,
                            width, height)
    for budget, ok in ((cap * 20 + bound, False), (cap * 20 + actual + extra + 4096, True)):
        svc = vt.Service(hbm_budget_bytes=budget, max_inflight=1, max_samples_per_launch=cap,
                         max_samples_per_piece=0)
        try:
            sid = svc.add_scene(sc["voxels"], sc["palette"])
            buf = pinned(torch, cam)
            rid = svc.submit(sid, cam, buf, 1, 3, 9)
            if ok:
                svc.wait(rid)
                img = buf.numpy().reshape(height, width, 4)
                og = po.Grid(sc["voxels"], sc["palette"])
                hits = po.render_view(og, po.make_camera(cam.as_dict()), None, 1, 3, 9)
                want = np.ascontiguousarray(hits["rgba"]).view(np.uint8).reshape(height, width, 4)
                np.testing.assert_array_equal(img, want)
            else:
                with pytest.raises(vt.VtError) as e:
                    svc.wait(rid)
                assert e.value.code == -2  # VT_ENOMEM
        finally:
            svc.stop()


def test_protocol_errors(torch):
    """Requests are consumed by the poll that reports them; a poll with no wait on a running
    request says "not ready"; bad arguments and unknown ids fail without disturbing the service."""
    scenes, views = small_world(2)
    svc = vt.Service(max_inflight=1)
    service_id = svc.id
    try:
        sid = svc.add_scene(scenes[0]["voxels"], scenes[0]["palette"])
        v = views[0]
        with pytest.raises(vt.VtError) as e:
            svc.submit(sid, v["camera"], None)  # no output buffer
        assert e.value.code == -1
        with pytest.raises(vt.VtError) as e:
            svc.submit(sid, v["camera"], pinned(torch, v["camera"]), spp=0)
        assert e.value.code == -1
        with pytest.raises(ValueError):
            svc.submit(sid, v["camera"], torch.zeros(16, dtype=torch.uint8, pin_memory=True))
        # 2^32 samples: refused before the (here far too small) output is touched
        r = vt.ServeRequest()
        r.scene, r.spp = sid, 1
        r.camera = vt.camera_look_at((-40.0, 80.0, -40.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0,
                                     65536, 65536)
        tiny = torch.zeros(16, dtype=torch.uint8, pin_memory=True)
        r.host_rgba = tiny.data_ptr()
        rid0 = ctypes.c_uint64(0)
        assert vt.lib().vt_serve_submit(svc.id, ctypes.byref(r), ctypes.byref(rid0)) == -9  # VT_ELIMIT
        with pytest.raises(vt.VtError) as e:
            svc.poll(123456789)
        assert e.value.code == -4  # VT_ENOTFOUND
        big = vt.camera_look_at((-40.0, 80.0, -40.0), (32.0, 16.0, 32.0), (0, 1, 0), 60.0, 1920, 1080)
        rid = svc.submit(sid, big, pinned(torch, big), 8)
        quick = svc.submit(sid, v["camera"], pinned(torch, v["camera"]), 1)
        assert svc.poll(quick, 0) is None  # queued behind the large request
        assert svc.wait(rid)["samples"] == 1920 * 1080 * 8
        assert svc.wait(quick)["samples"] == v["camera"].width * v["camera"].height
        with pytest.raises(vt.VtError) as e:
            svc.poll(rid)  # already reported
        assert e.value.code == -4
        assert svc.stats()["completed"] >= 2
    finally:
        svc.stop()
    assert vt.lib().vt_serve_poll(service_id, 1, 0, None) == -4  # the stopped service is gone


def test_scene_updates_page_chunks_into_the_cache(torch):
    """vt_serve_update_scene (the pager's chunk uploads, src/gen/pager.rs:52-78, into the scene
    cache): boxes written into a resident scene, the first a solid block at its centre and the
    rest from another thread while requests of the scene are in flight, and into a scene never
    built (twice over one box); afterwards every request's image equals the oracle's of the
    updated array, and the centre block changed the oracle's image of the first view."""
    import threading
    scenes, views = small_world(8)
    rng = np.random.default_rng(17)
    svc = vt.Service(max_inflight=2)
    try:
        sids = [svc.add_scene(s["voxels"].copy(), s["palette"]) for s in scenes]
        arrays = [svc._keep[sid][0] for sid in sids]
        v0 = next(v for v in views if v["scene"] == 0)
        buf = pinned(torch, v0["camera"])
        svc.wait(svc.submit(sids[0], v0["camera"], buf, v0["spp"], v0["seed"], v0["view_id"],
                            v0["light"]))
        original = dict(scenes[0], voxels=arrays[0].copy())
        svc.update_scene(sids[0], (16, 16, 16), np.full((32, 32, 32), 7, np.uint8))

        def chunk(arr):
            nz, ny, nx = arr.shape
            d, h, w = (int(rng.integers(4, 20)) for _ in range(3))
            org = (int(rng.integers(0, nx - w)), int(rng.integers(0, ny - h)), int(rng.integers(0, nz - d)))
            box = np.where(rng.random((d, h, w)) < 0.5, rng.integers(1, 256, (d, h, w)), 0)
            return org, box.astype(np.uint8)

        # resident scene 0, while its requests run on the dispatcher
        bufs = [pinned(torch, v0["camera"]) for _ in range(6)]
        rids = [svc.submit(sids[0], v0["camera"], b, v0["spp"], v0["seed"], v0["view_id"],
                           v0["light"]) for b in bufs]
        errors = []

        def pager():
            try:
                for _ in range(5):
                    org, box = chunk(arrays[0])
                    svc.update_scene(sids[0], org, box)
            except Exception as e:  # reported below
                errors.append(e)

        th = threading.Thread(target=pager)
        th.start()
        th.join()
        for r in rids:
            svc.wait(r)
        assert not errors, errors
        # a scene never built yet, and one updated twice over the same box
        org, box = chunk(arrays[1])
        svc.update_scene(sids[1], org, box)
        svc.update_scene(sids[1], org, box)
        for v in views:
            b = pinned(torch, v["camera"])
            svc.wait(svc.submit(sids[v["scene"]], v["camera"], b, v["spp"], v["seed"],
                                v["view_id"], v["light"]))
            img = b.numpy().reshape(v["camera"].height, v["camera"].width, 4)
            updated = dict(scenes[v["scene"]], voxels=arrays[v["scene"]])
            np.testing.assert_array_equal(img, oracle_image(updated, v),
                                          err_msg="view %d" % v["view_id"])
            if v is v0:
                assert not np.array_equal(img, oracle_image(original, v)), "update not visible"
        with pytest.raises(vt.VtError):
            vt.check(vt.lib().vt_serve_update_scene(svc.id, sids[0], 0, 0, 0, 0, 4, 4))
        with pytest.raises(vt.VtError):
            vt.check(vt.lib().vt_serve_update_scene(svc.id, sids[0], 60, 0, 0, 8, 4, 4))
        with pytest.raises(vt.VtError):
            vt.check(vt.lib().vt_serve_update_scene(svc.id, 99, 0, 0, 0, 1, 1, 1))
    finally:
        svc.stop()


def test_scene_updates_while_the_cache_evicts(torch):
    """Room for one scene at a time: requests alternating between two scenes evict each in turn
    while another thread pages boxes into the first; no update lands in a grid being evicted or
    rebuilt, and the final images equal the oracle's of the updated arrays."""
    import threading
    scenes, views = small_world(8)
    scenes, views = scenes[:2], [v for v in views if v["scene"] < 2]
    bound = max(grid_bound(s["n"]) for s in scenes)
    cap = 160 * 120 * 4
    svc = vt.Service(hbm_budget_bytes=bound + 1024 + cap * 20, max_inflight=1,
                     max_samples_per_launch=cap)
    rng = np.random.default_rng(5)
    try:
        sids = [svc.add_scene(s["voxels"].copy(), s["palette"]) for s in scenes]
        arrays = [svc._keep[sid][0] for sid in sids]
        errors, done = [], threading.Event()

        def pager():
            try:
                n = arrays[0].shape[0]
                while not done.is_set():
                    org = tuple(int(x) for x in rng.integers(0, n - 8, 3))
                    box = np.where(rng.random((8, 8, 8)) < 0.5, rng.integers(1, 256, (8, 8, 8)), 0)
                    svc.update_scene(sids[0], org, box.astype(np.uint8))
            except Exception as e:
                errors.append(e)

        th = threading.Thread(target=pager)
        th.start()
        try:
            for _ in range(3):
                for v in views:
                    svc.wait(svc.submit(sids[v["scene"]], v["camera"], pinned(torch, v["camera"]),
                                        v["spp"], v["seed"], v["view_id"], v["light"]))
        finally:
            done.set()
            th.join()
        assert not errors, errors
        assert svc.stats()["evictions"] > 0
        for v in views:
            b = pinned(torch, v["camera"])
            svc.wait(svc.submit(sids[v["scene"]], v["camera"], b, v["spp"], v["seed"],
                                v["view_id"], v["light"]))
            img = b.numpy().reshape(v["camera"].height, v["camera"].width, 4)
            updated = dict(scenes[v["scene"]], voxels=arrays[v["scene"]])
            np.testing.assert_array_equal(img, oracle_image(updated, v),
                                          err_msg="view %d" % v["view_id"])
    finally:
        svc.stop()
