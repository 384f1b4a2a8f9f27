"""The path-tracing estimator's CPU restatement: properties that pin it to the traversal it is
built on (an empty grid is the sky everywhere; with no bounces and no sun a pixel is the sky
weighted by its missing jittered samples, the same rays as the batched renderer's view 0)."""
import numpy as np

import vtrace_gb300 as vt
from oracle import pyoracle as po
from vtrace_gb300 import workloads

SKY = (0.6, 0.75, 1.0)


def test_empty_grid_is_sky():
    g = po.Grid(np.zeros((16, 24, 20), np.uint8), vt.gen_palette(1))
    cam = po.make_camera(vt.camera_look_at((-5, 30, -8), (10, 12, 8), (0, 1, 0), 60.0, 32, 24).as_dict())
    p = po.make_path_params(3, 4, 5, SKY, (0.0, 1.0, 0.0), (2.0, 2.0, 2.0))
    img, rays = po.path_trace(g, cam, p)
    np.testing.assert_array_equal(img[..., :3], np.broadcast_to(np.float32(SKY), img[..., :3].shape))
    assert rays == 32 * 24 * 3
    assert (img[..., 3] == 1).all()


def test_first_hits_are_the_jittered_view_rays():
    w = workloads.terrain256(n=48, width=40, height=30)
    g = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"].as_dict())
    spp, seed = 4, 17
    p = po.make_path_params(spp, 0, seed, SKY, (0.0, 1.0, 0.0), (0.0, 0.0, 0.0))
    img, rays = po.path_trace(g, cam, p)
    assert rays == 40 * 30 * spp
    hits = po.render_view(g, cam, None, spp, seed, 0).reshape(30, 40, spp)
    miss = (hits["face"] & po.FLAG_HIT) == 0
    want = np.zeros((30, 40, 3), np.float32)
    for s in range(spp):  # the sum in sample order, then one division
        want = (want + np.where(miss[..., s, None], np.float32(SKY), np.float32(0))).astype(np.float32)
    want = (want / np.float32(spp)).astype(np.float32)
    np.testing.assert_array_equal(img[..., :3], want)
    assert 0 < miss.mean() < 1


def test_rows_and_threads_do_not_change_the_image():
    w = workloads.terrain256(n=48, width=36, height=28)
    g = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"].as_dict())
    p = po.make_path_params(2, 3, 3, SKY, (0.36, 0.8, 0.48), (2.0, 1.9, 1.7))
    full, rays = po.path_trace(g, cam, p, threads=1)
    band, _ = po.path_trace(g, cam, p, threads=4, rows=(9, 20))
    np.testing.assert_array_equal(full[9:20], band)
    assert rays > 36 * 28 * 2 and full[..., :3].max() > 0
