"""The warp-time phase profile (vt_render_phases): the instrumented render build writes the same
records as vt_render (the oracle's), counts every warp of the launch, and charges cycles to the
traversal phases of camera rays and shadow rays; without a light no shadow ray runs, so the shadow
kind has only its tail (shading and the store)."""
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


@pytest.fixture(scope="module")
def frame(torch):
    # odd image size: partial warp tiles and blocks on both edges
    w = workloads.terrain256(n=96, width=333, height=203)
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    yield w, g
    g.destroy()


def records(torch, fn, cam):
    d = torch.full((cam.width * cam.height * 16,), 0xAB, dtype=torch.uint8, device="cuda")
    out = fn(d)
    torch.cuda.synchronize()
    return d.cpu().numpy().reshape(-1, 16), out


def test_phase_profile_records_and_phases(torch, frame):
    w, g = frame
    cam = w["camera"]
    light = workloads.seeded_light(1, shadows=True)
    plain, _ = records(torch, lambda d: vt.render(g, cam, light, d), cam)
    got, prof = records(torch, lambda d: vt.render_phases(g, cam, light, d), cam)
    assert int((got != plain).any(1).sum()) == 0
    og = po.Grid(w["voxels"], w["palette"])
    want = po.render(og, po.make_camera(cam.as_dict()),
                     po.make_light(list(light.dir), light.ambient, bool(light.shadows)))
    want = np.ascontiguousarray(want).view(np.uint8).reshape(-1, 16)
    assert int((got != want).any(1).sum()) == 0
    assert prof["warps"] == ((cam.width + 7) // 8) * ((cam.height + 3) // 4)
    for kind in ("camera", "shadow"):
        for ph in vt.PHASES:
            assert prof[kind][ph] > 0, (kind, ph, prof)
    assert all(v > 0 for v in prof["passes"].values()), prof["passes"]


def test_phase_profile_without_light_has_no_shadow_passes(torch, frame):
    w, g = frame
    cam = w["camera"]
    got, prof = records(torch, lambda d: vt.render_phases(g, cam, None, d), cam)
    plain, _ = records(torch, lambda d: vt.render(g, cam, None, d), cam)
    assert int((got != plain).any(1).sum()) == 0
    assert prof["passes"]["shadow_walk"] == 0 and prof["passes"]["shadow_cross"] == 0
    assert all(prof["shadow"][ph] == 0 for ph in vt.PHASES if ph != "tail"), prof["shadow"]
    assert prof["shadow"]["tail"] > 0 and prof["camera"]["walk"] > 0
