"""vt_grid_build_u8_noalloc: the brick build for callers that cannot allocate device memory while
they run (a chunk pager inside a frame loop, code recording into a captured stream).  Its output
must equal the allocating build's (vt_grid_create_u8 + vt_grid_download_bricks), call after call,
while the device's free memory stays where it was.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import vtrace_gb300 as vt

pytestmark = pytest.mark.gpu


def expected_payload(vox, directory):
    nz, ny, nx = vox.shape
    bx, by, bz = (nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8
    pad = np.zeros((bz * 8, by * 8, bx * 8), np.uint8)
    pad[:nz, :ny, :nx] = vox
    b = pad.reshape(bz, 8, by, 8, bx, 8).transpose(0, 2, 4, 1, 3, 5).reshape(-1, 512)
    occupied = (directory >> 31) == 0
    out = np.zeros((int(occupied.sum()), 512), np.uint8)
    out[directory[occupied]] = b[occupied]
    return out


def test_noalloc_build_matches_allocating_build():
    import torch
    assert torch.cuda.is_available()
    L = vt.lib()
    vt.init(0)
    cases = [vt.gen_terrain(128, 21), vt.gen_shapes((100, 72, 56), 4, count=30, rmin=2, rmax=12)]
    pal = vt.gen_palette(8)
    pal[9] &= 0x00FFFFFF  # an index present in the grids but not occupied
    d_pal = torch.from_numpy(pal.view(np.uint8)).cuda()
    # device buffers sized for the larger case, shared by both calls (the caller owns them)
    max_bricks = max(((v.shape[2] + 7) // 8) * ((v.shape[1] + 7) // 8) * ((v.shape[0] + 7) // 8)
                     for v in cases)
    d_dir = torch.empty(max_bricks * 4, dtype=torch.uint8, device="cuda")
    d_masks = torch.empty(max_bricks * 64, dtype=torch.uint8, device="cuda")
    d_payload = torch.empty(max_bricks * 512, dtype=torch.uint8, device="cuda")
    d_counts = torch.zeros(16, dtype=torch.uint8, device="cuda")
    inputs = [torch.from_numpy(np.ascontiguousarray(v).reshape(-1)).cuda() for v in cases]
    # warm-up: the first call on a device loads the library's module (its static scratch array
    # included) and looks up the array's address; measure free memory after that
    nz, ny, nx = cases[1].shape
    assert L.vt_grid_build_u8_noalloc(inputs[1].data_ptr(), d_pal.data_ptr(), nx, ny, nz,
                                      d_dir.data_ptr(), d_masks.data_ptr(), d_payload.data_ptr(),
                                      d_counts.data_ptr(), None) == 0
    vt.Grid.from_u8(cases[1], pal).destroy()
    torch.cuda.synchronize()
    # the window holds the no-allocation calls and the copies of their outputs to host memory
    # only; the allocating builds they are compared with run after it
    free_before = vt.device_info()["free_bytes"]
    results = []
    for vox, d_vox in zip(cases, inputs):
        nz, ny, nx = vox.shape
        rc = L.vt_grid_build_u8_noalloc(d_vox.data_ptr(), d_pal.data_ptr(), nx, ny, nz,
                                        d_dir.data_ptr(), d_masks.data_ptr(),
                                        d_payload.data_ptr(), d_counts.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        results.append((d_counts.cpu().numpy().view(np.uint64).copy(),
                        d_dir.cpu().numpy().view(np.uint32).copy(),
                        d_masks.cpu().numpy().view(np.uint64).copy(),
                        d_payload.cpu().numpy().copy()))
    torch.cuda.synchronize()
    free_after = vt.device_info()["free_bytes"]
    assert free_after == free_before
    for vox, (counts, dirs, masks, payload) in zip(cases, results):
        nz, ny, nx = vox.shape
        bricks = ((nx + 7) // 8) * ((ny + 7) // 8) * ((nz + 7) // 8)
        got_dir = dirs[:bricks]
        g = vt.Grid.from_u8(vox, pal)  # the allocating path (test side only)
        try:
            want_dir, want_masks = g.bricks()
            info = g.info()
        finally:
            g.destroy()
        np.testing.assert_array_equal(got_dir, want_dir)
        n = info["bricks_nonempty"]
        assert int(counts[0]) == n and int(counts[1]) == info["voxels_occupied"]
        np.testing.assert_array_equal(masks[: n * 8].reshape(-1, 8), want_masks)
        np.testing.assert_array_equal(payload[: n * 512].reshape(-1, 512),
                                      expected_payload(vox, got_dir))


def test_noalloc_build_rejects_grids_beyond_its_scratch():
    import torch
    L = vt.lib()
    buf = torch.empty(64, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    assert L.vt_grid_build_u8_noalloc(p, p, 512, 512, 512, p, p, p, p, None) == -9  # VT_ELIMIT
    assert L.vt_grid_build_u8_noalloc(p, p, 0, 8, 8, p, p, p, p, None) == -1       # VT_EINVAL
    assert L.vt_grid_build_u8_noalloc(None, p, 8, 8, 8, p, p, p, p, None) == -1
