"""Large-grid brick builds (more than 512 bricks, built by launches rather than the small-grid
graph; the words pass stages each occupied brick's voxels for the compaction, and the passes along
x read an occupancy bitmask): the directory with its distances, the masks, every payload byte and
the octant and long-box words equal brute-force restatements of the layout (lib/memory.c:353-366
gives the dense x-fastest input), for u8 grids with and without the "index != 0" occupancy
shortcut, RGBA8 texels, z-fastest chunks and device input, at sizes with partial bricks on every
axis and rows that are not 8-byte aligned."""
import numpy as np
import pytest

import vtrace_gb300 as vt
from test_gpu_parity import expected_bricks, expected_long, expected_octants

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    vt.init(0)
    return t


def padded_blocks(dense):
    """[bricks, 8, 8, 8, ...] blocks (z, y, x) of a [z, y, x, ...] array, zero past its edge."""
    nz, ny, nx = dense.shape[:3]
    bx, by, bz = (nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8
    pad = np.zeros((bz * 8, by * 8, bx * 8) + dense.shape[3:], dense.dtype)
    pad[:nz, :ny, :nx] = dense
    b = pad.reshape((bz, 8, by, 8, bx, 8) + dense.shape[3:])
    b = b.transpose((0, 2, 4, 1, 3, 5) + tuple(range(6, b.ndim)))
    return b.reshape((bz * by * bx, 8, 8, 8) + dense.shape[3:])


def check_layout(g, vox, pal, texels=None):
    d, m = g.bricks()
    wd, wm, occ = expected_bricks(vox, pal)
    np.testing.assert_array_equal(d, wd)
    np.testing.assert_array_equal(m, wm)
    info = g.info()
    assert info["voxels_occupied"] == occ and info["slots"] == len(wm) == info["bricks_nonempty"]
    full = (d >> 31) == 0
    blocks = padded_blocks(vox if texels is None else texels)
    want = np.zeros((len(wm),) + blocks.shape[1:], blocks.dtype)
    want[d[full]] = blocks[full]
    got = g.payload()
    if texels is not None:
        got = got.view(np.uint32)[..., 0]
    np.testing.assert_array_equal(got, want)
    # the empty-box words (octant and long boxes), against the brute-force restatements
    dims = vox.shape[::-1]
    oc = g.octants()
    np.testing.assert_array_equal(oc, expected_octants(d, dims))
    np.testing.assert_array_equal(g.long_boxes(), expected_long(d, oc, dims))


def random_vox(rng, dims, density):
    nx, ny, nz = dims
    v = rng.integers(1, 256, (nz, ny, nx))
    # clustered occupancy: most bricks empty, a few dense (the staged blocks vary)
    cell = rng.random(((nz + 15) // 16, (ny + 15) // 16, (nx + 15) // 16)) < density
    mask = np.kron(cell, np.ones((16, 16, 16), bool))[:nz, :ny, :nx] & (rng.random((nz, ny, nx)) < 0.5)
    return np.where(mask, v, 0).astype(np.uint8)


@pytest.mark.parametrize("dims,transparent", [
    ((203, 77, 91), False),   # rows not 8-byte aligned: the generic row path
    ((256, 61, 45), False),   # whole aligned rows except on the y and z edges
    ((96, 96, 100), True),    # an occupied-looking index with alpha 0: palette lookups
    ((64, 72, 80), False),
])
def test_u8_builds_match_the_layout(torch, dims, transparent):
    rng = np.random.default_rng(sum(dims))
    vox = random_vox(rng, dims, 0.3)
    pal = vt.gen_palette(3)
    if transparent:
        pal[5] &= 0x00FFFFFF
    g = vt.Grid.from_u8(vox, pal)
    try:
        assert g.info()["bricks_total"] > 512
        check_layout(g, vox, pal)
    finally:
        g.destroy()


def test_rgba8_z_fastest_and_device_builds_match_the_layout(torch):
    rng = np.random.default_rng(77)
    dims = (120, 88, 70)
    vox = random_vox(rng, dims, 0.35)
    pal = vt.gen_palette(9)
    pal[7] &= 0x00FFFFFF  # texels with alpha 0 inside occupied bricks stay in the payload
    texels = pal[vox]
    grids = [("rgba8", vt.Grid.from_rgba8(texels), texels),
             ("rgba8 z-fastest", vt.Grid.from_chunk(np.ascontiguousarray(texels.transpose(2, 1, 0))),
              texels),
             ("u8 z-fastest", vt.Grid.from_chunk(np.ascontiguousarray(vox.transpose(2, 1, 0)), pal),
              None)]
    d_vox = torch.from_numpy(vox.reshape(-1)).cuda()
    grids.append(("u8 device", vt.Grid.from_u8_device(d_vox, dims, pal), None))
    try:
        for what, g, tex in grids:
            try:
                check_layout(g, vox, pal, tex)
            except AssertionError as e:
                raise AssertionError("%s: %s" % (what, e))
        # the caller's device buffer is left as it was
        assert np.array_equal(d_vox.cpu().numpy(), vox.reshape(-1))
    finally:
        for _, g, _ in grids:
            g.destroy()


def test_payload_download_checks_its_capacity(torch):
    vox = random_vox(np.random.default_rng(5), (72, 72, 72), 0.5)
    g = vt.Grid.from_u8(vox, vt.gen_palette(1))
    try:
        slots = g.info()["slots"]
        assert slots > 0
        buf = np.zeros(slots * 512 - 1, np.uint8)
        with pytest.raises(vt.VtError):
            vt.check(vt.lib().vt_grid_download_payload(g.id, buf.ctypes.data, buf.nbytes))
    finally:
        g.destroy()
