"""MagicaVoxel ingest (src/voxel/magica_voxel.rs:18-44): the library's .vox reader against the
Python restatement in oracle/vox.py, on files written here and, where present, vtrace's assets."""
import os

import numpy as np
import pytest

import vtrace_gb300 as vt
from oracle import build as obuild
from oracle import vox as ovox

REF = obuild.reference_root()


def random_model(rng, size, count, ymax=None, zmax=None):
    sx, sy, sz = size
    ymax = sy if ymax is None else ymax
    zmax = sz if zmax is None else zmax
    # distinct positions, so that the later-wins overwrite order does not matter
    cells = rng.choice(sx * ymax * zmax, size=count, replace=False)
    x, r = cells // (ymax * zmax), cells % (ymax * zmax)
    y, z = r // zmax, r % zmax
    c = rng.integers(0, 256, count)
    return (sx, sy, sz), np.stack([x, y, z, c], 1).astype(np.uint8)


def palette(rng):
    p = rng.integers(0, 2**32, 256, dtype=np.uint64).astype(np.uint32)
    return p | np.uint32(0xFF000000)


def test_cubic_model_matches_restatement():
    rng = np.random.default_rng(1)
    m = random_model(rng, (16, 16, 16), 900)
    buf = ovox.write([m], palette(rng))
    got = vt.vox_model_chunk(buf)
    np.testing.assert_array_equal(got, ovox.model_chunk(buf))
    assert got.shape == (16, 16, 16, 4)
    assert (got[..., 3] != 0).sum() == 900
    assert vt.vox_inspect(buf) == {"version": 150, "models": 1, "has_palette": True}


def test_several_models_and_skipped_chunks():
    rng = np.random.default_rng(2)
    ms = [random_model(rng, (8, 12, 8), 200, ymax=8, zmax=8),   # y and z within both bounds
          random_model(rng, (5, 20, 7), 150, ymax=7),            # y < size.z, z < size.z <= size.y
          random_model(rng, (33, 9, 9), 500)]
    extra = [(b"nTRN", b"\x01\x02\x03\x04", b""), (b"LAYR", b"abcd", b""),
             (b"nGRP", b"", ovox._chunk(b"NOTE", b"xyz"))]
    buf = ovox.write(ms, palette(rng), version=200, pack=True, extra=extra)
    info = vt.vox_inspect(buf)
    assert info["models"] == 3 and info["version"] == 200
    for k in range(3):
        np.testing.assert_array_equal(vt.vox_model_chunk(buf, k), ovox.model_chunk(buf, k))


def test_palette_index_rule():
    # colour index c uses RGBA entry c - 1; c = 0 (not written by MagicaVoxel) saturates to 0
    pal = np.arange(256, dtype=np.uint32) | np.uint32(0xFF000000)
    vox = np.array([[0, 0, 0, 1], [1, 0, 0, 255], [2, 0, 0, 0], [3, 0, 0, 128]], np.uint8)
    buf = ovox.write([((4, 1, 1), vox)], pal)
    got = vt.vox_model_chunk(buf).view(np.uint32)[:, 0, 0, 0]
    np.testing.assert_array_equal(got & 0xFF, [0, 254, 0, 127])


def test_malformed_files_are_rejected():
    rng = np.random.default_rng(3)
    good = ovox.write([random_model(rng, (4, 4, 4), 10)], palette(rng))
    bad = {
        "magic": b"VOXX" + good[4:],
        "truncated": good[:-7],
        "no palette": ovox.write([random_model(rng, (4, 4, 4), 10)], None),
        # z = 5 maps to chunk y = size.y - 6 < 0 (vtrace's unwrap panics there)
        "outside": ovox.write([((4, 4, 8), np.array([[0, 0, 5, 1]], np.uint8))], palette(rng)),
    }
    for name, b in bad.items():
        with pytest.raises(vt.VtError) as e:
            vt.vox_model_chunk(b)
        assert e.value.code == -1, name
    with pytest.raises(vt.VtError) as e:
        vt.vox_model_chunk(good, 1)
    assert e.value.code == -4  # VT_ENOTFOUND


@pytest.mark.parametrize("name", ["AncientTemple", "Treasure"])
def test_vtrace_assets(name):
    if REF is None or not os.path.exists(os.path.join(REF, "assets", name + ".vox")):
        pytest.skip("vtrace's assets are not on this machine")
    path = os.path.join(REF, "assets", name + ".vox")
    buf = open(path, "rb").read()
    info = vt.vox_inspect(buf)
    assert info["models"] >= 1 and info["has_palette"]
    got = vt.vox_model_chunk(buf, 0)  # world.rs:65-70 uploads the first model
    np.testing.assert_array_equal(got, ovox.model_chunk(buf, 0))
    _, models, _ = ovox.parse(buf)
    assert (got[..., 3] != 0).sum() <= models[0][1].shape[0]
