"""CPU tests of the oracle: hand-derived known answers, the committed golden fixtures, an
independent pure-Python restatement, and (where the reference tree is present) the reference
fragment shader itself compiled as C++."""
import glob
import math
import os

import numpy as np
import pytest

from oracle import pyoracle as po

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
F = np.float32


def grid_with(shape, voxels, alpha=255):
    """Grid of `shape` (nx, ny, nz) with the given {(x, y, z): palette index} voxels."""
    nx, ny, nz = shape
    v = np.zeros((nz, ny, nx), np.uint8)
    for (x, y, z), idx in voxels.items():
        v[z, y, x] = idx
    pal = np.zeros(256, np.uint32)
    pal[1:] = (np.arange(1, 256, dtype=np.uint32) * 0x010203) & 0xFFFFFF
    pal[1:] |= np.uint32(alpha) << 24
    return po.Grid(v, pal)


def trace1(g, o, d):
    r = np.array([list(o) + list(d)], np.float32)
    return po.trace_rays(g, r, threads=1)[0]


def ties1(g, o, d):
    r = np.array([list(o) + list(d)], np.float32)
    return po.trace_rays(g, r, threads=1, stats=True)[1]["ties"]


# ------------------------------------------------------------------ known answers

def test_axis_ray_from_inside():
    g = grid_with((8, 8, 8), {(5, 3, 3): 9})
    h = trace1(g, (0.5, 3.5, 3.5), (1, 0, 0))
    assert (h["x"], h["y"], h["z"]) == (5, 3, 3)
    assert h["face"] & po.FLAG_HIT
    assert h["face"] & 7 == 2  # entered through the -X face
    assert h["t"] == F(4.5)
    assert h["palette_index"] == 9
    assert ties1(g, (0.5, 3.5, 3.5), (1, 0, 0)) == 0


def test_axis_ray_from_outside_enters_through_slab():
    g = grid_with((8, 8, 8), {(5, 3, 3): 9})
    h = trace1(g, (-2.0, 3.5, 3.5), (1, 0, 0))
    assert (h["x"], h["y"], h["z"], h["t"]) == (5, 3, 3, F(7.0))
    h = trace1(g, (12.0, 3.5, 3.5), (-1, 0, 0))
    assert (h["x"], h["face"] & 7, h["t"]) == (5, 1, F(6.0))  # +X face at x = 6


def test_hit_in_entry_voxel_uses_entry_face():
    g = grid_with((8, 8, 8), {(0, 2, 2): 4})
    h = trace1(g, (-3.0, 2.5, 2.5), (1, 0, 0))
    assert (h["x"], h["face"] & 7, h["t"]) == (0, 2, F(3.0))


def test_origin_inside_solid_voxel():
    g = grid_with((8, 8, 8), {(4, 4, 4): 4})
    h = trace1(g, (4.25, 4.5, 4.75), (0.3, -0.2, 0.9))
    assert (h["x"], h["y"], h["z"], h["face"] & 7, h["t"]) == (4, 4, 4, 0, F(0.0))


def test_diagonal_tie_steps_two_axes_and_flags_it():
    # From a voxel centre along (1,1,0): side_x == side_y each step, both axes advance at once
    g = grid_with((8, 8, 8), {(2, 2, 0): 3})
    d = np.array([1, 1, 0], np.float32) / np.sqrt(F(2))
    h = trace1(g, (0.5, 0.5, 0.5), d)
    assert (h["x"], h["y"], h["z"]) == (2, 2, 0)
    assert ties1(g, (0.5, 0.5, 0.5), d) == 1
    assert h["face"] & 7 == 2  # ties resolve to the x face first
    assert h["t"] == (F(2.0) - F(0.5)) / F(d[0])


def test_diagonal_tie_skips_edge_neighbours():
    # the voxels beside the diagonal are never visited on an exact tie
    g = grid_with((8, 8, 8), {(1, 0, 0): 3, (0, 1, 0): 3})
    d = np.array([1, 1, 0], np.float32) / np.sqrt(F(2))
    h = trace1(g, (0.5, 0.5, 0.5), d)
    assert not h["face"] & po.FLAG_HIT
    assert ties1(g, (0.5, 0.5, 0.5), d) == 1


def test_alpha_zero_is_empty():
    g = grid_with((8, 8, 8), {(5, 3, 3): 9}, alpha=0)
    h = trace1(g, (0.5, 3.5, 3.5), (1, 0, 0))
    assert not h["face"] & po.FLAG_HIT
    assert h["t"] == np.inf and h["x"] == 0xFFFF


def test_miss_pointing_away_and_parallel_outside():
    g = grid_with((8, 8, 8), {(5, 3, 3): 9})
    assert not trace1(g, (-1.0, 3.5, 3.5), (-1, 0, 0))["face"] & po.FLAG_HIT
    assert not trace1(g, (-1.0, 9.5, 3.5), (1, 0, 0))["face"] & po.FLAG_HIT


def test_origin_on_max_face_clamps_to_last_voxel():
    # trace.frag:68 clamps only the top: floor(min(pos, size - 1))
    g = grid_with((8, 8, 8), {(7, 3, 3): 2})
    h = trace1(g, (8.0, 3.5, 3.5), (-1, 0, 0))
    assert (h["x"], h["face"] & 7, h["t"]) == (7, 0, F(0.0))


def test_non_finite_ray_is_invalid_miss():
    g = grid_with((8, 8, 8), {(5, 3, 3): 9})
    for o, d in (((np.nan, 1, 1), (1, 0, 0)), ((1, 1, 1), (np.inf, 0, 0))):
        h = trace1(g, o, d)
        assert h["face"] & po.FLAG_INVALID and not h["face"] & po.FLAG_HIT


def test_degenerate_direction_runs_literal_loop():
    # d_y so small that len/d_y overflows and the start sits on the top face: side_y = 0*inf =
    # NaN, no mask bit is ever set, and the loop samples its start voxel until max_steps.
    g = grid_with((8, 8, 8), {(0, 7, 0): 5})
    h = trace1(g, (0.5, 8.0, 0.5), (1.0, 1e-39, 0.0))
    assert (h["x"], h["y"], h["z"], h["face"] & 7) == (0, 7, 0, 0)
    g2 = grid_with((8, 8, 8), {(3, 7, 0): 5})
    h2 = trace1(g2, (0.5, 8.0, 0.5), (1.0, 1e-39, 0.0))
    assert not h2["face"] & po.FLAG_HIT  # stuck in (0,7,0): never reaches x = 3


def test_zero_direction():
    g = grid_with((8, 8, 8), {(2, 2, 2): 5})
    assert trace1(g, (2.5, 2.5, 2.5), (0, 0, 0))["face"] & po.FLAG_HIT
    assert not trace1(g, (3.5, 2.5, 2.5), (0, 0, 0))["face"] & po.FLAG_HIT


def test_rgba_texel_grid():
    t = np.zeros((8, 8, 8), np.uint32)
    t[3, 3, 5] = 0x7F112233
    t[3, 3, 4] = 0x00FFFFFF  # alpha 0: empty
    g = po.Grid(texels=t)
    h = trace1(g, (0.5, 3.5, 3.5), (1, 0, 0))
    assert (h["x"], h["rgba"], h["palette_index"]) == (5, 0x7F112233, 0)


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kat:
        assert tuple(int(x) for x in po.philox(ctr, key)) == want


def test_shading_and_shadow_known_answer():
    # camera looking down -z at a floor voxel with a blocker between it and the light
    g = grid_with((8, 8, 8), {(4, 4, 0): 1, (4, 4, 3): 2})
    cam = po.make_camera({"origin": [4.5, 4.5, 6.5], "forward": [0, 0, -1], "right": [0.01, 0, 0],
                          "up": [0, 0.01, 0], "width": 1, "height": 1})
    lit = po.render(g, cam, po.make_light([0.0, 0.0, 1.0], 0.25, False), threads=1)[0, 0]
    # the camera sits inside the grid: the first voxel on the ray is (4,4,3) through +Z
    assert (lit["x"], lit["y"], lit["z"], lit["face"] & 7) == (4, 4, 3, 5)
    base = int(g.palette[2])
    for c in range(3):
        assert (int(lit["rgba"]) >> (8 * c)) & 255 == math.floor((base >> (8 * c) & 255) * 1.0 + 0.5)
    cam2 = po.make_camera({"origin": [4.5, 4.5, 2.5], "forward": [0, 0, -1], "right": [0.01, 0, 0],
                           "up": [0, 0.01, 0], "width": 1, "height": 1})
    sh = po.render(g, cam2, po.make_light([0.0, 0.0, 1.0], 0.25, True), threads=1)[0, 0]
    assert (sh["z"], sh["face"] & 7) == (0, 5)
    assert sh["face"] & po.FLAG_SHADOW_RAY and sh["face"] & po.FLAG_SHADOWED
    base = int(g.palette[1])
    for c in range(3):
        assert (int(sh["rgba"]) >> (8 * c)) & 255 == int(F((base >> (8 * c)) & 255) * F(0.25) + F(0.5))
    assert (int(sh["rgba"]) >> 24) == base >> 24


def test_render_miss_is_sky():
    g = grid_with((8, 8, 8), {})
    cam = po.make_camera({"origin": [4, 4, 20], "forward": [0, 0, -1], "right": [0.1, 0, 0],
                          "up": [0, 0.1, 0], "width": 4, "height": 3})
    img = po.render(g, cam, None, threads=1)
    assert (img["rgba"] == po.SKY_RGBA).all() and (img["t"] == np.inf).all()


# ------------------------------------------------------------------ golden fixtures

def load_golden(path):
    z = np.load(path)
    g = po.Grid(z["voxels"], z["palette"])
    cam = po.make_camera({"origin": z["cam_origin"], "forward": z["cam_forward"],
                          "right": z["cam_right"], "up": z["cam_up"],
                          "width": int(z["cam_size"][0]), "height": int(z["cam_size"][1])})
    L = z["light"]
    light = po.make_light(L[:3], float(L[3]), bool(L[4]))
    return z, g, cam, light


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_reproduces_golden(path):
    z, g, cam, light = load_golden(path)
    ora = po.trace_entry_points(g, z["entry_mp"], z["entry_s"])
    np.testing.assert_array_equal(ora, z["entry_expected"])
    hits = po.trace_rays(g, z["rays"], threads=2)
    np.testing.assert_array_equal(hits.view(np.uint8).reshape(-1, 16), z["ray_hits"])
    img = po.render(g, cam, light, threads=2)
    np.testing.assert_array_equal(img.view(np.uint8).reshape(-1, 16), z["render_hits"])


# ------------------------------------------------------------------ independent restatement

def py_trace(vox, pal, o, d):
    """trace.frag:68-87 once more, in pure Python over numpy float32 scalars."""
    nz, ny, nx = vox.shape
    size = [F(nx), F(ny), F(nz)]
    o = [F(x) for x in o]
    d = [F(x) for x in d]
    if not all(np.isfinite(o + d)):
        return None
    tn, tf, ax = F(-np.inf), F(np.inf), -1
    for a in range(3):
        if d[a] == 0:
            if o[a] < 0 or o[a] > size[a]:
                return None
            continue
        ta, tb = (F(0) - o[a]) / d[a], (size[a] - o[a]) / d[a]
        lo, hi = min(ta, tb), max(ta, tb)
        if lo > tn:
            tn, ax = lo, a
        tf = min(tf, hi)
    if tn > tf or tf < 0:
        return None
    if tn <= 0:
        pos = list(o)
    else:
        pos = [min(max(o[b] + tn * d[b], F(0)), size[b]) for b in range(3)]
        pos[ax] = F(0) if d[ax] > 0 else size[ax]
    ln = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
    v, st, dl, sd = [], [], [], []
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for a in range(3):
            m = size[a] - F(1) if size[a] - F(1) < pos[a] else pos[a]
            v.append(int(np.floor(m)))
            sg = F(1) if d[a] > 0 else (F(-1) if d[a] < 0 else F(0))
            st.append(int(sg))
            dl.append(abs(ln / d[a]))
            sd.append(((sg * (F(v[a]) - pos[a]) + sg * F(0.5)) + F(0.5)) * dl[a])
        steps, maxs = 0, nx + ny + nz
        while steps < maxs and all(0 <= v[a] < s for a, s in enumerate((nx, ny, nz))):
            if pal[vox[v[2], v[1], v[0]]] >> 24:
                return tuple(v), steps
            gm = lambda x, y: y if y < x else x  # noqa: E731
            m = [sd[0] <= gm(sd[1], sd[2]), sd[1] <= gm(sd[2], sd[0]), sd[2] <= gm(sd[0], sd[1])]
            for a in range(3):
                if m[a]:
                    sd[a] = sd[a] + dl[a]
                    v[a] += st[a]
            steps += 1
    return None


def test_oracle_matches_python_restatement():
    rng = np.random.default_rng(5)
    vox = np.where(rng.random((12, 10, 9)) < 0.04, rng.integers(1, 256, (12, 10, 9)), 0).astype(np.uint8)
    pal = np.zeros(256, np.uint32)
    pal[1:] = rng.integers(0, 1 << 24, 255, dtype=np.uint32) | (np.uint32(200) << 24)
    g = po.Grid(vox, pal)
    n = 1500
    o = (rng.random((n, 3)) * 16 - 3).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[:150, 0] = 0
    o[150:300] = np.floor(o[150:300]) + 0.5
    d[150:300] = rng.choice([-1.0, 1.0], (150, 3))
    hits = po.trace_rays(g, np.concatenate([o, d], 1), threads=1)
    for i in range(n):
        want = py_trace(vox, pal, o[i], d[i])
        h = hits[i]
        if want is None:
            assert not h["face"] & po.FLAG_HIT, i
        else:
            assert h["face"] & po.FLAG_HIT, i
            assert (h["x"], h["y"], h["z"]) == want[0], i


# ------------------------------------------------------------------ reference shader as C++

needs_ref = pytest.mark.skipif(not po.ref_available(), reason="reference source tree absent")


@needs_ref
@pytest.mark.parametrize("n,density", [(32, 0.05), (16, 0.3), (64, 0.01)])
def test_oracle_matches_reference_shader(n, density):
    rng = np.random.default_rng(n)
    vox = np.where(rng.random((n, n, n)) < density, rng.integers(1, 256, (n, n, n)), 0).astype(np.uint8)
    pal = np.zeros(256, np.uint32)
    pal[1:] = rng.integers(0, 1 << 24, 255, dtype=np.uint32) | (rng.integers(0, 256, 255, dtype=np.uint32) << 24)
    g = po.Grid(vox, pal)
    m = 60000
    mp = (rng.random((m, 3)) - 0.5).astype(np.float32)
    ax = rng.integers(0, 3, m // 2)
    mp[np.arange(m // 2), ax] = rng.choice([-0.5, 0.5], m // 2)
    s = rng.normal(size=(m, 3)).astype(np.float32)
    s[: m // 8, :2] = 0
    s[m // 8: m // 4, 2] = 0
    s[m // 4: m // 3] = rng.choice([-1.0, 1.0], (m // 3 - m // 4, 3))
    ref = po.ref_trace(g, mp, s, "select")
    ora = po.trace_entry_points(g, mp, s)
    np.testing.assert_array_equal(ref[:, 0], ora[:, 0])
    np.testing.assert_array_equal(ref[:, 4], ora[:, 4])
    hit = ref[:, 0] == 1
    np.testing.assert_array_equal(ref[hit, 1:4], ora[hit, 1:4])


@needs_ref
def test_literal_ieee_reading_only_differs_on_zero_components():
    """The literal IEEE product vec3(mask) * delta gives 0 * inf = NaN for axes with a zero
    direction component; everywhere else both readings of trace.frag agree."""
    rng = np.random.default_rng(9)
    n = 32
    vox = np.where(rng.random((n, n, n)) < 0.03, 1, 0).astype(np.uint8)
    pal = np.zeros(256, np.uint32)
    pal[1] = 0xFF00FF00
    g = po.Grid(vox, pal)
    m = 30000
    mp = (rng.random((m, 3)) - 0.5).astype(np.float32)
    s = rng.normal(size=(m, 3)).astype(np.float32)
    zero = rng.random((m, 3)) < 0.15
    s[zero] = 0
    s[(s == 0).all(1)] = 1
    a = po.ref_trace(g, mp, s, "select")
    b = po.ref_trace(g, mp, s, "ieee")
    differ = (a != b).any(1)
    assert differ.sum() > 0
    assert not (differ & ~(s == 0).any(1)).any()
