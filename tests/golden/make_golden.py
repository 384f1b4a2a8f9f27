"""Generates the golden traversal fixtures in tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

The reference has no golden vectors for its traversal, and its shader needs a graphics API.  This
script therefore pins every fixture in two independent ways before writing it:

1. the reference's own fragment shader (shaders/trace.frag), compiled as C++ through
   oracle/glsl_compat.hpp, traces the entry-point form of each case, and the CPU oracle must
   reproduce its hit flag, hit voxel and texel-fetch count exactly;
2. the oracle then produces the full hit records (ray-buffer and render forms), which are
   stored as the expected outputs.

The reference source tree must be present (it is only needed to regenerate the fixtures; the
tests read the committed .npz files).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def palette(rng):
    pal = np.zeros(256, np.uint32)
    rgb = rng.integers(0, 1 << 24, 255, dtype=np.uint32)
    alpha = rng.integers(1, 256, 255, dtype=np.uint32)
    pal[1:] = rgb | (alpha << 24)
    # a few indices with alpha 0: present in the grid but not occupied (trace.frag:78)
    pal[[7, 77, 177]] &= 0x00FFFFFF
    return pal


def sparse_grid(rng, shape, density):
    nz, ny, nx = shape
    v = np.where(rng.random(shape) < density, rng.integers(1, 256, shape), 0).astype(np.uint8)
    return v


def ray_cases(rng, n, dims):
    nx, ny, nz = dims
    size = np.array([nx, ny, nz], np.float32)
    o = (rng.random((n, 3)) * 1.6 - 0.3).astype(np.float32) * size  # inside and around
    d = rng.normal(size=(n, 3)).astype(np.float32)
    k = n // 8
    # axis-parallel and planar directions (sign() = 0, delta = inf)
    d[:k, 1:] = 0
    d[k:2 * k, 2] = 0
    # exact diagonals from voxel centres: multi-axis ties
    c = rng.integers(0, min(nx, ny, nz), (k, 3)).astype(np.float32) + 0.5
    o[2 * k:3 * k] = c
    d[2 * k:3 * k] = rng.choice([-1.0, 1.0], (k, 3)).astype(np.float32)
    d[2 * k:2 * k + k // 2, 2] = 0
    # origins on voxel corners (integer coordinates)
    o[3 * k:4 * k] = rng.integers(0, min(nx, ny, nz) + 1, (k, 3)).astype(np.float32)
    # degenerate: tiny components whose len/d overflows, zero vectors, and non-finite input
    d[4 * k:4 * k + 8] = np.array([1.0, 1e-39, 0.0], np.float32)
    o[4 * k:4 * k + 8, 1] = ny  # on the top face: side = 0 * inf = NaN
    d[4 * k + 8] = 0.0
    d[4 * k + 9] = np.array([np.inf, 1, 0], np.float32)
    o[4 * k + 10] = np.array([np.nan, 1, 1], np.float32)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def entry_cases(rng, n):
    mp = (rng.random((n, 3)) - 0.5).astype(np.float32)
    # put a third of the entry points on cube faces, like rasterised front faces
    k = n // 3
    ax = rng.integers(0, 3, k)
    mp[np.arange(k), ax] = rng.choice([-0.5, 0.5], k).astype(np.float32)
    s = rng.normal(size=(n, 3)).astype(np.float32)
    s[: n // 10, 1:] = 0
    s[n // 10: n // 5, 0] = 0
    return mp, s


def main():
    rng = np.random.default_rng(20261203)
    cases = {
        "sparse16": ((16, 16, 16), 0.06),
        "dense8": ((8, 8, 8), 0.5),
        "odd_24x40x32": ((32, 40, 24), 0.03),  # (nz, ny, nx): not multiples of 8
    }
    for name, (shape, density) in cases.items():
        vox = sparse_grid(rng, shape, density)
        pal = palette(rng)
        g = po.Grid(vox, pal)
        dims = (g.nx, g.ny, g.nz)
        # 1. entry-point form against the reference shader itself (power-of-two sizes only:
        #    the shader samples texel voxel/size, exact for powers of two)
        pot = all(x & (x - 1) == 0 for x in dims)
        mp, s = entry_cases(rng, 4000)
        ora = po.trace_entry_points(g, mp, s)
        if pot:
            ref = po.ref_trace(g, mp, s, "select")
            bad = np.nonzero((ref[:, 0] != ora[:, 0]) | (ref[:, 4] != ora[:, 4]) |
                             ((ref[:, 0] == 1) & (ref[:, 1:4] != ora[:, 1:4]).any(1)))[0]
            if len(bad):
                raise SystemExit("%s: oracle differs from trace.frag on %d cases, first %r %r"
                                 % (name, len(bad), ref[bad[0]], ora[bad[0]]))
        # 2. ray-buffer and render forms from the oracle
        rays = ray_cases(rng, 4000, dims)
        hits = po.trace_rays(g, rays, threads=1)
        cam = po.make_camera({
            "origin": [-0.5 * dims[0], 1.7 * dims[1], -0.9 * dims[2]],
            "forward": [0.55, -0.55, 0.63], "right": [0.42, 0.0, -0.37],
            "up": [0.21, 0.52, 0.27], "width": 40, "height": 30})
        light = po.make_light([0.3, 0.8, 0.52], 0.25, True)
        img = po.render(g, cam, light, threads=1)
        np.savez_compressed(
            os.path.join(OUT, "%s.npz" % name), voxels=vox, palette=pal, entry_mp=mp,
            entry_s=s, entry_expected=ora, entry_pinned_to_reference=np.array(pot), rays=rays,
            ray_hits=hits.view(np.uint8).reshape(-1, 16), cam_origin=np.array(cam.origin),
            cam_forward=np.array(cam.forward), cam_right=np.array(cam.right),
            cam_up=np.array(cam.up), cam_size=np.array([cam.width, cam.height]),
            light=np.array(list(light.dir) + [light.ambient, light.shadows], np.float32),
            render_hits=img.view(np.uint8).reshape(-1, 16))
        print("%s: %d entry cases (%s), %d rays (%d hits), %dx%d render" % (
            name, len(mp), "pinned to trace.frag" if pot else "oracle only", len(rays),
            int((hits["face"] & po.FLAG_HIT).astype(bool).sum()), cam.width, cam.height))


if __name__ == "__main__":
    main()
