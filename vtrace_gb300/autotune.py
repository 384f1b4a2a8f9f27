"""Autotuner for the tracing launches.

For an entry point (VT_KERNEL_RENDER, VT_KERNEL_TRACE_RAYS or VT_KERNEL_BATCH) and a workload
callable, it times every candidate launch shape with CUDA events on the launch stream, keeps the
fastest and installs it with vt_set_tuning.  The search spaces:

  render       the fused tile launch over warp tiles of 8x4, 4x8, 16x2 and 32x1 pixels and blocks
               of 1, 2, 4 and 8 warps (the pixel-tile shape and rays per block); the two-pass form
               (shadow rays compacted into full warps by a second kernel); persistent warps
               refilled once 8, 16 or 32 lanes are idle (the compaction interval); persistent
               warps taking whole tiles and tracing their queued shadow rays 32 at a time
  trace_rays   one thread per ray, or persistent warps with a refill threshold of 1, 4, 8, 16, 24
               or 32 idle lanes and 2 or as many as fit resident blocks per SM
  batch        whole tile units per warp over 8x4, 4x8, 16x2 and 32x1-pixel tiles, or per-lane
               refill at 4, 8 or 16 idle lanes, with 2 or as many as fit resident blocks per SM

The brick size is part of the grid layout (8^3, a 512-bit occupancy mask and a 512-byte payload
per brick: the mask is one 64-bit word per z-slice), and a warp traces one ray per lane, so
neither is searched.  Results do not depend on the choice: every candidate computes the same
records.
"""
import itertools

import numpy as np

from . import (KERNEL_BATCH, KERNEL_RENDER, KERNEL_TRACE_RAYS, TILE_4X8, TILE_8X4, TILE_16X2,
               TILE_32X1, TILE_NAMES, get_tuning, set_tuning)

FIELDS = ("refill_min", "blocks_per_sm", "persistent", "wavefront", "tile_shape", "block_warps")


def tuning(refill_min=32, blocks_per_sm=0, persistent=False, wavefront=False,
           tile_shape=TILE_8X4, block_warps=4):
    return {"refill_min": refill_min, "blocks_per_sm": blocks_per_sm,
            "persistent": bool(persistent), "wavefront": bool(wavefront),
            "tile_shape": tile_shape, "block_warps": block_warps}


def render_candidates(tiles=(TILE_8X4, TILE_4X8, TILE_16X2, TILE_32X1), warps=(1, 2, 4, 8),
                      refill=(8, 16, 32)):
    out = [tuning(tile_shape=t, block_warps=w) for t, w in itertools.product(tiles, warps)]
    out.append(tuning(wavefront=True))
    out += [tuning(refill_min=r, persistent=True) for r in refill]
    out.append(tuning(persistent=True, wavefront=True))  # whole tiles, shadow rays in full warps
    return out


def rays_candidates(refill=(1, 4, 8, 16, 24, 32), blocks=(0, 2)):
    out = [tuning()]
    out += [tuning(refill_min=r, blocks_per_sm=b, persistent=True)
            for r, b in itertools.product(refill, blocks)]
    return out


def batch_candidates(refill=(4, 8, 16), blocks=(0, 2),
                     tiles=(TILE_8X4, TILE_4X8, TILE_16X2, TILE_32X1)):
    out = [tuning(refill_min=32, blocks_per_sm=b, persistent=True, tile_shape=t)
           for t, b in itertools.product(tiles, blocks)]
    out += [tuning(refill_min=r, blocks_per_sm=b, persistent=True)
            for r, b in itertools.product(refill, blocks)]
    return out


def candidates(kernel):
    return {KERNEL_RENDER: render_candidates, KERNEL_TRACE_RAYS: rays_candidates,
            KERNEL_BATCH: batch_candidates}[kernel]()


def key(kernel, c):
    """A short name of candidate `c` of `kernel`."""
    if kernel == KERNEL_BATCH:
        form = ("tiles_%s" % TILE_NAMES[c["tile_shape"]] if c["refill_min"] >= 32
                else "lanes_r%d" % c["refill_min"])
        return "%s_b%d" % (form, c["blocks_per_sm"])
    if c["persistent"] and c["wavefront"] and kernel == KERNEL_RENDER:
        return "queued_shadows_b%d" % c["blocks_per_sm"]
    if c["persistent"]:
        return "persistent_r%d_b%d" % (c["refill_min"], c["blocks_per_sm"])
    if c["wavefront"]:
        return "two_pass"
    if kernel == KERNEL_RENDER:
        return "tiles_%s_w%d" % (TILE_NAMES[c["tile_shape"]], c["block_warps"])
    return "tiles"


def install(kernel, c):
    set_tuning(kernel, **{f: c[f] for f in FIELDS})


def time_ms(fn, stream, repeats=5, warmup=2, flush=None):
    """Median device time of fn() in ms, CUDA events on `stream` (a torch.cuda.Stream)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for k in range(repeats):
        if flush is not None:
            flush.fill_(k & 0xFF)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def autotune(kernel, run, stream, cands=None, repeats=5, flush=None, prepare=None):
    """Times `run()` under each candidate tuning of `kernel` and installs the fastest.

    `prepare()` is called after each vt_set_tuning (a batch, whose shape is fixed when it is
    created, rebuilds itself there).  Returns (best, {candidate key: ms}); on an exception the
    tuning in force before the call is put back."""
    cands = cands or candidates(kernel)
    saved = get_tuning(kernel)
    results = {}
    best, best_ms = None, float("inf")
    try:
        for c in cands:
            install(kernel, c)
            if prepare is not None:
                prepare()
            ms = time_ms(run, stream, repeats=repeats, flush=flush)
            results[key(kernel, c)] = ms
            if ms < best_ms:
                best, best_ms = c, ms
    finally:
        install(kernel, best or saved)
        if prepare is not None:
            prepare()
    return best, results
