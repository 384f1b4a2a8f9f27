"""Autotuner for the tracing launches.

For an entry point (VT_KERNEL_RENDER, VT_KERNEL_TRACE_RAYS or VT_KERNEL_BATCH) and a workload
callable, it times every candidate launch shape — tile launch vs persistent warps, the refill
threshold (how many idle lanes trigger a warp refill: the compaction interval), the resident
blocks per SM — with CUDA events on the launch stream, keeps the fastest and installs it with
vt_set_tuning.  The brick size is part of the grid layout (8^3, a 512-bit occupancy mask per
brick) and the warp width is fixed at one ray per lane, so they are not searched.
"""
import itertools

import numpy as np

from . import KERNEL_BATCH, get_tuning, set_tuning

DEFAULT_REFILL = (1, 4, 8, 16, 24, 32)
DEFAULT_BLOCKS = (0, 2)


def candidates(refill=DEFAULT_REFILL, blocks=DEFAULT_BLOCKS, tiles=True, wavefront=False):
    out = []
    if tiles:
        out.append({"refill_min": 32, "blocks_per_sm": 0, "persistent": False})
    if wavefront:
        out.append({"refill_min": 32, "blocks_per_sm": 0, "persistent": False, "wavefront": True})
    for r, b in itertools.product(refill, blocks):
        out.append({"refill_min": r, "blocks_per_sm": b, "persistent": True})
    return out


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
    created, rebuilds itself there).  Returns (best, {candidate key: ms})."""
    cands = cands or candidates(tiles=kernel != KERNEL_BATCH)
    saved = get_tuning(kernel)
    results = {}
    best, best_ms = None, float("inf")
    try:
        for c in cands:
            set_tuning(kernel, c["refill_min"], c["blocks_per_sm"], c["persistent"],
                       c.get("wavefront", False))
            if prepare is not None:
                prepare()
            ms = time_ms(run, stream, repeats=repeats, flush=flush)
            key = "%s_r%d_b%d" % ("persistent" if c["persistent"] else
                                  ("wavefront" if c.get("wavefront") else "tiles"),
                                  c["refill_min"], c["blocks_per_sm"])
            results[key] = ms
            if ms < best_ms:
                best, best_ms = c, ms
    finally:
        chosen = best or saved
        set_tuning(kernel, chosen["refill_min"], chosen["blocks_per_sm"], chosen["persistent"],
                   chosen.get("wavefront", False))
        if prepare is not None:
            prepare()
    return best, results
