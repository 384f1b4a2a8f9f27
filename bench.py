#!/usr/bin/env python3
"""Benchmark: first-hit voxel traversal throughput (Mrays/s) on one GB300.

Workload (default ``shapes1024``): a 1024^3 u8 palette-index grid with 10,000 seeded boxes and
spheres (radius 2-40), rendered at 1920x1080 with one primary ray per pixel plus one hard-shadow
ray per lit hit toward a seeded directional light.  A step is one frame: one ``vt_render``
launch over the whole image.  Rays counted = primary rays + shadow rays actually traced.

  value        device time of the render kernel (CUDA events on the launching stream), grid
               resident in HBM, L2 flushed (256 MiB write) between timed frames
  e2e          the same frame through ``vt_render_host``: camera/light in, all hit records copied
               back to pinned host memory every step, host wall clock
  roofline     algorithmic bytes of the render kernel per launch (per ray: 4 B per brick
               directory entry visited, 64 B per occupied-brick mask entered, 5 B payload and
               palette per hit, 16 B hit record) / kernel time, against the measured HBM copy
               bandwidth
  cpu_baseline the CPU oracle (the reference traversal restated in C) on bands of rows of the same
               frame, all host cores

``--impl reference`` times that CPU restatement alone (rank 0 only).  Under torchrun (N > 1) each
rank renders its own replica of the frame (replicas only: rays are independent and nothing is
exchanged); value = all ranks' rays / max-over-ranks time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s (1080p, 1024^3 grid)"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=["shapes1024", "terrain256", "cave512", "multiview", "serve",
                                        "pager_world", "pathtrace", "paging"],
                   default="shapes1024")
    p.add_argument("--serve-requests", type=int, default=1000,
                   help="requests of the serving comparison added to the headline run (0: skip)")
    p.add_argument("--cpu-seconds", type=float, default=2.0,
                   help="wall-clock budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--views", type=int, default=64,
                   help="views of the multiview configuration (fewer for small profiling runs)")
    return p.parse_args()


def path_launches(tuning, spp, bounces, pixels):
    """Kernels one vt_path_trace launches under `tuning`, per frame.

    Wavefront form, per chunk of samples (up to 16 spp, 16M paths): the vertex-0 kernel, then
    per later vertex the path-ray trace, the shading, the sun-ray trace and the sun light, then
    the resolve.  Persistent form: the path kernel and the resolve
    per chunk (up to 16 spp, 64M samples).  Per-pixel form: one kernel."""
    if tuning["wavefront"]:
        sn = max(1, min(spp, 16, (16 << 20) // pixels))
        return -(-spp // sn) * (2 + 4 * bounces)
    if tuning["persistent"]:
        sn = max(1, min(spp, 16, (64 << 20) // pixels))
        return -(-spp // sn) * 2
    return 1


def max_over_ranks(x, device):
    """The largest of every rank's `x` (all ranks call it; one all-reduce)."""
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, seconds, world):
    """Whole-job rate of `world` replicas that each processed `units_per_rank` units, timed by
    the slowest rank's `seconds` (weak scaling, no data-path exchange)."""
    return world * units_per_rank / seconds


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def profiled_traffic(workload):
    """DRAM bytes per launch of the render kernel from the committed ncu summary, or None."""
    import re
    path = os.path.join(ROOT, "profiles", "render_%s.md" % workload)
    try:
        m = re.search(r"\| dram_bytes_per_launch \| (\d+) \|", open(path).read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def build_workload(name):
    from vtrace_gb300 import workloads
    return workloads.shapes1024() if name == "shapes1024" else workloads.terrain256()


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        self.t0 = time.time()

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def cpu_sample(w, seconds, threads=0, frame=None):
    """The CPU oracle on bands of 8 rows spread over the frame until `seconds` of wall time; with
    the GPU's `frame` (hit records [H, W]) also the number of records of those bands that differ
    from the oracle's."""
    from oracle import pyoracle as po
    og = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"].as_dict())
    L = w["light"]
    light = po.make_light(list(L.dir), L.ambient, bool(L.shadows))
    threads = threads or po.hardware_threads()
    H = cam.height
    band = 8
    order = np.random.default_rng(0).permutation(H // band)
    rays = 0
    rows = 0
    differ = 0
    t0 = time.perf_counter()
    for b in order:
        r0 = int(b) * band
        hits, st = po.render(og, cam, light, threads=threads, stats=True, rows=(r0, r0 + band))
        rays += st["rays"]
        rows += band
        if frame is not None:
            got = frame[r0:r0 + band].view(np.uint8).reshape(-1, 16)
            differ += int((got != hits.view(np.uint8).reshape(-1, 16)).any(1).sum())
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    out = {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
           "sample": "%d of %d rows of the %dx%d frame in 8-row bands (%d rays incl. shadow "
                     "rays), %.1f s wall" % (rows, H, cam.width, H, rays, dt)}
    if frame is not None:
        out["records_differing_from_gpu"] = differ
    return out


def tie_divergence(w, grid, n=1 << 18):
    """Seeded uniform rays in the grid, traced on the GPU and by the oracle in binary32 and
    binary64: binary32 records that differ (must be 0), rays whose binary32 and binary64 hits
    differ, and those of them that pass an exact binary32 tie (an iteration stepping two or three
    axes at once)."""
    import torch
    import vtrace_gb300 as vt
    from oracle import pyoracle as po
    nx = w["voxels"].shape[::-1]
    rays = vt.gen_rays_uniform(nx, 77, n)
    d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    vt.trace_rays(grid, d_rays, n, d_hits)
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(vt.HIT_DTYPE)
    og = po.Grid(w["voxels"], w["palette"])
    h32 = po.trace_rays(og, rays)
    h64 = po.trace_rays_f64(og, rays)
    hit = (h32["face"] & po.FLAG_HIT) != 0
    same = hit & (h64["hit"] == 1) & (h32["x"] == h64["v"][:, 0]) & (h32["y"] == h64["v"][:, 1]) & \
        (h32["z"] == h64["v"][:, 2]) & ((h32["face"] & 7) == h64["face"])
    div = np.nonzero((hit != (h64["hit"] == 1)) | (hit & ~same))[0]
    tie_div = sum(1 for i in div if po.trace_rays(og, rays[i:i + 1], stats=True)[1]["ties"] > 0)
    return {"rays": n, "gpu_records_differing_from_oracle":
            int((got.view(np.uint8).reshape(-1, 16) != h32.view(np.uint8).reshape(-1, 16)).any(1).sum()),
            "fp64_divergent_rate": len(div) / n, "tie_divergent_rate": tie_div / n,
            "note": "uniform rays in the benchmark grid; divergence from binary64 is the binary32 "
                    "recurrence resolving near-ties (within rounding of an edge) differently"}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    from oracle import pyoracle as po
    w = build_workload(args.config)
    og = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"].as_dict())
    L = w["light"]
    light = po.make_light(list(L.dir), L.ambient, bool(L.shadows))
    threads = po.hardware_threads()
    H = cam.height
    # a step renders one contiguous band of rows at a seeded offset (bands cycle over the
    # frame); the band is sized to ~0.25 s from a first 8-row sample and capped so the whole
    # run stays within a few minutes
    t0 = time.perf_counter()
    po.render(og, cam, light, threads=threads, rows=(H // 2, H // 2 + 8))
    per_row = (time.perf_counter() - t0) / 8
    rows_per_step = max(1, min(H, int(0.25 / max(per_row, 1e-6))))
    budget_rows = int(150.0 / max(per_row, 1e-6))
    rows_per_step = max(1, min(rows_per_step, budget_rows // max(1, args.steps + args.warmup)))
    offsets = np.random.default_rng(1).integers(0, H - rows_per_step + 1, args.steps + args.warmup)

    def step(k):
        r0 = int(offsets[k])
        _, st = po.render(og, cam, light, threads=threads, stats=True,
                          rows=(r0, r0 + rows_per_step))
        return st["rays"]

    for k in range(args.warmup):
        step(k)
    rays = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        rays += step(args.warmup + k)
    dt = time.perf_counter() - t0
    value = rays / dt / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": w["name"], "sample_rows_per_step": rows_per_step},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": "a band of %d contiguous rows of the frame per step at "
                                   "seeded offsets, %d host threads" % (rows_per_step, threads)},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import vtrace_gb300 as vt

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    vt.init(dev)
    w = build_workload(args.config)
    cam, light = w["camera"], w["light"]
    grid = vt.Grid.from_u8(w["voxels"], w["palette"])
    npx = cam.width * cam.height
    d_hits = torch.empty(npx * 16, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()  # the render and its events share this stream
    torch.cuda.set_stream(stream)

    # counters of one frame (counting kernel, not timed): rays traced and algorithmic bytes, and
    # the frame's distinct footprint
    stats = vt.render_stats(grid, cam, light, d_hits)
    fp = vt.render_footprint(grid, cam, light, d_hits)
    unique_bytes = (4 * fp["bricks"] + 64 * fp["nonempty_bricks"] + 512 * fp["hit_bricks"] +
                    16 * npx)
    rays_per_frame = stats["rays"]
    algo_bytes = (4 * stats["bricks_entered"] + 64 * stats["nonempty_bricks_entered"] +
                  5 * stats["hits"] + 16 * npx)
    # the per-ray figure as first written for this path: a 64-byte mask for every brick entered,
    # empty or not, 1 B per voxel tested in occupied bricks, 4 B palette entry per hit, 16 B record
    spec_bytes = (64 * stats["bricks_entered"] + stats["voxels_tested"] + 4 * stats["hits"] +
                  16 * npx)

    for _ in range(args.warmup):
        vt.render(grid, cam, light, d_hits, stream)
    torch.cuda.synchronize()
    shadow_rays = int(((d_hits.view(-1, 16)[:, 7] & vt.FLAG_SHADOW_RAY) != 0).sum().item())
    assert shadow_rays + npx == rays_per_frame, (shadow_rays, npx, rays_per_frame)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.fill_(k & 0xFF)  # 256 MiB write: evicts the 129 MB L2 between frames
        starts[k].record(stream)
        vt.render(grid, cam, light, d_hits, stream)
        ends[k].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    value = replica_rate(rays_per_frame, ms * 1e-3, world) / 1e6

    # end to end through the C ABI with a pinned host output buffer
    host_out = torch.empty(npx * 16, dtype=torch.uint8, pin_memory=True)
    for _ in range(2):
        vt.render_host(grid, cam, light, out=host_out)
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vt.render_host(grid, cam, light, out=host_out)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_times) / len(e2e_times)
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e = {"value": replica_rate(rays_per_frame, e2e_s, world) / 1e6, "unit": "Mrays/s",
           "h2d_bytes_per_step": 76, "d2h_bytes_per_step": npx * 16,
           "path": "vt_render_host (C ABI), pinned host output"}

    peak, peak_kind = measured_peak()
    achieved = algo_bytes / (ms * 1e-3) / 1e9
    metric = METRIC if args.config == "shapes1024" else "Mrays/s (%dx%d, %d^3 grid)" % (
        cam.width, cam.height, w["voxels"].shape[0])
    line = {
        "metric": metric, "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators, no dataset)",
        "config": {"workload": w["name"], "grid": list(w["voxels"].shape[::-1]),
                   "image": [cam.width, cam.height], "spp": 1, "shadow_rays": shadow_rays,
                   "rays_per_frame": rays_per_frame, "l2": "flushed (256 MiB write) between "
                   "timed frames", "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": e2e,
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": profiled_traffic("shapes1024_1080p") if args.config == "shapes1024" else None,
                     "traffic_source": "profiles/render_shapes1024_1080p.md (ncu, one launch)",
                     "algorithmic_bytes_per_launch": algo_bytes,
                     "kernel": "vt::render_kernel<false>",
                     "as_first_specified": {
                         "bytes_per_launch": spec_bytes,
                         "achieved": spec_bytes / (ms * 1e-3) / 1e9,
                         "frac": spec_bytes / (ms * 1e-3) / 1e9 / peak,
                         "note": "64 B per brick entered including empty ones (the brick layout "
                         "reads a 4 B directory entry there) + 1 B per voxel tested + 4 B per hit "
                         "+ 16 B record"},
                     "unique_footprint": {
                         "bytes_per_launch": unique_bytes,
                         "achieved": unique_bytes / (ms * 1e-3) / 1e9,
                         "frac": unique_bytes / (ms * 1e-3) / 1e9 / peak,
                         "bricks": fp, "note": "distinct directory entries x 4 B + masks x 64 B "
                         "+ hit bricks' payload x 512 B + 16 B records, along the reference's "
                         "iteration path"}},
        "clocks": clocks,
        "grid_info": grid.info(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        frame = d_hits.cpu().numpy().view(vt.HIT_DTYPE).reshape(cam.height, cam.width)
        line["cpu_baseline"] = cpu_sample(w, args.cpu_seconds, frame=frame)
        line["parity"] = tie_divergence(w, grid)
    grid.destroy()
    del d_hits
    if rank == 0 and args.serve_requests > 0 and world == 1 and args.config == "shapes1024":
        line["serve"] = serve_compare(args.serve_requests, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def serve_run(vt, svc_kwargs, scenes, reqs, torch):
    """Feeds `reqs` at their Poisson arrival times into a service; returns latency/throughput."""
    import threading
    svc = vt.Service(**svc_kwargs)
    try:
        sids = [svc.add_scene(sc["voxels"], sc["palette"]) for sc in scenes]
        sizes = [r["camera"].width * r["camera"].height * 4 for r in reqs]
        out = torch.empty(sum(sizes), dtype=torch.uint8, pin_memory=True)
        offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        # warm the grid cache (scene builds are not part of request latency)
        for sid, sc in zip(sids, scenes):
            c = vt.camera_look_at((-1.0, 1.0, -1.0), (1.0, 1.0, 1.0), (0, 1, 0), 60.0, 8, 8)
            svc.wait(svc.submit(sid, c, out[:256].data_ptr(), 1))
        ids = [None] * len(reqs)
        t0 = time.perf_counter() + 0.05

        def feeder():
            for k, r in enumerate(reqs):
                delay = t0 + r["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                ids[k] = svc.submit(sids[r["scene"]], r["camera"], out.data_ptr() + int(offs[k]),
                                    r["spp"], r["seed"], r["view_id"], r["light"])

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        timings = [svc.wait(i, 600.0) for i in ids]
        st = svc.stats()
    finally:
        svc.stop()
    lat = np.array([(t["done_ns"] - t["submit_ns"]) / 1e6 for t in timings])
    first = min(t["submit_ns"] for t in timings)
    last = max(t["done_ns"] for t in timings)
    samples = sum(t["samples"] for t in timings)
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "makespan_s": (last - first) / 1e9,
            "msamples_per_s": samples / ((last - first) / 1e9) / 1e6,
            "launches": st["launches"] - len(scenes), "requests": len(reqs)}


def serve_compare(n_requests, stream=None, n_scenes=32):
    """Batched continuous serving vs plain per-request launches on the same Poisson stream."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import workloads
    scenes = workloads.serving_scenes(n_scenes)
    reqs = workloads.serving_requests(scenes, n_requests)
    batched = serve_run(vt, {}, scenes, reqs, torch)
    plain = serve_run(vt, {"plain": True}, scenes, reqs, torch)
    # the same requests all submitted at once: the offered load is above either mode's capacity,
    # so the makespan measures throughput
    burst = [dict(r, t=0.0) for r in reqs]
    batched_sat = serve_run(vt, {}, scenes, burst, torch)
    plain_sat = serve_run(vt, {"plain": True}, scenes, burst, torch)
    return {"workload": "%d scenes 128^3-1024^3, %d requests, Poisson 2000/s, 320x240-1920x1080, "
                        "1-8 spp (rays = camera samples)" % (n_scenes, n_requests),
            "batched": batched, "plain": plain,
            "throughput_ratio": batched["msamples_per_s"] / plain["msamples_per_s"],
            "p99_ratio": batched["p99_ms"] / plain["p99_ms"],
            "saturated": {"batched": batched_sat, "plain": plain_sat,
                          "throughput_ratio": batched_sat["msamples_per_s"] / plain_sat["msamples_per_s"],
                          "p99_ratio": batched_sat["p99_ms"] / plain_sat["p99_ms"]}}


def run_config(args):
    """Non-headline configurations: one JSON line each (measured parity cases)."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import workloads, autotune
    torch.cuda.set_device(0)
    vt.init(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    line = {"steps": args.steps, "warmup": args.warmup, "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (seeded generators, no dataset)"}
    if args.config == "cave512":
        w = workloads.cave512()
        g = vt.Grid.from_u8(w["voxels"], w["palette"])
        n = w["rays"].shape[0]
        d_rays = torch.from_numpy(w["rays"].view(np.uint8).reshape(-1)).cuda()
        d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
        ms = autotune.time_ms(lambda: vt.trace_rays(g, d_rays, n, d_hits, stream), stream,
                              repeats=args.steps, warmup=args.warmup, flush=flush)
        st = vt.trace_rays_stats(g, d_rays, n, d_hits)
        host_rays = torch.from_numpy(w["rays"]).pin_memory()
        host_hits = torch.empty(n * 16, dtype=torch.uint8, pin_memory=True)
        vt.lib().vt_trace_rays_host(g.id, host_rays.data_ptr(), n, host_hits.data_ptr())
        t0 = time.perf_counter()
        for _ in range(args.steps):
            vt.check(vt.lib().vt_trace_rays_host(g.id, host_rays.data_ptr(), n, host_hits.data_ptr()))
        e2e_s = (time.perf_counter() - t0) / args.steps
        algo = 40 * n + 4 * st["bricks_entered"] + 64 * st["nonempty_bricks_entered"]
        peak, kind = measured_peak()
        line.update(metric="Mrays/s (16M incoherent rays, 512^3 cave)", value=n / ms / 1e3,
                    unit="Mrays/s", ms_per_step=ms, config={"workload": w["name"]},
                    e2e={"value": n / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n,
                         "d2h_bytes_per_step": 16 * n},
                    roofline={"bound": "hbm", "achieved": algo / ms / 1e6, "peak": peak,
                              "unit": "GB/s", "frac": algo / ms / 1e6 / peak,
                              "peak_source": kind, "algorithmic_bytes_per_launch": algo},
                    tuning=vt.get_tuning(vt.KERNEL_TRACE_RAYS), gpu_launches=args.steps)
        g.destroy()
    elif args.config == "multiview":
        scenes, views = workloads.multiview(n_views=args.views)
        grids = [vt.Grid.from_u8(sc["voxels"], sc["palette"]) for sc in scenes]
        bufs, specs = [], []
        for v in views:
            c = v["camera"]
            b = torch.empty(c.width * c.height * v["spp"] * 16, dtype=torch.uint8, device="cuda")
            bufs.append(b)
            specs.append(vt.make_view(grids[v["scene"]], c, b, v["spp"], v["seed"], v["view_id"],
                                      v["light"]))
        batch = vt.Batch(specs)
        ms = autotune.time_ms(lambda: batch.run(stream), stream, repeats=args.steps,
                              warmup=args.warmup, flush=flush)
        shadow = sum(int(((b.view(-1, 16)[:, 7] & vt.FLAG_SHADOW_RAY) != 0).sum().item()) for b in bufs)
        rays = batch.primary_rays + shadow
        singles = [vt.Batch([sp]) for sp in specs]
        ms_single = autotune.time_ms(lambda: [x.run(stream) for x in singles], stream,
                                     repeats=max(1, args.steps // 2), warmup=1, flush=flush)
        line.update(metric="Mrays/s (%d views over 8 scenes, 1-4 spp, one graph replay)" % len(views),
                    value=rays / ms / 1e3, unit="Mrays/s", ms_per_step=ms,
                    config={"workload": "multiview", "views": len(views),
                            "primary_rays": batch.primary_rays, "shadow_rays": shadow},
                    per_view_launches={"ms": ms_single, "value": rays / ms_single / 1e3},
                    gpu_launches=args.steps)
        for x in singles + [batch]:
            x.destroy()
        for gr in grids:
            gr.destroy()
    elif args.config == "pathtrace":
        # multi-bounce diffuse path tracing over the 1024^3 shapes grid at 1080p
        w = workloads.shapes1024()
        g = vt.Grid.from_u8(w["voxels"], w["palette"])
        cam = w["camera"]
        p = vt.make_path_params(spp=2, max_bounces=3, seed=1, sun_dir=tuple(w["light"].dir))
        d_out = torch.empty(cam.width * cam.height * 16, dtype=torch.uint8, device="cuda")
        d_rays = torch.zeros(1, dtype=torch.int64, device="cuda")
        vt.path_trace(g, cam, p, d_out, d_rays, stream)
        torch.cuda.synchronize()
        rays = int(d_rays.item())
        ms = autotune.time_ms(lambda: vt.path_trace(g, cam, p, d_out, None, stream), stream,
                              repeats=args.steps, warmup=args.warmup, flush=flush)
        p8 = vt.make_path_params(spp=2, max_bounces=3, seed=1, sun_dir=tuple(w["light"].dir),
                                 out_format=vt.PATH_OUT_RGBA8)
        host_img = torch.empty(cam.width * cam.height * 4, dtype=torch.uint8, pin_memory=True)
        vt.path_trace_host(g, cam, p8, out=host_img)
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 4)):
            vt.path_trace_host(g, cam, p8, out=host_img)
        e2e_s = (time.perf_counter() - t0) / max(1, args.steps // 4)
        line.update(metric="Mrays/s (path tracing, 1080p, 1024^3 grid, 2 spp, 3 bounces + sun)",
                    value=rays / ms / 1e3, unit="Mrays/s", ms_per_step=ms,
                    config={"workload": w["name"] + "_pt_spp2_b3", "rays_per_frame": rays,
                            "samples_per_frame": cam.width * cam.height * 2},
                    e2e={"value": rays / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 96,
                         "d2h_bytes_per_step": cam.width * cam.height * 4,
                         "path": "vt_path_trace_host (C ABI), RGBA8 out to pinned host memory"},
                    gpu_launches=path_launches(vt.get_tuning(vt.KERNEL_PATH), 2, 3,
                                               cam.width * cam.height) * args.steps)
        if not args.no_cpu_baseline:
            from oracle import pyoracle as po
            og = po.Grid(w["voxels"], w["palette"])
            op = po.make_path_params(2, 3, 1, list(p.sky), list(p.sun_dir), list(p.sun))
            rows = (cam.height // 2 - 4, cam.height // 2 + 4)
            t0 = time.perf_counter()
            band, band_rays = po.path_trace(og, po.make_camera(cam.as_dict()), op, rows=rows)
            cpu_s = time.perf_counter() - t0
            got = d_out.cpu().numpy().view(np.float32).reshape(cam.height, cam.width, 4)
            line["cpu_baseline"] = {"value": band_rays / cpu_s / 1e6, "unit": "Mrays/s",
                                    "cores": po.hardware_threads(), "kind": "port",
                                    "sample": "rows %d-%d of the frame (%d rays)" % (rows[0], rows[1] - 1, band_rays)}
            line["parity"] = {"band_pixels_differing_from_oracle":
                              int((got[rows[0]:rows[1]] != band).any(-1).sum())}
        g.destroy()
    elif args.config == "paging":
        # chunk streaming into the resident 1024^3 grid: 16^3 chunks written in place
        w = workloads.shapes1024()
        g = vt.Grid.from_u8(w["voxels"], w["palette"])
        rng = np.random.default_rng(9)
        n = w["voxels"].shape[0]
        chunks = []
        for k in range(args.steps + args.warmup):
            org = tuple(int(rng.integers(0, n // 16)) * 16 for _ in range(3))
            fill = k % 2 == 0
            c = np.where(rng.random((16, 16, 16)) < 0.3, rng.integers(1, 256, (16, 16, 16)), 0) if fill else np.zeros((16, 16, 16))
            chunks.append((org, np.ascontiguousarray(c.astype(np.uint8))))
        for org, c in chunks[:args.warmup]:
            g.update(org, c)
        t0 = time.perf_counter()
        for org, c in chunks[args.warmup:]:
            g.update(org, c)
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        cam, light = w["camera"], w["light"]
        d_hits = torch.empty(cam.width * cam.height * 16, dtype=torch.uint8, device="cuda")
        frame_ms = autotune.time_ms(lambda: vt.render(g, cam, light, d_hits, stream), stream,
                                    repeats=10, warmup=2, flush=flush)
        line.update(metric="chunk updates/s (16^3 chunks written into a resident 1024^3 grid)",
                    value=1e3 / ms, unit="chunks/s", ms_per_step=ms,
                    config={"workload": "shapes1024_paging_16cube", "chunk_bytes": 4096,
                            "bricks_total": g.info()["bricks_total"]},
                    e2e={"value": 1e3 / ms, "unit": "chunks/s", "h2d_bytes_per_step": 4096,
                         "d2h_bytes_per_step": 8 * 2 * 8 + 8,
                         "path": "vt_grid_update (C ABI), synchronous, host wall clock"},
                    frame_after_updates_ms=frame_ms,
                    # merge, scatter, 3 distance, 3 octant, run and long-box kernels per chunk
                    gpu_launches=10 * args.steps)
        g.destroy()
    elif args.config == "pager_world":
        # the reference-compatible frame (render_tick) over vtrace's own world shape
        import ctypes
        world = workloads.pager_world()
        os.environ["VTRACE_WIDTH"], os.environ["VTRACE_HEIGHT"] = (str(world["width"]),
                                                                  str(world["height"]))
        L = vt.lib()
        assert L.entry() == 0
        t0 = time.perf_counter()
        for t in world["textures"]:
            nz, ny, nx = t.shape
            vt.check(L.add_texture(t.ctypes.data, nx, ny, nz))
        upload_s = time.perf_counter() - t0
        insts = world["instances"]
        ptr = L.start_update_instances(len(insts))
        ctypes.memmove(ptr, insts.ctypes.data, insts.nbytes)
        vt.check(L.end_update_instances(len(insts)))
        info = vt.RenderTickInfo(world["P"].ctypes.data, world["C"].ctypes.data)
        ww, hh = ctypes.c_int32(0), ctypes.c_int32(0)
        lib_stream = torch.cuda.ExternalStream(L.vt_get_stream())
        tick = lambda: vt.check(L.render_tick(ctypes.byref(ww), ctypes.byref(hh), ctypes.byref(info)))
        # device time of the frame's launches (instance records, binning, per-pixel kernel) on the
        # library stream
        ms = autotune.time_ms(tick, lib_stream, repeats=args.steps, warmup=args.warmup, flush=flush)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tick()
        e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
        fb = np.zeros((hh.value, ww.value, 4), np.uint8)
        vt.check(L.vt_framebuffer_download(fb.ctypes.data, fb.nbytes))
        L.cleanup()
        px = world["width"] * world["height"]
        line.update(metric="Mpixels/s (render_tick, %dx%d, %d instances)" % (
                        world["width"], world["height"], len(insts)),
                    value=px / ms / 1e3, unit="Mpixels/s", ms_per_step=ms,
                    config={"workload": world["name"], "textures": len(world["textures"]),
                            "instances": len(insts), "texture_upload_s": upload_s},
                    e2e={"value": px / e2e_ms / 1e3, "unit": "Mpixels/s",
                         "h2d_bytes_per_step": int(insts.nbytes) + 128, "d2h_bytes_per_step": 0,
                         "path": "render_tick (C ABI), host wall clock"},
                    # instance records, tile binning, per-pixel compositing
                    gpu_launches=3 * args.steps)
        if not args.no_cpu_baseline:
            from oracle import pyoracle as po
            grids = [po.Grid(texels=t) for t in world["textures"]]
            t0 = time.perf_counter()
            want = po.compat_render(grids, insts, world["P"], world["C"], world["width"],
                                    world["height"])
            cpu_s = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": px / cpu_s / 1e6, "unit": "Mpixels/s",
                                    "cores": po.hardware_threads(), "kind": "port",
                                    "sample": "the whole frame, every instance per pixel"}
            line["parity"] = {"pixels_differing_from_oracle": int((fb != want).any(-1).sum())}
    else:  # serve
        r = serve_compare(max(args.serve_requests, 2000))
        line.update(metric="serve p50/p99 latency and Msamples/s vs plain per-request launches",
                    value=r["batched"]["msamples_per_s"], unit="Msamples/s",
                    ms_per_step=r["batched"]["p50_ms"], config={"workload": r["workload"]},
                    serve=r)
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config in ("cave512", "multiview", "serve", "pager_world", "pathtrace", "paging"):
        return run_config(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
