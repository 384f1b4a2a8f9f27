#!/usr/bin/env python3
"""Benchmark: first-hit voxel traversal throughput (Mrays/s) on one GB300.

Workload (default ``shapes1024``): a 1024^3 u8 palette-index grid with 10,000 seeded boxes and
spheres (radius 2-40), rendered at 1920x1080 with one primary ray per pixel plus one hard-shadow
ray per lit hit toward a seeded directional light.  A step is one frame: one ``vt_render``
launch over the whole image.  Rays counted = primary rays + shadow rays actually traced.

  value        device time of the render kernel (CUDA events on the launching stream), grid
               resident in HBM, L2 flushed (256 MiB write) between timed frames
  e2e          the same frame through ``vt_render_host``: camera/light in, all hit records written
               to pinned host memory every step, host wall clock
  roofline     algorithmic bytes of the render kernel per launch (per ray: 4 B per brick
               directory entry visited, 64 B per occupied-brick mask entered, 5 B payload and
               palette per hit, 16 B hit record) / kernel time, against the measured HBM copy
               bandwidth
  cpu_baseline the CPU oracle (the reference traversal restated in C) on the whole frame, all host
               cores; its records are compared with the GPU's
  tuning       the autotuner's choice and timing table for the render, ray-buffer and batch
               launches (installed before each is timed)
  parity       binary32 against binary64 traversal of the frame's own camera and shadow rays (and
               of uniform rays): divergence and tie-divergence rates, t accuracy
  terrain256, cave512, multiview
               the other traversal configurations (640x480 over 256^3; 16M incoherent rays in a
               512^3 cave; 64 views over 8 scenes in one graph replay), each with its device and
               end-to-end rate, roofline, CPU baseline, records compared with the oracle and the
               clocks sampled during its own timed region
  serve        continuous batching against plain per-request launches on a Poisson stream, with
               the fraction of the plain mode's makespan its kernels kept the GPU busy

``--impl reference`` times the reference traversal restated on the CPU (the oracle), whole frame
per step, on all host cores (rank 0 only); its process loads the oracle alone (the workload is
generated in a child process and handed over as arrays).  Under torchrun (N > 1) each rank
renders its own replica of the frame (replicas only: rays are independent and nothing is
exchanged); value = all ranks' rays / max-over-ranks time.
"""
import argparse
import json
import math
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s (1080p, 1024^3 grid)"
FALLBACK_HBM_GBS = 6800.0
L2_NOTE = "flushed (256 MiB write) between timed steps"


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
                   help="wall-clock budget of the bounded CPU samples (ray buffers, views)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="headline frame only (no terrain256 / cave512 / multiview keys)")
    p.add_argument("--no-tune", action="store_true", help="keep the library's default tunings")
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
    """DRAM bytes per launch of the render kernel from the committed ncu summary, with where and
    when that capture was made, or None."""
    import re
    path = os.path.join(ROOT, "profiles", "render_%s.md" % workload)
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"\| dram_bytes_per_launch \| (\d+) \|", text)
    if not m:
        return None
    when = re.search(r"^Captured: (.+)$", text, re.M)
    inst = re.search(r"\| warp_instructions_per_launch \| (\d+) \|", text)
    return {"bytes": int(m.group(1)), "source": "profiles/render_%s.md" % workload,
            "captured": when.group(1).strip() if when else None,
            "warp_instructions": int(inst.group(1)) if inst else None}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def roofline(algo_bytes, ms, kernel, **extra):
    peak, kind = measured_peak()
    achieved = algo_bytes / (ms * 1e-3) / 1e9
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": kind, "traffic": None,
           "algorithmic_bytes_per_launch": int(algo_bytes), "kernel": kernel}
    out.update(extra)
    return out


def phase_shares(prof):
    """Shares of the frame's warp time by ray kind and traversal phase (vt_render_phases)."""
    total = sum(sum(prof[k].values()) for k in ("camera", "shadow"))
    out = {k: {ph: round(v / total, 4) for ph, v in prof[k].items()} for k in ("camera", "shadow")}
    out["passes"] = prof["passes"]
    out["warps"] = prof["warps"]
    out["note"] = ("share of warp residency per phase (SM clock read at warp-synchronous points "
                   "of an instrumented build of the default 8x4-tile launch): load latency "
                   "included, which other warps hide in this issue-bound kernel, so not a "
                   "share of issue slots")
    return out


def stats_bytes(st, records, io_per_ray=0):
    """Algorithmic bytes of a launch from its traversal counters: 4 B per brick directory entry
    visited, 64 B per occupied brick's mask entered, 5 B per hit (payload byte + palette entry),
    16 B per record written, plus `io_per_ray` B of ray input per ray."""
    return (4 * st["bricks_entered"] + 64 * st["nonempty_bricks_entered"] + 5 * st["hits"] +
            16 * records + io_per_ray * st["rays"])


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


def timed_steps(fn, stream, steps, flush, min_seconds=0.0, est_ms=None):
    """Device time per step of fn() (CUDA events on `stream`, L2 flushed before each step) over
    `steps` steps, or more when `min_seconds` asks for a longer timed region (so that the clock
    sampler sees it).  Returns (mean ms, steps run)."""
    import torch
    if min_seconds > 0 and est_ms:
        steps = max(steps, int(math.ceil(min_seconds * 1e3 / (est_ms + 0.05))))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps, steps


# ------------------------------------------------------------------ workload handoff

def save_workload(name, path):
    """Writes workload `name` (camera, light, voxels, palette) under directory `path`; run in a
    child process by the reference arm, which itself never loads libvtrace."""
    from vtrace_gb300 import workloads
    w = workloads.shapes1024() if name == "shapes1024" else workloads.terrain256()
    np.save(os.path.join(path, "voxels.npy"), w["voxels"])
    np.save(os.path.join(path, "palette.npy"), w["palette"])
    L = w["light"]
    meta = {"name": w["name"], "camera": w["camera"].as_dict(),
            "light": {"dir": list(L.dir), "ambient": L.ambient, "shadows": bool(L.shadows)}}
    with open(os.path.join(path, "meta.json"), "w") as f:
        json.dump(meta, f)


def load_workload(path):
    with open(os.path.join(path, "meta.json")) as f:
        meta = json.load(f)
    meta["voxels"] = np.load(os.path.join(path, "voxels.npy"))
    meta["palette"] = np.load(os.path.join(path, "palette.npy"))
    return meta


def frame_config(name, voxels_shape, width, height, shadow_rays, rays_per_frame, world):
    return {"workload": name, "grid": list(voxels_shape[::-1]), "image": [width, height],
            "spp": 1, "shadow_rays": int(shadow_rays), "rays_per_frame": int(rays_per_frame),
            "l2": L2_NOTE, "parallelism": "replicas" if world > 1 else "single GPU"}


# ------------------------------------------------------------------ reference arm

def run_reference(args):
    """The oracle (the reference traversal restated in C, dense grid, no empty-space skipping)
    renders the whole frame each step on all host cores.  The workload is generated by a child
    process; this process maps the oracle's library only."""
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    from oracle import pyoracle as po
    tmp = tempfile.mkdtemp(prefix="vt_ref_workload_")
    try:
        code = ("import sys; sys.path.insert(0, %r); import bench; bench.save_workload(%r, %r)"
                % (ROOT, args.config if args.config == "terrain256" else "shapes1024", tmp))
        subprocess.run([sys.executable, "-c", code], check=True)
        w = load_workload(tmp)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    og = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"])
    L = w["light"]
    light = po.make_light(L["dir"], L["ambient"], L["shadows"])
    threads = po.hardware_threads()

    def step():
        _, st = po.render(og, cam, light, threads=threads, stats=True)
        return st

    for _ in range(args.warmup):
        step()
    rays = shadow = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = step()
        rays += st["rays"]
        shadow += st["shadow_rays"]
    dt = time.perf_counter() - t0
    value = rays / dt / 1e6
    metric = METRIC if args.config != "terrain256" else "Mrays/s (640x480, 256^3 grid)"
    line = {
        "metric": metric, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators, no dataset)", "impl": "reference",
        "config": frame_config(w["name"], w["voxels"].shape, cam.width, cam.height,
                               shadow // args.steps, rays // args.steps, 1),
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": "the whole %dx%d frame (%d rays incl. shadow rays) per step, "
                                   "%d host threads" % (cam.width, cam.height,
                                                        rays // args.steps, threads)},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ CPU samples and parity

def oracle_frame(w, threads=0, rows=None):
    from oracle import pyoracle as po
    og = po.Grid(w["voxels"], w["palette"])
    cam = po.make_camera(w["camera"].as_dict())
    L = w["light"]
    light = po.make_light(list(L.dir), L.ambient, bool(L.shadows))
    return og, cam, light


def cpu_frame(w, frame):
    """The CPU oracle on the whole frame, all host cores; with the GPU's `frame` (hit records
    [H, W]) the number of its records that differ from the oracle's."""
    from oracle import pyoracle as po
    og, cam, light = oracle_frame(w)
    threads = po.hardware_threads()
    t0 = time.perf_counter()
    hits, st = po.render(og, cam, light, threads=threads, stats=True)
    dt = time.perf_counter() - t0
    differ = int((frame.view(np.uint8).reshape(-1, 16) != hits.view(np.uint8).reshape(-1, 16)).any(1).sum())
    return {"value": st["rays"] / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": "the whole %dx%d frame (%d rays incl. shadow rays), %.2f s wall"
                      % (cam.width, cam.height, st["rays"], dt),
            "records_differing_from_gpu": differ}


def divergence(og, rays, gpu_hits=None):
    """binary32 (the reference's arithmetic) against binary64 traversal of `rays`: rays whose
    hit (flag, voxel, face) differs, those of them that pass an exact binary32 tie (an iteration
    stepping two or three axes at once), and the largest relative error of binary32 t where both
    agree."""
    from oracle import pyoracle as po
    h32 = po.trace_rays(og, rays)
    h64 = po.trace_rays_f64(og, rays)
    hit = (h32["face"] & po.FLAG_HIT) != 0
    same = hit & (h64["hit"] == 1) & (h32["x"] == h64["v"][:, 0]) & (h32["y"] == h64["v"][:, 1]) & \
        (h32["z"] == h64["v"][:, 2]) & ((h32["face"] & 7) == h64["face"])
    div = np.nonzero((hit != (h64["hit"] == 1)) | (hit & ~same))[0]
    tie_div = sum(1 for i in div if po.trace_rays(og, rays[i:i + 1], stats=True)[1]["ties"] > 0)
    both = same & (h64["t"] > 0)
    rel = np.abs(h32["t"][both].astype(np.float64) - h64["t"][both]) / h64["t"][both]
    out = {"rays": int(rays.shape[0]), "fp64_divergent": int(len(div)),
           "fp64_divergent_rate": len(div) / rays.shape[0], "tie_divergent": int(tie_div),
           "tie_divergent_rate": tie_div / rays.shape[0],
           "t_max_rel_err": float(rel.max()) if rel.size else 0.0,
           "t_rel_err_above_1e-5": int((rel > 1e-5).sum())}
    if gpu_hits is not None:
        out["gpu_records_differing_from_oracle"] = int(
            (gpu_hits.view(np.uint8).reshape(-1, 16) != h32.view(np.uint8).reshape(-1, 16)).any(1).sum())
    return out


def frame_parity(w, grid, frame):
    """Tie divergence on the headline frame's own rays (every camera ray, every shadow ray the
    frame traced) and on seeded uniform rays in the grid, the latter also traced on the GPU."""
    import torch
    import vtrace_gb300 as vt
    from oracle import pyoracle as po
    og, cam, light = oracle_frame(w)
    cam_rays, sh_rays = po.frame_rays(cam, light, frame)
    n = 1 << 18
    nx = w["voxels"].shape[::-1]
    rays = vt.gen_rays_uniform(nx, 77, n)
    d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    vt.trace_rays(grid, d_rays, n, d_hits)
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(vt.HIT_DTYPE)
    return {"camera_rays": divergence(og, cam_rays), "shadow_rays": divergence(og, sh_rays),
            "uniform_rays": divergence(og, rays.view(np.float32).reshape(-1, 6), got),
            "note": "binary32 is the reference's arithmetic (trace.frag:83-85) and the GPU matches "
                    "it bit for bit; binary64 resolves rays passing within rounding of a voxel "
                    "edge differently; tie_divergent counts those that also pass an exact "
                    "binary32 tie"}


# ------------------------------------------------------------------ our arm

def run_ours(args):
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import autotune

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    vt.init(dev)
    from vtrace_gb300 import workloads
    w = workloads.shapes1024() if args.config == "shapes1024" else workloads.terrain256()
    cam, light = w["camera"], w["light"]
    grid = vt.Grid.from_u8(w["voxels"], w["palette"])
    npx = cam.width * cam.height
    d_hits = torch.empty(npx * 16, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()  # the render and its events share this stream
    torch.cuda.set_stream(stream)

    tuning = {}
    if not args.no_tune:
        best, table = autotune.autotune(vt.KERNEL_RENDER,
                                        lambda: vt.render(grid, cam, light, d_hits, stream),
                                        stream, repeats=5, flush=flush)
        tuning["render"] = {"chosen": autotune.key(vt.KERNEL_RENDER, best), "ms": table}

    # counters of one frame (counting kernel, not timed): rays traced and algorithmic bytes, and
    # the frame's distinct footprint
    stats = vt.render_stats(grid, cam, light, d_hits)
    fp = vt.render_footprint(grid, cam, light, d_hits)
    phases = phase_shares(vt.render_phases(grid, cam, light, d_hits))
    unique_bytes = (4 * fp["bricks"] + 64 * fp["nonempty_bricks"] + 512 * fp["hit_bricks"] +
                    16 * npx)
    rays_per_frame = stats["rays"]
    algo_bytes = stats_bytes(stats, npx)
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

    metric = METRIC if args.config == "shapes1024" else "Mrays/s (%dx%d, %d^3 grid)" % (
        cam.width, cam.height, w["voxels"].shape[0])
    traffic = profiled_traffic("shapes1024_1080p") if args.config == "shapes1024" else None
    issue = None
    if traffic and traffic.get("warp_instructions") and clocks and clocks.get("sm_mhz"):
        # the kernel's real bound: warp instructions issued per second (count from the committed
        # ncu capture of the same launch, time from this run) against 4 issue slots per SM per
        # clock at the SM clock sampled during the timed region
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        achieved_gips = traffic["warp_instructions"] / (ms * 1e-3) / 1e9
        peak_gips = 4 * sms * clocks["sm_mhz"] * 1e6 / 1e9
        issue = {"bound": "issue", "achieved": achieved_gips, "peak": peak_gips,
                 "unit": "G warp instructions/s", "frac": achieved_gips / peak_gips,
                 "warp_instructions_per_launch": traffic["warp_instructions"],
                 "source": "instruction count of the default 8x4-tile launch from %s; 4 issue "
                           "slots x %d SMs x the SM clock sampled here" % (traffic["source"], sms)}
    line = {
        "metric": metric, "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators, no dataset)", "impl": "ours",
        "config": frame_config(w["name"], w["voxels"].shape, cam.width, cam.height, shadow_rays,
                               rays_per_frame, world),
        "e2e": e2e,
        "gpu_launches": args.steps,
        "roofline": roofline(
            algo_bytes, ms, "vt::render_kernel<false>",
            traffic=traffic["bytes"] if traffic else None,
            traffic_source=("%s (ncu, one launch, captured %s)" % (traffic["source"],
                                                                  traffic["captured"])
                            if traffic else None),
            as_first_specified={
                "bytes_per_launch": spec_bytes,
                "achieved": spec_bytes / (ms * 1e-3) / 1e9,
                "frac": spec_bytes / (ms * 1e-3) / 1e9 / measured_peak()[0],
                "note": "64 B per brick entered including empty ones (the brick layout reads a "
                        "4 B directory entry there) + 1 B per voxel tested + 4 B per hit + 16 B "
                        "record"},
            unique_footprint={
                "bytes_per_launch": unique_bytes,
                "achieved": unique_bytes / (ms * 1e-3) / 1e9,
                "frac": unique_bytes / (ms * 1e-3) / 1e9 / measured_peak()[0],
                "bricks": fp, "note": "distinct directory entries x 4 B + masks x 64 B + hit "
                "bricks' payload x 512 B + 16 B records, along the reference's iteration path"},
            issue=issue),
        "clocks": clocks,
        "grid_info": grid.info(),
        "phase_profile": phases,
    }
    if tuning:
        tuning["render"]["installed"] = vt.get_tuning(vt.KERNEL_RENDER)
    if rank == 0 and not args.no_cpu_baseline:
        frame = d_hits.cpu().numpy().view(vt.HIT_DTYPE).reshape(cam.height, cam.width)
        line["cpu_baseline"] = cpu_frame(w, frame)
        line["parity"] = frame_parity(w, grid, frame)
    extras = rank == 0 and world == 1 and args.config == "shapes1024" and not args.no_extras
    digest = grid_digest(grid) if extras else None
    grid.destroy()
    del d_hits
    if extras:
        line["grid_build"] = bench_build(w, digest, stream, dev)
        line["terrain256"] = bench_frame(args, workloads.terrain256(), stream, flush, dev)
        line["cave512"] = bench_rays(args, stream, flush, dev, tuning)
        line["multiview"] = bench_multiview(args, stream, flush, dev, tuning)
    if tuning:
        tuning["brick_size"] = "8^3, fixed by the grid layout (one 64-bit mask word per z-slice)"
        line["tuning"] = tuning
    if rank == 0 and args.serve_requests > 0 and world == 1 and args.config == "shapes1024":
        line["serve"] = serve_compare(args.serve_requests, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def grid_digest(grid):
    """SHA-256 of a grid's directory, masks and payloads (its brick layout)."""
    import hashlib
    h = hashlib.sha256()
    d, m = grid.bricks()
    for a in (d, m, grid.payload()):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def bench_build(w, digest, stream, dev, repeats=10, warmup=3):
    """The brick build of the headline grid from voxels already in device memory
    (vt_grid_create_u8_device, a synchronous call: words, scan, count readback, the grid's one
    allocation, compaction, distance, octant and long-box passes), timed by the host clock per call
    with the grid destroyed between calls; the layout must equal the host-input build's."""
    import torch
    import vtrace_gb300 as vt
    vox = w["voxels"]
    nz, ny, nx = vox.shape
    d_vox = torch.from_numpy(np.ascontiguousarray(vox).reshape(-1)).to("cuda")
    torch.cuda.synchronize()
    for _ in range(warmup):
        vt.Grid.from_u8_device(d_vox, (nx, ny, nz), w["palette"], stream).destroy()
    sampler = ClockSampler(dev)
    sampler.start()
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        g = vt.Grid.from_u8_device(d_vox, (nx, ny, nz), w["palette"], stream)
        times.append((time.perf_counter() - t0) * 1e3)
        g.destroy()
    clocks = sampler.stop()
    g = vt.Grid.from_u8_device(d_vox, (nx, ny, nz), w["palette"], stream)
    same = grid_digest(g) == digest
    info = g.info()
    g.destroy()
    del d_vox
    ms = float(np.median(times))
    return {"ms": ms, "ms_min": min(times), "repeats": repeats,
            "input_gbs": vox.nbytes / (ms * 1e-3) / 1e9, "input_bytes": int(vox.nbytes),
            "bricks_nonempty": info["bricks_nonempty"], "device_bytes": info["device_bytes"],
            "layout_equal_to_host_input_build": same,
            "path": "vt_grid_create_u8_device (C ABI), synchronous, host wall clock, grid destroyed "
                    "between calls (its allocation included)",
            "clocks": clocks}


def bench_frame(args, w, stream, flush, dev):
    """One render configuration (the frame of `w`): device and end-to-end rate, roofline, the
    whole frame against the oracle, clocks of its own timed region."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import autotune
    cam, light = w["camera"], w["light"]
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    npx = cam.width * cam.height
    d = torch.empty(npx * 16, dtype=torch.uint8, device="cuda")
    st = vt.render_stats(g, cam, light, d)
    run = lambda: vt.render(g, cam, light, d, stream)
    for _ in range(args.warmup):
        run()
    est = max(1e-3, autotune.time_ms(run, stream, 3, 0))
    sampler = ClockSampler(dev)
    sampler.start()
    ms, steps = timed_steps(run, stream, args.steps, flush, min_seconds=0.5, est_ms=est)
    clocks = sampler.stop()
    host = torch.empty(npx * 16, dtype=torch.uint8, pin_memory=True)
    vt.render_host(g, cam, light, out=host)
    t0 = time.perf_counter()
    reps = max(args.steps, 20)
    for _ in range(reps):
        vt.render_host(g, cam, light, out=host)
    e2e_s = (time.perf_counter() - t0) / reps
    out = {"metric": "Mrays/s (%dx%d, %d^3 grid)" % (cam.width, cam.height, w["voxels"].shape[0]),
           "value": st["rays"] / ms / 1e3, "unit": "Mrays/s", "ms_per_step": ms, "steps": steps,
           "config": frame_config(w["name"], w["voxels"].shape, cam.width, cam.height,
                                  st["shadow_rays"], st["rays"], 1),
           "e2e": {"value": st["rays"] / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 76,
                   "d2h_bytes_per_step": npx * 16,
                   "path": "vt_render_host (C ABI), pinned host output, host wall clock"},
           "roofline": roofline(stats_bytes(st, npx), ms, "vt::render_kernel<false>"),
           "gpu_launches": steps, "clocks": clocks}
    if not args.no_cpu_baseline:
        frame = d.cpu().numpy().view(vt.HIT_DTYPE).reshape(cam.height, cam.width)
        out["cpu_baseline"] = cpu_frame(w, frame)
    g.destroy()
    return out


def bench_rays(args, stream, flush, dev, tuning):
    """The incoherent ray buffer: 16,777,216 rays in the 512^3 cave through vt_trace_rays."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import autotune, workloads
    from oracle import pyoracle as po
    w = workloads.cave512()
    g = vt.Grid.from_u8(w["voxels"], w["palette"])
    n = w["rays"].shape[0]
    d_rays = torch.from_numpy(w["rays"].view(np.uint8).reshape(-1)).cuda()
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    run = lambda: vt.trace_rays(g, d_rays, n, d_hits, stream)
    if not args.no_tune:
        best, table = autotune.autotune(vt.KERNEL_TRACE_RAYS, run, stream, repeats=5, flush=flush)
        tuning["trace_rays"] = {"chosen": autotune.key(vt.KERNEL_TRACE_RAYS, best), "ms": table,
                                "installed": vt.get_tuning(vt.KERNEL_TRACE_RAYS)}
    st = vt.trace_rays_stats(g, d_rays, n, d_hits)
    for _ in range(args.warmup):
        run()
    sampler = ClockSampler(dev)
    sampler.start()
    ms, steps = timed_steps(run, stream, args.steps, flush, min_seconds=0.5, est_ms=2.5)
    clocks = sampler.stop()
    host_rays = torch.from_numpy(w["rays"]).pin_memory()
    host_hits = torch.empty(n * 16, dtype=torch.uint8, pin_memory=True)
    vt.check(vt.lib().vt_trace_rays_host(g.id, host_rays.data_ptr(), n, host_hits.data_ptr()))
    reps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(reps):
        vt.check(vt.lib().vt_trace_rays_host(g.id, host_rays.data_ptr(), n, host_hits.data_ptr()))
    e2e_s = (time.perf_counter() - t0) / reps
    out = {"metric": "Mrays/s (16M incoherent rays, 512^3 cave)", "value": n / ms / 1e3,
           "unit": "Mrays/s", "ms_per_step": ms, "steps": steps,
           "config": {"workload": w["name"], "grid": [512, 512, 512], "rays": n, "l2": L2_NOTE},
           "e2e": {"value": n / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n,
                   "d2h_bytes_per_step": 16 * n,
                   "path": "vt_trace_rays_host (C ABI), pinned host rays and records, host wall "
                           "clock"},
           "roofline": roofline(stats_bytes(st, n, io_per_ray=24), ms,
                                "vt::trace_rays_persistent_kernel"
                                if vt.get_tuning(vt.KERNEL_TRACE_RAYS)["persistent"]
                                else "vt::trace_rays_kernel<false>"),
           "gpu_launches": steps, "clocks": clocks}
    if not args.no_cpu_baseline:
        # a seeded sample of the rays, grown until the time budget is spent
        got = host_hits.numpy().view(vt.HIT_DTYPE)
        og = po.Grid(w["voxels"], w["palette"])
        order = np.random.default_rng(5).permutation(n)
        threads = po.hardware_threads()
        done, differ, chunk = 0, 0, 1 << 18
        t0 = time.perf_counter()
        while done < n and time.perf_counter() - t0 < args.cpu_seconds:
            idx = np.sort(order[done:done + chunk])
            want = po.trace_rays(og, w["rays"][idx].view(np.float32).reshape(-1, 6), threads)
            differ += int((got[idx].view(np.uint8).reshape(-1, 16) !=
                           want.view(np.uint8).reshape(-1, 16)).any(1).sum())
            done += len(idx)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": done / dt / 1e6, "unit": "Mrays/s", "cores": threads,
                               "kind": "port", "sample": "%d seeded rays of the 16M (%.1f s wall)"
                                                         % (done, dt),
                               "records_differing_from_gpu": differ}
    g.destroy()
    return out


def bench_multiview(args, stream, flush, dev, tuning):
    """64 views over 8 scenes in one persistent launch replayed from its CUDA graph."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import autotune, workloads
    from oracle import pyoracle as po
    scenes, views = workloads.multiview(n_views=args.views)
    grids = [vt.Grid.from_u8(sc["voxels"], sc["palette"]) for sc in scenes]
    bufs = []
    for v in views:
        c = v["camera"]
        bufs.append(torch.empty(c.width * c.height * v["spp"] * 16, dtype=torch.uint8, device="cuda"))

    def specs(outs):
        return [vt.make_view(grids[v["scene"]], v["camera"], b, v["spp"], v["seed"], v["view_id"],
                             v["light"]) for v, b in zip(views, outs)]

    holder = {"b": vt.Batch(specs(bufs))}

    def prepare():
        holder["b"].destroy()
        holder["b"] = vt.Batch(specs(bufs))

    run = lambda: holder["b"].run(stream)
    if not args.no_tune:
        best, table = autotune.autotune(vt.KERNEL_BATCH, run, stream, repeats=3, flush=flush,
                                        prepare=prepare)
        tuning["batch"] = {"chosen": autotune.key(vt.KERNEL_BATCH, best), "ms": table,
                           "installed": vt.get_tuning(vt.KERNEL_BATCH)}
    batch = holder["b"]
    st = batch.stats()
    for _ in range(args.warmup):
        run()
    sampler = ClockSampler(dev)
    sampler.start()
    ms, steps = timed_steps(run, stream, args.steps, flush, min_seconds=0.5, est_ms=20.0)
    clocks = sampler.stop()
    records = batch.primary_rays
    singles = [vt.Batch([sp]) for sp in specs(bufs)]
    ms_single = autotune.time_ms(lambda: [x.run(stream) for x in singles], stream,
                                 repeats=max(1, args.steps // 4), warmup=1, flush=flush)
    for x in singles:
        x.destroy()
    # end to end: the graph replay, then every view's records copied to page-locked host memory
    # on the same stream (copy engines; kernel stores over the host link measured slower)
    host = [torch.empty(b.numel(), dtype=torch.uint8, pin_memory=True) for b in bufs]

    def replay_and_copy():
        batch.run(stream)
        with torch.cuda.stream(stream):
            for h, b in zip(host, bufs):
                h.copy_(b, non_blocking=True)
        stream.synchronize()

    replay_and_copy()
    reps = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(reps):
        replay_and_copy()
    e2e_s = (time.perf_counter() - t0) / reps
    # the same views as four batches of about equal samples, each one's records copied out on a
    # second stream while the next batch renders (copies overlap the traversal)
    order_split, acc, parts = [], 0, [[]]
    total = sum(b.numel() for b in bufs)
    for i, b in enumerate(bufs):
        if acc >= (len(parts)) * total / 4 and len(parts) < 4:
            parts.append([])
        parts[-1].append(i)
        acc += b.numel()
    all_specs = specs(bufs)
    sub = [vt.Batch([all_specs[i] for i in part]) for part in parts if part]
    copy_stream = torch.cuda.Stream()
    events = [torch.cuda.Event() for _ in sub]

    def pipelined():
        for k, (bt, part) in enumerate(zip(sub, [p for p in parts if p])):
            bt.run(stream)
            events[k].record(stream)
            copy_stream.wait_event(events[k])
            with torch.cuda.stream(copy_stream):
                for i in part:
                    host[i].copy_(bufs[i], non_blocking=True)
        copy_stream.synchronize()
        stream.synchronize()

    pipelined()
    t0 = time.perf_counter()
    for _ in range(reps):
        pipelined()
    e2e_pipe_s = (time.perf_counter() - t0) / reps
    for bt in sub:
        bt.destroy()
    out = {"metric": "Mrays/s (%d views over 8 scenes, 1-4 spp, one graph replay)" % len(views),
           "value": st["rays"] / ms / 1e3, "unit": "Mrays/s", "ms_per_step": ms, "steps": steps,
           "config": {"workload": "multiview", "views": len(views), "primary_rays": records,
                      "shadow_rays": st["shadow_rays"], "l2": L2_NOTE},
           "per_view_launches": {"ms": ms_single, "value": st["rays"] / ms_single / 1e3},
           "e2e_pipelined": {"value": st["rays"] / e2e_pipe_s / 1e6, "unit": "Mrays/s",
                             "batches": len(sub), "d2h_bytes_per_step": 16 * records,
                             "path": "the views as %d vt_batch_run launches of about equal samples "
                                     "on one stream, each batch's records copied to page-locked "
                                     "host memory on a second stream while the next renders"
                                     % len(sub)},
           "e2e": {"value": st["rays"] / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 16 * records,
                   "path": "vt_batch_run (C ABI), then each view's records copied to page-locked "
                           "host memory on the launch stream, host wall clock; views and cameras "
                           "are fixed in the graph"},
           "roofline": roofline(stats_bytes(st, records), ms, "vt::batch_tile_kernel<false>"
                                if vt.get_tuning(vt.KERNEL_BATCH)["refill_min"] >= 32
                                else "vt::batch_kernel"),
           "gpu_launches": steps, "clocks": clocks}
    if not args.no_cpu_baseline:
        # the smallest views, every sample against the oracle
        order = sorted(range(len(views)), key=lambda i: views[i]["camera"].width *
                       views[i]["camera"].height * views[i]["spp"])
        ogrids = {}
        threads = po.hardware_threads()
        differ = samples = rays = 0
        checked = []
        t0 = time.perf_counter()
        for i in order:
            v = views[i]
            if v["scene"] not in ogrids:
                sc = scenes[v["scene"]]
                ogrids[v["scene"]] = po.Grid(sc["voxels"], sc["palette"])
            L = v["light"]
            want, wst = po.render_view(ogrids[v["scene"]], po.make_camera(v["camera"].as_dict()),
                                       po.make_light(list(L.dir), L.ambient, bool(L.shadows)),
                                       v["spp"], v["seed"], v["view_id"], threads, stats=True)
            got = bufs[i].cpu().numpy()
            differ += int((got.reshape(-1, 16) != want.view(np.uint8).reshape(-1, 16)).any(1).sum())
            samples += want.shape[0]
            rays += wst["rays"]
            checked.append(i)
            if time.perf_counter() - t0 >= args.cpu_seconds:
                break
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": threads,
                               "kind": "port", "sample": "the %d smallest views (%d samples), "
                                                         "%.1f s wall" % (len(checked), samples, dt),
                               "records_differing_from_gpu": differ}
    batch.destroy()
    for gr in grids:
        gr.destroy()
    return out


# ------------------------------------------------------------------ serving

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
        st0 = svc.stats()
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
    makespan = (last - first) / 1e9
    out = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "makespan_s": makespan,
           "msamples_per_s": samples / makespan / 1e6,
           "launches": st["launches"] - st0["launches"], "requests": len(reqs)}
    busy = (st["device_ns"] - st0["device_ns"]) / 1e9
    if svc_kwargs.get("plain"):
        # one launch at a time: the launches' summed device time is the time the GPU was busy
        out["device_busy_s"] = busy
        out["device_busy_fraction"] = busy / makespan
    else:
        out["launch_device_s_sum"] = busy  # concurrent launches overlap: not a busy time
    return out


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
    sat = {"batched": batched_sat, "plain": plain_sat,
           "throughput_ratio": batched_sat["msamples_per_s"] / plain_sat["msamples_per_s"],
           "p99_ratio": batched_sat["p99_ms"] / plain_sat["p99_ms"]}
    if plain_sat.get("device_busy_fraction"):
        # plain launches run one at a time, so their summed device time is the time the GPU was
        # busy; packing can only recover the rest (plus what fuller launches gain in lane use)
        sat["plain_busy_fraction"] = plain_sat["device_busy_fraction"]
        sat["throughput_bound_from_idle_time"] = 1.0 / plain_sat["device_busy_fraction"]
    return {"workload": "%d scenes 128^3-1024^3, %d requests, Poisson 2000/s, 320x240-1920x1080, "
                        "1-8 spp (rays = camera samples)" % (n_scenes, n_requests),
            "batched": batched, "plain": plain,
            "throughput_ratio": batched["msamples_per_s"] / plain["msamples_per_s"],
            "p99_ratio": batched["p99_ms"] / plain["p99_ms"],
            "p50_ratio": batched["p50_ms"] / plain["p50_ms"],
            "saturated": sat}


# ------------------------------------------------------------------ single configurations

def run_config(args):
    """Non-headline configurations: one JSON line each (measured parity cases)."""
    import torch
    import vtrace_gb300 as vt
    from vtrace_gb300 import workloads, autotune
    torch.cuda.set_device(0)
    vt.init(0)
    dev = torch.cuda.current_device()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    line = {"steps": args.steps, "warmup": args.warmup, "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (seeded generators, no dataset)", "impl": "ours"}
    tuning = {}
    if args.config in ("terrain256", "cave512", "multiview"):
        if args.config == "terrain256":
            r = bench_frame(args, workloads.terrain256(), stream, flush, dev)
        elif args.config == "cave512":
            r = bench_rays(args, stream, flush, dev, tuning)
        else:
            r = bench_multiview(args, stream, flush, dev, tuning)
        line.update(r)
        if tuning:
            line["tuning"] = tuning
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
        sampler = ClockSampler(dev)
        sampler.start()
        ms = autotune.time_ms(lambda: vt.path_trace(g, cam, p, d_out, None, stream), stream,
                              repeats=args.steps, warmup=args.warmup, flush=flush)
        clocks = sampler.stop()
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
                                               cam.width * cam.height) * args.steps,
                    clocks=clocks)
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
        sampler = ClockSampler(dev)
        sampler.start()
        t0 = time.perf_counter()
        for org, c in chunks[args.warmup:]:
            g.update(org, c)
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        clocks = sampler.stop()
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
                    gpu_launches=10 * args.steps, clocks=clocks)
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
        sampler = ClockSampler(dev)
        sampler.start()
        ms = autotune.time_ms(tick, lib_stream, repeats=args.steps, warmup=args.warmup, flush=flush)
        clocks = sampler.stop()
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
                    gpu_launches=3 * args.steps, clocks=clocks)
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
                    ms_per_step=r["batched"]["makespan_s"] * 1e3 / r["batched"]["requests"],
                    config={"workload": r["workload"]}, serve=r,
                    ms_per_step_note="makespan per request (the service has no fixed step)")
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config in ("cave512", "multiview", "serve", "pager_world", "pathtrace", "paging",
                       "terrain256"):
        return run_config(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
