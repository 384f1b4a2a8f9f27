"""The benchmark's reference arm runs the oracle alone: its process never maps libvtrace.so (the
seeded workload comes from a child process as arrays), it renders the whole frame each step, and
its line carries the same config keys as the GPU arm's.  Runs on the CPU, on the small terrain
frame."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHECK = """
import json, sys
sys.path.insert(0, %r)
sys.argv = ["bench.py", "--impl", "reference", "--config", "terrain256", "--steps", "2",
            "--warmup", "1"]
import bench
bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"libvtrace_mapped": "libvtrace" in maps, "oracle_mapped": "libvt_oracle" in maps,
                  "package_imported": "vtrace_gb300" in sys.modules}))
"""


def test_reference_arm_loads_the_oracle_only():
    out = subprocess.run([sys.executable, "-c", CHECK % ROOT], check=True, capture_output=True,
                         text=True, timeout=600).stdout.strip().splitlines()
    line = json.loads(out[-2])
    maps = json.loads(out[-1])
    assert maps == {"libvtrace_mapped": False, "oracle_mapped": True, "package_imported": False}
    assert line["impl"] == "reference"
    assert line["steps"] == 2 and line["warmup"] == 1
    cfg = line["config"]
    assert set(cfg) == {"workload", "grid", "image", "spp", "shadow_rays", "rays_per_frame", "l2",
                        "parallelism"}
    assert cfg["workload"] == "terrain256_640x480" and cfg["image"] == [640, 480]
    assert cfg["rays_per_frame"] >= 640 * 480  # the whole frame, shadow rays included
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port"
