"""The C ABI from a C host: tests/c_host/replay.c drives the seven reference entry points in
src/render.rs's order.  On CPU the program must compile and link against include/vtrace.h and
libvtrace.so; on the GPU its frame must equal the oracle's restatement of the reference frame."""
import os
import subprocess

import numpy as np
import pytest

import vtrace_gb300 as vt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_host", "replay.c")
DIMS = [(16, 16, 16), (12, 20, 10)]


def build(tmp_path):
    lib = vt.library_path()
    vt.lib()  # builds it if needed
    exe = str(tmp_path / "replay")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           SRC, "-o", exe, "-L", os.path.dirname(lib), "-l:" + os.path.basename(lib),
           "-Wl,-rpath," + os.path.dirname(lib), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return exe


def test_c_host_compiles_and_links(tmp_path):
    assert os.path.exists(build(tmp_path))


@pytest.mark.gpu
def test_c_host_frame_matches_oracle(tmp_path):
    from oracle import pyoracle as po
    exe = build(tmp_path)
    out = str(tmp_path / "frame.bin")
    r = subprocess.run([exe, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout
    raw = open(out, "rb").read()
    w, h, n = np.frombuffer(raw, np.int32, 3)
    off = 12
    P = np.frombuffer(raw, np.float32, 16, off)
    C = np.frombuffer(raw, np.float32, 16, off + 64)
    inst = np.frombuffer(raw, np.float32, 16 * n, off + 128).reshape(n, 16)
    off += 128 + 64 * n
    grids = []
    for nx, ny, nz in DIMS:
        t = np.frombuffer(raw, np.uint32, nx * ny * nz, off).reshape(nz, ny, nx)
        off += 4 * nx * ny * nz
        grids.append(po.Grid(texels=t))
    fb = np.frombuffer(raw, np.uint8, w * h * 4, off).reshape(h, w, 4)
    want = po.compat_render(grids, inst, P, C, int(w), int(h))
    assert (fb != want).any(-1).sum() == 0
    sky = np.array([0xC0, 0xE8, 0xF6, 0xFF], np.uint8)
    assert (fb != sky).any(-1).mean() > 0.02
