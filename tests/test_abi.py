"""CPU tests of the C ABI library: it builds and loads without a GPU, exports every symbol the
public header declares, and its host-side logic (generators, camera, argument checks) behaves."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import vtrace_gb300 as vt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?[\s\*])([A-Za-z_]\w*)\s*\([^;{]*\)\s*;",
                             text, flags=re.M):
            if not m.group(0).lstrip().startswith(("typedef", "#")):
                names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("entry", "render_tick", "get_input_data_pointer", "add_texture",
                "start_update_instances", "end_update_instances", "cleanup"):
        assert ref in names
    assert "vt_render" in names and "vt_trace_rays" in names


def test_library_exports_every_declared_symbol():
    path = vt.lib() and vt.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], stdout=subprocess.PIPE,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    bound = {name for name, _, _ in vt.SIGNATURES}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_struct_layouts_match_header():
    assert vt.HIT_DTYPE.itemsize == 16 and vt.RAY_DTYPE.itemsize == 24
    assert ctypes.sizeof(vt.Camera) == 56
    assert ctypes.sizeof(vt.Light) == 20
    assert ctypes.sizeof(vt.TraceStats) == 64
    assert ctypes.sizeof(vt.UserInput) == 40


def test_argument_errors_need_no_gpu():
    L = vt.lib()
    assert L.vt_grid_create_u8(None, None, 1, 1, 1) == -1
    v = np.zeros(8, np.uint8)
    p = np.zeros(256, np.uint32)
    assert L.vt_grid_create_u8(v.ctypes.data, p.ctypes.data, 0, 1, 1) == -1
    assert L.vt_grid_create_u8(v.ctypes.data, p.ctypes.data, 70000, 1, 1) == -1
    assert "65535" in vt.last_error()
    assert L.vt_grid_destroy(12345) == -4
    assert L.vt_gen_cave(8, 8, 8, 1, 1.5, v.ctypes.data) == -1
    with pytest.raises(vt.VtError):
        vt.check(L.vt_grid_destroy(-1))


def test_generators_are_deterministic_and_hit_their_occupancy():
    a = vt.gen_terrain(96, 7)
    b = vt.gen_terrain(96, 7)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, vt.gen_terrain(96, 8))
    assert 0.25 < (a > 0).mean() < 0.35
    c = vt.gen_cave(96, 3)
    assert 0.40 < (c > 0).mean() < 0.50
    s = vt.gen_shapes(256, 2, count=600, rmin=2, rmax=40)
    assert np.array_equal(s, vt.gen_shapes(256, 2, count=600, rmin=2, rmax=40))
    assert 0.0 < (s > 0).mean() < 0.2
    pal = vt.gen_palette(1)
    assert pal[0] == 0 and ((pal[1:] >> 24) >= 1).all()


def test_generator_terrain_is_a_heightfield():
    a = vt.gen_terrain((40, 32, 24), 11)
    filled = a > 0
    # every column is solid from y = 0 up to its height
    h = filled.sum(axis=1)  # [z, x]
    ys = np.arange(32)[None, :, None]
    assert np.array_equal(filled, ys < h[:, None, :])


def test_uniform_rays():
    r = vt.gen_rays_uniform(64, 5, 20000)
    assert (r[:, :3] >= 0).all() and (r[:, :3] < 64).all()
    n = np.linalg.norm(r[:, 3:].astype(np.float64), axis=1)
    assert np.allclose(n, 1.0, atol=1e-6)
    # roughly isotropic
    assert np.abs(r[:, 3:].mean(0)).max() < 0.03
    assert np.array_equal(r, vt.gen_rays_uniform(64, 5, 20000))


def test_camera_look_at():
    c = vt.camera_look_at((0, 0, 10), (0, 0, 0), (0, 1, 0), 60.0, 200, 100)
    f = np.array(c.forward)
    assert np.allclose(f, [0, 0, -1])
    th = np.tan(np.radians(30))
    assert np.allclose(c.up, [0, th, 0], atol=1e-7)
    assert np.allclose(c.right, [2 * th, 0, 0], atol=1e-7)
    with pytest.raises(vt.VtError):
        vt.camera_look_at((0, 0, 0), (0, 0, 0))


STRUCTS = [("vt_camera", "Camera"), ("vt_light", "Light"), ("vt_grid_info", "GridInfo"),
           ("vt_trace_stats", "TraceStats"), ("vt_tuning", "Tuning"), ("vt_view", "View"),
           ("vt_serve_config", "ServeConfig"), ("vt_serve_request", "ServeRequest"),
           ("vt_serve_timing", "ServeTiming"), ("vt_serve_stats", "ServeStats"),
           ("vt_path_params", "PathParams"), ("vt_footprint", "Footprint"),
           ("vt_vox_info", "VoxInfo"), ("vt_vox_model", "VoxModel"),
           ("render_tick_info", "RenderTickInfo"), ("user_input", "UserInput")]


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler gives the header's
    struct (a mirror that is too small lets the library write past it)."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "vtrace.h"', "int main(void) {"]
    for cname, pyname in STRUCTS:
        cls = getattr(vt, pyname)
        lines.append('printf("%s @sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                           str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, pyname in STRUCTS:
        cls = getattr(vt, pyname)
        assert ctypes.sizeof(cls) == got[(cname, "@sizeof")], cname
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == got[(cname, fname)], (cname, fname)
