"""ctypes/numpy front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by the tests, the smoke check and the benchmark's CPU-baseline leg; never by the product
path.  Wraps ``libvt_oracle.so`` (the C restatement) and, where it was built, the reference
shader compiled as C++ (``oracle/_ref``).
"""
import ctypes
import os

import numpy as np

from . import build as _build

HIT_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"), ("palette_index", "u1"),
                      ("face", "u1"), ("t", "<f4"), ("rgba", "<u4")])
assert HIT_DTYPE.itemsize == 16

FLAG_SHADOW_RAY = 0x08
FLAG_INVALID = 0x10
FLAG_SHADOWED = 0x20
FLAG_HIT = 0x80
SKY_RGBA = 0xFFF6E8C0


class _Grid(ctypes.Structure):
    _fields_ = [("voxels", ctypes.c_void_p), ("palette", ctypes.c_void_p),
                ("texels", ctypes.c_void_p), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("nz", ctypes.c_int32), ("brick_nonempty", ctypes.c_void_p)]


class Camera(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("forward", ctypes.c_float * 3),
                ("right", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class Light(ctypes.Structure):
    _fields_ = [("dir", ctypes.c_float * 3), ("ambient", ctypes.c_float),
                ("shadows", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "rays", "shadow_rays", "hits", "steps", "bricks_entered", "nonempty_bricks_entered",
        "voxels_tested", "ties")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Hit64(ctypes.Structure):
    _fields_ = [("hit", ctypes.c_int32), ("v", ctypes.c_int32 * 3), ("face", ctypes.c_int32),
                ("tie", ctypes.c_int32), ("t", ctypes.c_double)]


HIT64_DTYPE = np.dtype([("hit", "<i4"), ("v", "<i4", 3), ("face", "<i4"), ("tie", "<i4"),
                        ("t", "<f8")])
assert HIT64_DTYPE.itemsize == ctypes.sizeof(Hit64)

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        vp, u64, i32, u32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32
        L.vto_grid_prepare.argtypes = [ctypes.POINTER(_Grid)]
        L.vto_grid_release.argtypes = [ctypes.POINTER(_Grid)]
        L.vto_render.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(Camera),
                                 ctypes.POINTER(Light), vp, i32, ctypes.POINTER(Stats)]
        L.vto_render_rows.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(Camera),
                                      ctypes.POINTER(Light), u32, u32, vp, i32,
                                      ctypes.POINTER(Stats)]
        L.vto_render_view.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(Camera),
                                      ctypes.POINTER(Light), u32, u32, u32, vp, i32,
                                      ctypes.POINTER(Stats)]
        L.vto_trace_rays.argtypes = [ctypes.POINTER(_Grid), vp, u64, vp, i32,
                                     ctypes.POINTER(Stats)]
        L.vto_trace_rays_f64.argtypes = [ctypes.POINTER(_Grid), vp, u64, vp, i32]
        L.vto_trace_entry_points.argtypes = [ctypes.POINTER(_Grid), u64, vp, vp, vp]
        L.vto_philox4x32_10.argtypes = [vp, vp, vp]
        L.vto_jitter.argtypes = [u32, u32, u32, u32, u32, ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float)]
        L.vto_raygen.argtypes = [ctypes.POINTER(Camera), u32, u32, ctypes.c_float,
                                 ctypes.c_float, vp, vp]
        L.vto_hardware_threads.restype = ctypes.c_int
        L.vto_frame_rays.argtypes = [ctypes.POINTER(Camera), ctypes.POINTER(Light), vp, vp, vp]
        L.vto_frame_rays.restype = u64
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Grid:
    """A dense grid for the oracle: u8 palette indices + palette, or RGBA8 texels.

    ``voxels`` is indexed [z, y, x] (x fastest in memory)."""

    def __init__(self, voxels=None, palette=None, texels=None):
        if texels is not None:
            self.texels = np.ascontiguousarray(texels, dtype=np.uint32)
            nz, ny, nx = self.texels.shape
            self.voxels = None
            self.palette = None
        else:
            self.voxels = np.ascontiguousarray(voxels, dtype=np.uint8)
            self.palette = np.ascontiguousarray(palette, dtype=np.uint32)
            assert self.palette.shape == (256,)
            nz, ny, nx = self.voxels.shape
            self.texels = None
        self.nx, self.ny, self.nz = nx, ny, nz
        self._g = _Grid()
        self._g.voxels = self.voxels.ctypes.data if self.voxels is not None else None
        self._g.palette = self.palette.ctypes.data if self.palette is not None else None
        self._g.texels = self.texels.ctypes.data if self.texels is not None else None
        self._g.nx, self._g.ny, self._g.nz = nx, ny, nz
        self._g.brick_nonempty = None
        if lib().vto_grid_prepare(ctypes.byref(self._g)) != 0:
            raise MemoryError("oracle grid preparation failed")

    def __del__(self):
        if getattr(self, "_g", None) is not None and _lib is not None:
            _lib.vto_grid_release(ctypes.byref(self._g))
            self._g = None

    def rgba_bytes(self):
        """RGBA8 texels as [z, y, x, 4] bytes (the reference's add_texture layout)."""
        if self.texels is not None:
            t = self.texels
        else:
            t = self.palette[self.voxels]
        return np.ascontiguousarray(t).view(np.uint8).reshape(self.nz, self.ny, self.nx, 4)


def make_camera(cam_fields):
    c = Camera()
    for k in ("origin", "forward", "right", "up"):
        getattr(c, k)[:] = [float(v) for v in cam_fields[k]]
    c.width, c.height = int(cam_fields["width"]), int(cam_fields["height"])
    return c


def make_light(dir3, ambient=0.25, shadows=True):
    L = Light()
    L.dir[:] = [float(v) for v in dir3]
    L.ambient = float(ambient)
    L.shadows = 1 if shadows else 0
    return L


def trace_rays(grid, rays, threads=0, stats=False):
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    hits = np.zeros(rays.shape[0], dtype=HIT_DTYPE)
    st = Stats()
    lib().vto_trace_rays(ctypes.byref(grid._g), _ptr(rays), rays.shape[0], _ptr(hits), threads,
                         ctypes.byref(st) if stats else None)
    return (hits, st.as_dict()) if stats else hits


def trace_rays_f64(grid, rays, threads=0):
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    hits = np.zeros(rays.shape[0], dtype=HIT64_DTYPE)
    lib().vto_trace_rays_f64(ctypes.byref(grid._g), _ptr(rays), rays.shape[0], _ptr(hits),
                             threads)
    return hits


def render(grid, camera, light=None, threads=0, stats=False, rows=None):
    """Image of camera.height x camera.width records (or only rows [r0, r1))."""
    r0, r1 = (0, camera.height) if rows is None else rows
    hits = np.zeros((r1 - r0) * camera.width, dtype=HIT_DTYPE)
    st = Stats()
    lib().vto_render_rows(ctypes.byref(grid._g), ctypes.byref(camera),
                          ctypes.byref(light) if light is not None else None, r0, r1,
                          _ptr(hits), threads, ctypes.byref(st) if stats else None)
    hits = hits.reshape(r1 - r0, camera.width)
    return (hits, st.as_dict()) if stats else hits


def render_view(grid, camera, light, spp, seed, view, threads=0, stats=False):
    hits = np.zeros(camera.height * camera.width * spp, dtype=HIT_DTYPE)
    st = Stats()
    lib().vto_render_view(ctypes.byref(grid._g), ctypes.byref(camera),
                          ctypes.byref(light) if light is not None else None, spp, seed, view,
                          _ptr(hits), threads, ctypes.byref(st) if stats else None)
    return (hits, st.as_dict()) if stats else hits


def trace_entry_points(grid, mp, s):
    mp = np.ascontiguousarray(mp, dtype=np.float32).reshape(-1, 3)
    s = np.ascontiguousarray(s, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((mp.shape[0], 5), dtype=np.int32)
    lib().vto_trace_entry_points(ctypes.byref(grid._g), mp.shape[0], _ptr(mp), _ptr(s), _ptr(out))
    return out


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().vto_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


def frame_rays(camera, light, hits):
    """The camera ray of every pixel and the shadow ray of every record of `hits` (the frame's
    records, [height, width] or flat) that traced one, as [n, 6] float32 ray buffers."""
    hits = np.ascontiguousarray(hits).reshape(-1)
    npx = camera.width * camera.height
    assert hits.shape[0] == npx and hits.dtype.itemsize == 16
    cam_rays = np.zeros((npx, 6), np.float32)
    sh_rays = np.zeros((npx, 6), np.float32)
    ns = lib().vto_frame_rays(ctypes.byref(camera), ctypes.byref(light) if light is not None else None,
                              _ptr(hits), _ptr(cam_rays), _ptr(sh_rays))
    return cam_rays, sh_rays[:ns].copy()


def raygen(camera, px, py, jx=0.5, jy=0.5):
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    lib().vto_raygen(ctypes.byref(camera), px, py, jx, jy, _ptr(o), _ptr(d))
    return o, d


def hardware_threads():
    return int(lib().vto_hardware_threads())


# ------------------------------------------------------------------ reference shader as C++

_ref_libs = {}


def ref_available():
    return os.path.exists(_build.ref_so("select")) or os.path.exists(_build.SHADER)


def ref_lib(variant="select"):
    if variant not in _ref_libs:
        built = _build.build_ref()
        path = _build.ref_so(variant)
        if path not in built:
            return None
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.vtref_trace.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                  vp, vp, vp, vp]
        _ref_libs[variant] = L
    return _ref_libs[variant]


def ref_trace(grid, mp, s, variant="select", colours=False):
    """Runs shaders/trace.frag (compiled as C++) for model-space entry points mp and direction
    vectors s; returns int32 [n, 5] = {hit, x, y, z, fetches} (and RGBA float colours)."""
    L = ref_lib(variant)
    if L is None:
        raise RuntimeError("reference shader build unavailable")
    rgba = np.ascontiguousarray(grid.rgba_bytes())
    mp = np.ascontiguousarray(mp, dtype=np.float32).reshape(-1, 3)
    s = np.ascontiguousarray(s, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((mp.shape[0], 5), dtype=np.int32)
    col = np.zeros((mp.shape[0], 4), dtype=np.float32)
    L.vtref_trace(_ptr(rgba), grid.nx, grid.ny, grid.nz, mp.shape[0], _ptr(mp), _ptr(s),
                  _ptr(out), _ptr(col))
    return (out, col) if colours else out


def compat_render(grids, instances, P, C, width, height, threads=0):
    """The reference's multi-instance frame (see vto_compat_render): RGBA8 [height, width, 4]."""
    L = lib()
    arr = (_Grid * max(1, len(grids)))()
    for i, g in enumerate(grids):
        arr[i] = g._g
    inst = np.ascontiguousarray(instances, dtype=np.float32).reshape(-1, 16)
    P = np.ascontiguousarray(P, dtype=np.float32).reshape(16)
    C = np.ascontiguousarray(C, dtype=np.float32).reshape(16)
    out = np.zeros((height, width, 4), np.uint8)
    L.vto_compat_render.argtypes = [ctypes.POINTER(_Grid), ctypes.c_uint32, ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_int]
    rc = L.vto_compat_render(arr, len(grids), _ptr(inst), inst.shape[0], _ptr(P), _ptr(C),
                             width, height, _ptr(out), threads)
    if rc != 0:
        raise ValueError("singular projection or camera matrix")
    return out


class PathParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("out_format", ctypes.c_uint32),
                ("sky", ctypes.c_float * 3), ("sun_dir", ctypes.c_float * 3),
                ("sun", ctypes.c_float * 3)]


def make_path_params(spp, max_bounces, seed, sky, sun_dir, sun):
    p = PathParams()
    p.spp, p.max_bounces, p.seed, p.out_format = spp, max_bounces, seed, 0
    p.sky[:], p.sun_dir[:], p.sun[:] = list(sky), list(sun_dir), list(sun)
    return p


def path_trace(grid, camera, params, threads=0, rows=None):
    """The path-tracing estimator restated: (float32 [rows, width, 4], rays traced) for the rows
    (row0, row1) of the image (all by default)."""
    L = lib()
    r0, r1 = rows if rows is not None else (0, camera.height)
    out = np.zeros((r1 - r0, camera.width, 4), np.float32)
    rays = ctypes.c_uint64(0)
    L.vto_path_trace.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(Camera),
                                 ctypes.POINTER(PathParams), ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    L.vto_path_trace.restype = None
    L.vto_path_trace(ctypes.byref(grid._g), ctypes.byref(camera), ctypes.byref(params), r0, r1,
                     _ptr(out), threads, ctypes.byref(rays))
    return out, rays.value


def path_rgba8(img):
    """VT_PATH_OUT_RGBA8 of a float image: clamp to [0, 1], x 255 + 0.5 truncated, alpha 255."""
    c = np.clip(img[..., :3], np.float32(0), np.float32(1)).astype(np.float32)
    q = (c * np.float32(255.0) + np.float32(0.5)).astype(np.uint32)
    out = np.full(img.shape[:2] + (4,), 255, np.uint8)
    out[..., :3] = q.astype(np.uint8)
    return out
