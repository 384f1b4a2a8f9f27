"""vtrace_gb300 — GB300-native voxel ray traversal behind vtrace's C ABI.

Python host-side mirror of ``include/vtrace.h``: thin ctypes bindings over ``libvtrace.so``
(CUDA kernels for sm_103a).  There is no CPU fallback: every call goes to the CUDA library, and
loading fails loudly when the library is missing or cannot be built.

Device buffers are passed as raw pointers (ints) or objects with ``data_ptr()`` (e.g. torch CUDA
tensors); streams as raw ``cudaStream_t`` values (ints, e.g. ``torch.cuda.current_stream()
.cuda_stream``) or None for the library's own stream.
"""
import ctypes
import os

import numpy as np

from . import build as _build

HIT_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"), ("palette_index", "u1"),
                      ("face", "u1"), ("t", "<f4"), ("rgba", "<u4")])
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3)])

VT_OK = 0
ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ENOTFOUND", -5: "ETIMEDOUT",
          -6: "EBUSY", -7: "ECANCELED", -8: "ENOTREADY", -9: "ELIMIT"}
FACE_MASK = 0x07
FLAG_SHADOW_RAY = 0x08
FLAG_INVALID = 0x10
FLAG_SHADOWED = 0x20
FLAG_HIT = 0x80
SKY_RGBA = 0xFFF6E8C0
PAYLOAD_U8 = 1
PAYLOAD_RGBA8 = 2
ORDER_X_FASTEST = 0
ORDER_Z_FASTEST = 1


class VtError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "ERROR"), code, message))
        self.code = code


class Camera(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("forward", ctypes.c_float * 3),
                ("right", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]

    def as_dict(self):
        return {"origin": list(self.origin), "forward": list(self.forward),
                "right": list(self.right), "up": list(self.up), "width": self.width,
                "height": self.height}


class Light(ctypes.Structure):
    _fields_ = [("dir", ctypes.c_float * 3), ("ambient", ctypes.c_float),
                ("shadows", ctypes.c_uint32)]


class GridInfo(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32),
                ("bricks_x", ctypes.c_uint32), ("bricks_y", ctypes.c_uint32),
                ("bricks_z", ctypes.c_uint32), ("bricks_total", ctypes.c_uint64),
                ("bricks_nonempty", ctypes.c_uint64), ("voxels_occupied", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("payload_format", ctypes.c_uint32),
                ("slots", ctypes.c_uint32)]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class TraceStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "rays", "shadow_rays", "hits", "steps", "bricks_entered", "nonempty_bricks_entered",
        "voxels_tested", "ties")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [("refill_min", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_int32),
                ("persistent", ctypes.c_uint32), ("wavefront", ctypes.c_uint32),
                ("tile_shape", ctypes.c_uint32), ("block_warps", ctypes.c_uint32)]


TILE_8X4, TILE_4X8, TILE_16X2, TILE_32X1 = 0, 1, 2, 3
TILE_NAMES = {TILE_8X4: "8x4", TILE_4X8: "4x8", TILE_16X2: "16x2", TILE_32X1: "32x1"}


KERNEL_RENDER, KERNEL_TRACE_RAYS, KERNEL_BATCH, KERNEL_PATH = 1, 2, 3, 4


class View(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int32), ("spp", ctypes.c_uint32), ("seed", ctypes.c_uint32),
                ("view_id", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("camera", Camera),
                ("light", Light), ("d_out", ctypes.c_void_p)]


VIEW_LIGHT = 1


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_views_per_launch", ctypes.c_uint32),
                ("max_samples_per_launch", ctypes.c_uint64), ("poll_interval_us", ctypes.c_uint32),
                ("refill_min", ctypes.c_uint32), ("max_samples_per_piece", ctypes.c_uint64)]


class ServeRequest(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int32), ("spp", ctypes.c_uint32), ("seed", ctypes.c_uint32),
                ("view_id", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("camera", Camera),
                ("light", Light), ("host_rgba", ctypes.c_void_p)]


class ServeTiming(ctypes.Structure):
    _fields_ = [("submit_ns", ctypes.c_int64), ("launch_ns", ctypes.c_int64),
                ("done_ns", ctypes.c_int64), ("samples", ctypes.c_uint64)]


class ServeStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "submitted", "completed", "launches", "views_launched", "samples", "scene_loads",
        "evictions", "resident_bytes", "pending", "device_ns")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class PathParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("out_format", ctypes.c_uint32),
                ("sky", ctypes.c_float * 3), ("sun_dir", ctypes.c_float * 3),
                ("sun", ctypes.c_float * 3)]


PATH_OUT_F32X4 = 0
PATH_OUT_RGBA8 = 1


def make_path_params(spp=4, max_bounces=3, seed=0, out_format=PATH_OUT_F32X4,
                     sky=(0.6, 0.75, 1.0), sun_dir=(0.3, 0.8, 0.52), sun=(2.5, 2.3, 2.0)):
    p = PathParams()
    p.spp, p.max_bounces, p.seed, p.out_format = spp, max_bounces, seed, out_format
    p.sky[:] = [float(x) for x in sky]
    n = float(np.sqrt(np.sum(np.square(np.asarray(sun_dir, np.float64)))))
    p.sun_dir[:] = [float(np.float32(x / n)) for x in sun_dir]
    p.sun[:] = [float(x) for x in sun]
    return p


class Footprint(ctypes.Structure):
    _fields_ = [("bricks", ctypes.c_uint64), ("nonempty_bricks", ctypes.c_uint64),
                ("hit_bricks", ctypes.c_uint64), ("reserved", ctypes.c_uint64)]


PHASES = ("setup", "loop", "walk", "cross_box", "cross_chains", "cross_finish", "tail")


class PhaseProfile(ctypes.Structure):
    _fields_ = [("warp_cycles", (ctypes.c_uint64 * len(PHASES)) * 2),
                ("passes", (ctypes.c_uint64 * 2) * 2), ("warps", ctypes.c_uint64)]


class VoxInfo(ctypes.Structure):
    _fields_ = [("version", ctypes.c_uint32), ("models", ctypes.c_uint32),
                ("has_palette", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class VoxModel(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32 * 3), ("voxels", ctypes.c_uint32)]


class RenderTickInfo(ctypes.Structure):
    _fields_ = [("perspective", ctypes.c_void_p), ("camera", ctypes.c_void_p)]


class UserInput(ctypes.Structure):
    _fields_ = [("keys", ctypes.c_uint8 * 6), ("mouse_x", ctypes.c_double),
                ("mouse_y", ctypes.c_double), ("last_mouse_x", ctypes.c_double),
                ("last_mouse_y", ctypes.c_double)]


_lib = None

# (name, restype, argtypes) of every symbol include/vtrace.h declares
_vp, _i32, _u32, _u64, _f32 = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_float)
SIGNATURES = [
    ("vt_init", _i32, [_i32]),
    ("vt_shutdown", None, []),
    ("vt_last_error", ctypes.c_char_p, []),
    ("vt_version", _u32, []),
    ("vt_device_info", _i32, [_vp, _vp, _vp, _vp]),
    ("vt_get_stream", _vp, []),
    ("vt_get_tuning", _i32, [_i32, ctypes.POINTER(Tuning)]),
    ("vt_set_tuning", _i32, [_i32, ctypes.POINTER(Tuning)]),
    ("vt_grid_create_u8", _i32, [_vp, _vp, _u32, _u32, _u32]),
    ("vt_grid_create_u8_device", _i32, [_vp, _vp, _u32, _u32, _u32, _vp]),
    ("vt_grid_create_rgba8", _i32, [_vp, _u32, _u32, _u32]),
    ("vt_grid_create", _i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32]),
    ("vt_grid_destroy", _i32, [_i32]),
    ("vt_grid_update", _i32, [_i32, _vp, _u32, _u32, _u32, _u32, _u32, _u32, _u32]),
    ("vt_grid_build_u8_noalloc", _i32, [_vp, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp]),
    ("vt_grid_get_info", _i32, [_i32, ctypes.POINTER(GridInfo)]),
    ("vt_grid_download_bricks", _i32, [_i32, _vp, _vp]),
    ("vt_grid_download_octants", _i32, [_i32, _vp]),
    ("vt_grid_download_long", _i32, [_i32, _vp]),
    ("vt_grid_download_payload", _i32, [_i32, _vp, _u64]),
    ("vt_trace_rays", _i32, [_i32, _vp, _u64, _vp, _vp]),
    ("vt_trace_rays_host", _i32, [_i32, _vp, _u64, _vp]),
    ("vt_render", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(Light), _vp, _vp]),
    ("vt_render_host", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(Light), _vp]),
    ("vt_render_stats", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(Light), _vp,
                               ctypes.POINTER(TraceStats)]),
    ("vt_render_footprint", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(Light), _vp,
                                   ctypes.POINTER(Footprint)]),
    ("vt_render_phases", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(Light), _vp,
                                ctypes.POINTER(PhaseProfile)]),
    ("vt_trace_rays_stats", _i32, [_i32, _vp, _u64, _vp, ctypes.POINTER(TraceStats)]),
    ("vt_path_trace", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(PathParams), _vp, _vp,
                             _vp]),
    ("vt_path_trace_host", _i32, [_i32, ctypes.POINTER(Camera), ctypes.POINTER(PathParams), _vp,
                                  ctypes.POINTER(ctypes.c_uint64)]),
    ("vt_batch_create", _i32, [ctypes.POINTER(View), _u32, ctypes.POINTER(ctypes.c_int32)]),
    ("vt_batch_run", _i32, [_i32, _vp]),
    ("vt_batch_run_direct", _i32, [_i32, _vp]),
    ("vt_batch_info", _i32, [_i32, _vp, _vp]),
    ("vt_batch_stats", _i32, [_i32, ctypes.POINTER(TraceStats)]),
    ("vt_batch_destroy", _i32, [_i32]),
    ("vt_serve_default_config", _i32, [ctypes.POINTER(ServeConfig)]),
    ("vt_serve_start", _i32, [ctypes.POINTER(ServeConfig), ctypes.POINTER(ctypes.c_int32)]),
    ("vt_serve_add_scene", _i32, [_i32, _vp, _vp, _u32, _u32, _u32, ctypes.POINTER(ctypes.c_int32)]),
    ("vt_serve_update_scene", _i32, [_i32, _i32, _u32, _u32, _u32, _u32, _u32, _u32]),
    ("vt_serve_submit", _i32, [_i32, ctypes.POINTER(ServeRequest), ctypes.POINTER(ctypes.c_uint64)]),
    ("vt_serve_poll", _i32, [_i32, _u64, _u32, ctypes.POINTER(ServeTiming)]),
    ("vt_serve_get_stats", _i32, [_i32, ctypes.POINTER(ServeStats)]),
    ("vt_serve_stop", _i32, [_i32]),
    ("vt_camera_look_at", _i32, [_vp, _vp, _vp, _f32, _u32, _u32, ctypes.POINTER(Camera)]),
    ("vt_vox_inspect", _i32, [_vp, _u64, ctypes.POINTER(VoxInfo)]),
    ("vt_vox_model_info", _i32, [_vp, _u64, _u32, ctypes.POINTER(VoxModel)]),
    ("vt_vox_model_chunk", _i32, [_vp, _u64, _u32, _vp, _u64]),
    ("vt_gen_palette", _i32, [_u32, _vp]),
    ("vt_gen_terrain", _i32, [_u32, _u32, _u32, _u32, _u32, _f32, _vp]),
    ("vt_gen_shapes", _i32, [_u32, _u32, _u32, _u32, _u32, _f32, _f32, _vp]),
    ("vt_gen_cave", _i32, [_u32, _u32, _u32, _u32, _f32, _vp]),
    ("vt_gen_rays_uniform", _i32, [_u32, _u32, _u32, _u32, _u64, _vp]),
    ("entry", _u64, []),
    ("render_tick", _i32, [_vp, _vp, ctypes.POINTER(RenderTickInfo)]),
    ("get_input_data_pointer", ctypes.POINTER(UserInput), []),
    ("add_texture", _i32, [_vp, _u32, _u32, _u32]),
    ("start_update_instances", ctypes.POINTER(ctypes.c_float), [_u32]),
    ("end_update_instances", _i32, [_u32]),
    ("cleanup", None, []),
    ("vt_framebuffer_download", _i32, [_vp, _u64]),
]


def library_path():
    return _build.LIB


def lib():
    """The loaded libvtrace.so, built in-tree first if needed.  Raises if it cannot be had."""
    global _lib
    if _lib is None:
        path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError("libvtrace.so was not built")
        L = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    return lib().vt_last_error().decode()


def check(rc):
    if rc < 0:
        raise VtError(rc, last_error())
    return rc


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError("expected a pointer, an ndarray or a tensor, got %r" % type(x))


CUDA_STREAM_LEGACY = 0x1


def _stream(s):
    """None -> the library's own stream; 0 (the legacy default stream's handle, e.g. torch's
    default stream) -> cudaStreamLegacy; anything else is passed through."""
    if s is None:
        return None
    h = s if isinstance(s, int) else s.cuda_stream
    return h if h != 0 else CUDA_STREAM_LEGACY


def init(device=0):
    check(lib().vt_init(device))


def device_info():
    d, sm = ctypes.c_int32(), ctypes.c_int32()
    f, t = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().vt_device_info(ctypes.byref(d), ctypes.byref(sm), ctypes.byref(f),
                               ctypes.byref(t)))
    return {"device": d.value, "sm_count": sm.value, "free_bytes": f.value,
            "total_bytes": t.value}


def get_tuning(kernel):
    t = Tuning()
    check(lib().vt_get_tuning(kernel, ctypes.byref(t)))
    return {"refill_min": t.refill_min, "blocks_per_sm": t.blocks_per_sm,
            "persistent": t.persistent, "wavefront": t.wavefront, "tile_shape": t.tile_shape,
            "block_warps": t.block_warps}


def set_tuning(kernel, refill_min=16, blocks_per_sm=0, persistent=True, wavefront=False,
               tile_shape=TILE_8X4, block_warps=4):
    t = Tuning(refill_min, blocks_per_sm, 1 if persistent else 0, 1 if wavefront else 0,
               tile_shape, block_warps)
    check(lib().vt_set_tuning(kernel, ctypes.byref(t)))


# ---------------------------------------------------------------- content

def gen_palette(seed):
    pal = np.zeros(256, np.uint32)
    check(lib().vt_gen_palette(seed, pal.ctypes.data))
    return pal


def gen_terrain(n, seed, octaves=5, occupancy=0.3):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    v = np.empty((nz, ny, nx), np.uint8)
    check(lib().vt_gen_terrain(nx, ny, nz, seed, octaves, occupancy, v.ctypes.data))
    return v


def gen_shapes(n, seed, count=10000, rmin=2.0, rmax=40.0):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    v = np.empty((nz, ny, nx), np.uint8)
    check(lib().vt_gen_shapes(nx, ny, nz, seed, count, rmin, rmax, v.ctypes.data))
    return v


def gen_cave(n, seed, occupancy=0.45):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    v = np.empty((nz, ny, nx), np.uint8)
    check(lib().vt_gen_cave(nx, ny, nz, seed, occupancy, v.ctypes.data))
    return v


def gen_rays_uniform(n_grid, seed, count):
    nx, ny, nz = (n_grid, n_grid, n_grid) if isinstance(n_grid, int) else n_grid
    r = np.empty((count, 6), np.float32)
    check(lib().vt_gen_rays_uniform(nx, ny, nz, seed, count, r.ctypes.data))
    return r


def camera_look_at(eye, target, up=(0.0, 1.0, 0.0), vfov_degrees=60.0, width=640,
                   height=480):
    c = Camera()
    e = (ctypes.c_float * 3)(*eye)
    t = (ctypes.c_float * 3)(*target)
    u = (ctypes.c_float * 3)(*up)
    check(lib().vt_camera_look_at(e, t, u, vfov_degrees, width, height, ctypes.byref(c)))
    return c


def make_light(direction, ambient=0.25, shadows=True):
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    L = Light()
    L.dir[:] = [float(np.float32(x)) for x in d]
    L.ambient = ambient
    L.shadows = 1 if shadows else 0
    return L


# ---------------------------------------------------------------- MagicaVoxel models

def _vox_bytes(src):
    if isinstance(src, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(src), np.uint8)
    with open(src, "rb") as f:
        return np.frombuffer(f.read(), np.uint8)


def vox_inspect(src):
    """src: a path or the bytes of a .vox file -> {"version", "models", "has_palette"}."""
    b = _vox_bytes(src)
    info = VoxInfo()
    check(lib().vt_vox_inspect(b.ctypes.data, b.size, ctypes.byref(info)))
    return {"version": info.version, "models": info.models, "has_palette": bool(info.has_palette)}


def vox_model_chunk(src, model=0):
    """The RGBA8 texture vtrace builds from a .vox model (src/voxel/magica_voxel.rs:18-44), as a
    uint8 array indexed [x, y, z, channel] (the chunk's z-fastest order), shape
    (size.x, size.y, size.z, 4)."""
    b = _vox_bytes(src)
    m = VoxModel()
    check(lib().vt_vox_model_info(b.ctypes.data, b.size, model, ctypes.byref(m)))
    sx, sy, sz = m.size
    out = np.zeros((sx, sy, sz, 4), np.uint8)
    check(lib().vt_vox_model_chunk(b.ctypes.data, b.size, model, out.ctypes.data, out.nbytes))
    return out


# ---------------------------------------------------------------- grids

class Grid:
    """A brick grid resident on the device (ids are the library's grid ids)."""

    def __init__(self, gid):
        self.id = gid

    @classmethod
    def from_u8(cls, voxels, palette):
        voxels = np.ascontiguousarray(voxels, np.uint8)
        palette = np.ascontiguousarray(palette, np.uint32)
        if palette.shape != (256,):
            raise ValueError("palette must hold 256 RGBA8 entries")
        nz, ny, nx = voxels.shape
        return cls(check(lib().vt_grid_create_u8(voxels.ctypes.data, palette.ctypes.data,
                                                 nx, ny, nz)))

    @classmethod
    def from_u8_device(cls, d_voxels, dims, palette, stream=None):
        nx, ny, nz = dims
        palette = np.ascontiguousarray(palette, np.uint32)
        return cls(check(lib().vt_grid_create_u8_device(_ptr(d_voxels), palette.ctypes.data,
                                                        nx, ny, nz, _stream(stream))))

    @classmethod
    def from_rgba8(cls, rgba):
        """rgba: uint8 [z, y, x, 4] or uint32 [z, y, x] texels."""
        a = np.ascontiguousarray(rgba)
        if a.dtype == np.uint32:
            nz, ny, nx = a.shape
        else:
            a = a.astype(np.uint8, copy=False)
            nz, ny, nx, _ = a.shape
        return cls(check(lib().vt_grid_create_rgba8(a.ctypes.data, nx, ny, nz)))

    @classmethod
    def from_chunk(cls, data, palette=None):
        """A z-fastest chunk (RawDynamicChunk order): numpy array indexed [x, y, z] of u8 palette
        indices (palette required), or [x, y, z, 4] u8 / [x, y, z] u32 RGBA8 texels.  Grid voxel
        (x, y, z) is data[x, y, z]."""
        a = np.ascontiguousarray(data)
        if palette is not None:
            a = a.astype(np.uint8, copy=False)
            nx, ny, nz = a.shape
            pal = np.ascontiguousarray(palette, np.uint32)
            return cls(check(lib().vt_grid_create(a.ctypes.data, PAYLOAD_U8, ORDER_Z_FASTEST,
                                                  pal.ctypes.data, nx, ny, nz)))
        if a.dtype == np.uint32:
            nx, ny, nz = a.shape
        else:
            a = a.astype(np.uint8, copy=False)
            nx, ny, nz, _ = a.shape
        return cls(check(lib().vt_grid_create(a.ctypes.data, PAYLOAD_RGBA8, ORDER_Z_FASTEST, None,
                                              nx, ny, nz)))

    def update(self, origin, voxels, order=ORDER_X_FASTEST):
        """Write a box of voxels at origin (x0, y0, z0): x-fastest arrays are indexed [z, y, x]
        (u8 indices, or [z, y, x, 4] u8 / [z, y, x] u32 texels for RGBA8 grids), z-fastest
        arrays [x, y, z]."""
        a = np.ascontiguousarray(voxels)
        if a.dtype != np.uint32 and a.ndim == 4:
            a = a.astype(np.uint8, copy=False).view(np.uint32)[..., 0]
        shape = a.shape if order == ORDER_Z_FASTEST else a.shape[::-1]
        w, h, d = shape
        x0, y0, z0 = origin
        check(lib().vt_grid_update(self.id, a.ctypes.data, order, x0, y0, z0, w, h, d))

    def info(self):
        gi = GridInfo()
        check(lib().vt_grid_get_info(self.id, ctypes.byref(gi)))
        return gi.as_dict()

    def bricks(self):
        inf = self.info()
        d = np.zeros(inf["bricks_total"], np.uint32)
        m = np.zeros(max(1, inf["slots"]) * 8, np.uint64)
        check(lib().vt_grid_download_bricks(self.id, d.ctypes.data, m.ctypes.data))
        return d, m[: inf["slots"] * 8].reshape(-1, 8)

    def octants(self):
        out = np.zeros(self.info()["bricks_total"], np.uint32)
        check(lib().vt_grid_download_octants(self.id, out.ctypes.data))
        return out

    def long_boxes(self):
        """Long-box words [3, bricks_total] (axis x, y, z)."""
        out = np.zeros(3 * self.info()["bricks_total"], np.uint32)
        check(lib().vt_grid_download_long(self.id, out.ctypes.data))
        return out.reshape(3, -1)

    def payload(self):
        """Brick payloads by slot: [slots, 8, 8, 8] u8 indices (z, y, x), or [slots, 8, 8, 8, 4]
        RGBA8 texels."""
        inf = self.info()
        rgba = inf["payload_format"] == PAYLOAD_RGBA8
        out = np.zeros(max(1, inf["slots"]) * 512 * (4 if rgba else 1), np.uint8)
        check(lib().vt_grid_download_payload(self.id, out.ctypes.data, out.nbytes))
        out = out[: inf["slots"] * 512 * (4 if rgba else 1)]
        return out.reshape(-1, 8, 8, 8, 4) if rgba else out.reshape(-1, 8, 8, 8)

    def destroy(self):
        if self.id is not None and self.id >= 0:
            check(lib().vt_grid_destroy(self.id))
            self.id = None


# ---------------------------------------------------------------- tracing

def trace_rays(grid, d_rays, n, d_hits, stream=None):
    """Asynchronous: n rays (device, 24 B each) -> n hit records (device, 16 B each)."""
    check(lib().vt_trace_rays(grid.id, _ptr(d_rays), n, _ptr(d_hits), _stream(stream)))


def trace_rays_host(grid, rays):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    hits = np.zeros(rays.shape[0], HIT_DTYPE)
    check(lib().vt_trace_rays_host(grid.id, rays.ctypes.data, rays.shape[0], hits.ctypes.data))
    return hits


def trace_rays_stats(grid, d_rays, n, d_hits):
    st = TraceStats()
    check(lib().vt_trace_rays_stats(grid.id, _ptr(d_rays), n, _ptr(d_hits), ctypes.byref(st)))
    return st.as_dict()


def render(grid, camera, light, d_hits, stream=None):
    """Asynchronous: camera.width*camera.height records into d_hits (device)."""
    check(lib().vt_render(grid.id, ctypes.byref(camera),
                          ctypes.byref(light) if light is not None else None, _ptr(d_hits),
                          _stream(stream)))


def _nbytes(x):
    return x.nbytes if isinstance(x, np.ndarray) else x.numel() * x.element_size()


def render_host(grid, camera, light=None, out=None):
    if out is not None and _nbytes(out) < camera.height * camera.width * 16:
        raise ValueError("render_host: out holds fewer than width*height 16-byte records")
    hits = out if out is not None else np.zeros(camera.height * camera.width, HIT_DTYPE)
    check(lib().vt_render_host(grid.id, ctypes.byref(camera),
                               ctypes.byref(light) if light is not None else None,
                               _ptr(hits)))
    return hits.reshape(camera.height, camera.width) if out is None else hits


def path_trace(grid, camera, params, d_out, d_rays=None, stream=None):
    """Asynchronous: width*height pixels (float4 or RGBA8 per params.out_format) into d_out
    (device); d_rays (device u64) accumulates the rays traced."""
    check(lib().vt_path_trace(grid.id, ctypes.byref(camera), ctypes.byref(params), _ptr(d_out),
                              _ptr(d_rays), _stream(stream)))


def path_trace_host(grid, camera, params, out=None):
    """-> (image [height, width, 4] float32 or uint8, rays traced).  `out`: optional host buffer
    of the image's size (a page-locked one is written by the kernel directly)."""
    px = 16 if params.out_format == PATH_OUT_F32X4 else 4
    if out is None:
        dt = np.float32 if params.out_format == PATH_OUT_F32X4 else np.uint8
        out = np.zeros((camera.height, camera.width, 4), dt)
    elif _nbytes(out) < camera.height * camera.width * px:
        raise ValueError("path_trace_host: out is smaller than the image")
    rays = ctypes.c_uint64(0)
    check(lib().vt_path_trace_host(grid.id, ctypes.byref(camera), ctypes.byref(params),
                                   _ptr(out), ctypes.byref(rays)))
    return out, rays.value


def render_footprint(grid, camera, light, d_hits):
    """Distinct bricks one frame touches: {"bricks", "nonempty_bricks", "hit_bricks"}."""
    fp = Footprint()
    check(lib().vt_render_footprint(grid.id, ctypes.byref(camera),
                                    ctypes.byref(light) if light is not None else None,
                                    _ptr(d_hits), ctypes.byref(fp)))
    return {"bricks": fp.bricks, "nonempty_bricks": fp.nonempty_bricks, "hit_bricks": fp.hit_bricks}


def render_phases(grid, camera, light, d_hits):
    """Warp-time phase profile of one frame (vt_render_phases; same records in `d_hits` as
    render): {"camera": {phase: warp cycles}, "shadow": {...}, "passes": {"camera_walk",
    "camera_cross", "shadow_walk", "shadow_cross"}, "warps": n}, phases as in PHASES."""
    pp = PhaseProfile()
    check(lib().vt_render_phases(grid.id, ctypes.byref(camera),
                                 ctypes.byref(light) if light is not None else None,
                                 _ptr(d_hits), ctypes.byref(pp)))
    out = {kind: {ph: int(pp.warp_cycles[k][i]) for i, ph in enumerate(PHASES)}
           for k, kind in enumerate(("camera", "shadow"))}
    out["passes"] = {"camera_walk": int(pp.passes[0][0]), "camera_cross": int(pp.passes[0][1]),
                     "shadow_walk": int(pp.passes[1][0]), "shadow_cross": int(pp.passes[1][1])}
    out["warps"] = int(pp.warps)
    return out


def render_stats(grid, camera, light, d_hits):
    st = TraceStats()
    check(lib().vt_render_stats(grid.id, ctypes.byref(camera),
                                ctypes.byref(light) if light is not None else None,
                                _ptr(d_hits), ctypes.byref(st)))
    return st.as_dict()


# ---------------------------------------------------------------- batched multi-view

class Batch:
    """Many views (grid, camera, spp, light, device output) rendered by one persistent launch
    replayed from a captured CUDA graph."""

    def __init__(self, views):
        arr = (View * len(views))(*views)
        bid = ctypes.c_int32(-1)
        check(lib().vt_batch_create(arr, len(views), ctypes.byref(bid)))
        self.id = bid.value
        p, w = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().vt_batch_info(self.id, ctypes.byref(p), ctypes.byref(w)))
        self.primary_rays, self.work_items = p.value, w.value

    def run(self, stream=None, graph=True):
        f = lib().vt_batch_run if graph else lib().vt_batch_run_direct
        check(f(self.id, _stream(stream)))

    def stats(self):
        """Counting run (same records, slower kernel build): traversal counters as a dict."""
        st = TraceStats()
        check(lib().vt_batch_stats(self.id, ctypes.byref(st)))
        return st.as_dict()

    def destroy(self):
        if self.id is not None:
            check(lib().vt_batch_destroy(self.id))
            self.id = None


def make_view(grid, camera, d_out, spp=1, seed=0, view_id=0, light=None):
    v = View()
    v.grid = grid.id if isinstance(grid, Grid) else int(grid)
    v.spp, v.seed, v.view_id = spp, seed, view_id
    v.flags = VIEW_LIGHT if light is not None else 0
    v.camera = camera
    if light is not None:
        v.light = light
    v.d_out = _ptr(d_out)
    return v


# ---------------------------------------------------------------- serving

class Service:
    """Continuous-batching render service (see vt_serve_* in include/vtrace.h)."""

    def __init__(self, hbm_budget_bytes=None, max_inflight=None, max_views_per_launch=None,
                 max_samples_per_launch=None, plain=False, refill_min=None,
                 max_samples_per_piece=None):
        """plain: the per-request baseline (one unsplit request per launch, one launch at a time,
        a slot buffer of 32M samples so that requests up to 1920x1080 x 16 spp need no
        temporary)."""
        cfg = ServeConfig()
        check(lib().vt_serve_default_config(ctypes.byref(cfg)))
        if hbm_budget_bytes is not None:
            cfg.hbm_budget_bytes = hbm_budget_bytes
        if max_inflight is not None:
            cfg.max_inflight = max_inflight
        if max_views_per_launch is not None:
            cfg.max_views_per_launch = max_views_per_launch
        if max_samples_per_launch is not None:
            cfg.max_samples_per_launch = max_samples_per_launch
        if refill_min is not None:
            cfg.refill_min = refill_min
        if max_samples_per_piece is not None:
            cfg.max_samples_per_piece = max_samples_per_piece
        if plain:
            cfg.max_inflight, cfg.max_views_per_launch, cfg.max_samples_per_piece = 1, 1, 0
            if max_samples_per_launch is None:
                cfg.max_samples_per_launch = 32 << 20
        sid = ctypes.c_int32(-1)
        check(lib().vt_serve_start(ctypes.byref(cfg), ctypes.byref(sid)))
        self.id = sid.value
        self._keep = {}

    def add_scene(self, voxels, palette):
        """Registers a [z, y, x] u8 scene; the service reads this array (kept here) for its
        builds."""
        voxels = np.ascontiguousarray(voxels, np.uint8)
        palette = np.ascontiguousarray(palette, np.uint32)
        nz, ny, nx = voxels.shape
        out = ctypes.c_int32(-1)
        check(lib().vt_serve_add_scene(self.id, voxels.ctypes.data, palette.ctypes.data, nx, ny,
                                       nz, ctypes.byref(out)))
        self._keep[out.value] = (voxels, palette)
        return out.value

    def update_scene(self, scene, origin, voxels):
        """Writes a [d, h, w] u8 box at origin (x0, y0, z0) into the scene's registered array and
        into its resident grid (vt_serve_update_scene)."""
        arr = self._keep[scene][0]
        box = np.asarray(voxels, np.uint8)
        d, h, w = box.shape
        x0, y0, z0 = origin
        arr[z0:z0 + d, y0:y0 + h, x0:x0 + w] = box
        check(lib().vt_serve_update_scene(self.id, scene, x0, y0, z0, w, h, d))

    def submit(self, scene, camera, out_rgba, spp=1, seed=0, view_id=0, light=None):
        if out_rgba is not None and not isinstance(out_rgba, int) and \
                _nbytes(out_rgba) < camera.width * camera.height * 4:
            raise ValueError("submit: out_rgba is smaller than the width x height RGBA8 image")
        r = ServeRequest()
        r.scene, r.spp, r.seed, r.view_id = scene, spp, seed, view_id
        r.flags = VIEW_LIGHT if light is not None else 0
        r.camera = camera
        if light is not None:
            r.light = light
        r.host_rgba = _ptr(out_rgba)
        rid = ctypes.c_uint64(0)
        check(lib().vt_serve_submit(self.id, ctypes.byref(r), ctypes.byref(rid)))
        return rid.value

    def poll(self, request_id, timeout_us=0):
        """None while the request runs; its timing dict when done; raises on a failure."""
        t = ServeTiming()
        rc = lib().vt_serve_poll(self.id, request_id, timeout_us, ctypes.byref(t))
        if rc == -8:
            return None
        check(rc)
        return {"submit_ns": t.submit_ns, "launch_ns": t.launch_ns, "done_ns": t.done_ns,
                "samples": t.samples}

    def wait(self, request_id, timeout_s=60.0):
        timing = self.poll(request_id, int(timeout_s * 1e6))
        if timing is None:
            raise VtError(-5, "request %d not done after %.1f s" % (request_id, timeout_s))
        return timing

    def stats(self):
        st = ServeStats()
        check(lib().vt_serve_get_stats(self.id, ctypes.byref(st)))
        return st.as_dict()

    def stop(self):
        if self.id is not None:
            check(lib().vt_serve_stop(self.id))
            self.id = None
