"""Pure-Python restatement of vtrace's .vox model loading (TEST INFRASTRUCTURE ONLY).

Follows src/voxel/magica_voxel.rs:18-44 and the dot_vox 4.1.0 crate it calls (Cargo.lock:127-129;
the crate is not vendored with vtrace, so its behaviour is restated from the published MagicaVoxel
file format and the crate's documentation):

- a file is "VOX ", an int32 version, then chunks (4-byte id, int32 content size, int32 children
  size, content, children); MAIN's children hold the rest;
- models are (SIZE, XYZI) pairs in file order; an XYZI voxel is (x, y, z, c) bytes;
- a voxel's palette index is c - 1 saturating at 0, into the RGBA chunk read as 256 u32 LE;
- the texture of a model is a RawDynamicChunk(size.x, size.y, size.z) of Color 0 with voxel
  (x, y, z) written at (x, size.y - z - 1, y) (magica_voxel.rs:31-37), stored z-fastest
  (src/voxel/rawchunk.rs:292).

Also a writer of .vox files, to make test inputs.
"""
import struct

import numpy as np


def _chunks(buf, start, end):
    p = start
    while p < end:
        if end - p < 12:
            raise ValueError("truncated chunk header")
        cid = buf[p:p + 4]
        n, m = struct.unpack_from("<II", buf, p + 4)
        c0 = p + 12
        if c0 + n + m > end:
            raise ValueError("chunk extends past the end of the file")
        yield cid, c0, n, m
        p = c0 + n + m


def parse(buf):
    """-> (version, [(size (x, y, z), voxels uint8 [k, 4])], palette uint32[256] or None)."""
    buf = bytes(buf)
    if len(buf) < 8 or buf[:4] != b"VOX ":
        raise ValueError("not a .vox file")
    version = struct.unpack_from("<I", buf, 4)[0]
    models, palette = [], None

    def walk(start, end):
        nonlocal palette
        for cid, c0, n, m in _chunks(buf, start, end):
            if cid == b"MAIN":
                walk(c0 + n, c0 + n + m)
            elif cid == b"SIZE":
                models.append([struct.unpack_from("<III", buf, c0), None])
            elif cid == b"XYZI":
                k = struct.unpack_from("<I", buf, c0)[0]
                models[-1][1] = np.frombuffer(buf, np.uint8, 4 * k, c0 + 4).reshape(k, 4)
            elif cid == b"RGBA":
                palette = np.frombuffer(buf, "<u4", 256, c0).astype(np.uint32)

    walk(8, len(buf))
    return version, [(tuple(s), v) for s, v in models], palette


def model_chunk(buf, model=0):
    """The model's texture as uint8 [x, y, z, 4] (chunk order), per magica_voxel.rs:18-44."""
    _, models, palette = parse(buf)
    (sx, sy, sz), vox = models[model]
    out = np.zeros((sx, sy, sz), np.uint32)
    for x, y, z, c in vox.tolist():
        if x >= sx or z >= sy or y >= sz:
            raise IndexError("voxel maps outside the chunk")
        out[x, sy - z - 1, y] = palette[max(c, 1) - 1]
    return out.view(np.uint8).reshape(sx, sy, sz, 4)


def _chunk(cid, content=b"", children=b""):
    return cid + struct.pack("<II", len(content), len(children)) + content + children


def write(models, palette, version=150, pack=False, extra=()):
    """Bytes of a .vox file.  models: [((sx, sy, sz), voxels uint8 [k, 4])]; palette: 256 u32 or
    None (no RGBA chunk); extra: (id, content, children) chunks inserted before the models."""
    body = b""
    if pack:
        body += _chunk(b"PACK", struct.pack("<I", len(models)))
    for cid, content, children in extra:
        body += _chunk(cid, content, children)
    for (sx, sy, sz), vox in models:
        vox = np.ascontiguousarray(vox, np.uint8).reshape(-1, 4)
        body += _chunk(b"SIZE", struct.pack("<III", sx, sy, sz))
        body += _chunk(b"XYZI", struct.pack("<I", vox.shape[0]) + vox.tobytes())
    if palette is not None:
        body += _chunk(b"RGBA", np.ascontiguousarray(palette, "<u4").tobytes())
    return b"VOX " + struct.pack("<I", version) + _chunk(b"MAIN", b"", body)
