// vt_vox.cpp — MagicaVoxel .vox models as the textures vtrace builds from them.
//
// vtrace loads .vox files with the dot_vox crate (4.1.0, Cargo.lock:127-129) and turns each model
// into a RawDynamicChunk<Color> (src/voxel/magica_voxel.rs:18-44), the buffer it hands to
// add_texture.  This file restates both steps from the published file format and the crate's
// documented behaviour:
//
//   file     "VOX " magic, int32 version, then chunks: 4-byte id, int32 content bytes, int32
//            children bytes, content, children.  MAIN holds every other chunk as children.
//            Each model is a SIZE chunk (int32 x, y, z) followed by an XYZI chunk (int32 count,
//            then count x (u8 x, y, z, colour index)).  RGBA holds 256 RGBA8 colours; colour
//            index c (1..255) is its entry c - 1.  Every other chunk (PACK, nTRN, nGRP, nSHP,
//            LAYR, MATL, rOBJ, ...) carries nothing this path uses and is skipped.
//   dot_vox  models in file order; a voxel's palette index is c - 1 (saturating at 0); the
//            palette is the RGBA chunk as little-endian u32.  A file without an RGBA chunk
//            would take MagicaVoxel's built-in default palette, which is not restated here:
//            such files are rejected.
//   chunk    RawDynamicChunk::new(size.x, size.y, size.z) filled with Color 0, then each voxel
//            (x, y, z, i) is stored at chunk coordinate (x, size.y - z - 1, y)
//            (magica_voxel.rs:31-37); the chunk keeps (cx, cy, cz) at cz + sz * (cy + sy * cx)
//            (rawchunk.rs:292).  Where that coordinate falls outside the chunk (z >= size.y or
//            y >= size.z on a model whose y and z sizes differ) the reference's unwrap panics;
//            here the call fails with VT_EINVAL.
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "vt_internal.h"
#include "vtrace.h"

namespace {

struct VoxModel {
    uint32_t sx = 0, sy = 0, sz = 0;
    const uint8_t* xyzi = nullptr;  // count x 4 bytes
    uint32_t count = 0;
    bool has_xyzi = false;
};

struct VoxFile {
    uint32_t version = 0;
    std::vector<VoxModel> models;
    const uint8_t* rgba = nullptr;  // 256 x 4 bytes
};

uint32_t rd32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Walks the chunks in [p, end); MAIN's children are walked in place.  Returns an empty string on
// success, else what is wrong.
std::string walk(const uint8_t* p, const uint8_t* end, VoxFile& f, int depth) {
    if (depth > 64) return "chunks nested too deeply";
    while (p < end) {
        if (end - p < 12) return "truncated chunk header";
        const uint8_t* id = p;
        const uint64_t n = rd32(p + 4), m = rd32(p + 8);
        p += 12;
        if ((uint64_t)(end - p) < n + m) return "chunk extends past the end of the file";
        const uint8_t* content = p;
        if (!memcmp(id, "MAIN", 4)) {
            std::string err = walk(content + n, content + n + m, f, depth + 1);
            if (!err.empty()) return err;
        } else if (!memcmp(id, "SIZE", 4)) {
            if (n < 12) return "SIZE chunk shorter than 12 bytes";
            const uint32_t x = rd32(content), y = rd32(content + 4), z = rd32(content + 8);
            if (x == 0 || y == 0 || z == 0 || x > 65535 || y > 65535 || z > 65535)
                return "model size outside 1..65535";
            VoxModel md;
            md.sx = x;
            md.sy = y;
            md.sz = z;
            f.models.push_back(md);
        } else if (!memcmp(id, "XYZI", 4)) {
            if (f.models.empty() || f.models.back().has_xyzi) return "XYZI chunk without a SIZE chunk";
            if (n < 4) return "XYZI chunk shorter than 4 bytes";
            const uint64_t count = rd32(content);
            if (count * 4 > n - 4) return "XYZI voxel count exceeds the chunk";
            f.models.back().xyzi = content + 4;
            f.models.back().count = (uint32_t)count;
            f.models.back().has_xyzi = true;
        } else if (!memcmp(id, "RGBA", 4)) {
            if (n < 1024) return "RGBA chunk shorter than 1024 bytes";
            f.rgba = content;
        }
        p = content + n + m;
    }
    return std::string();
}

int32_t parse(const uint8_t* bytes, uint64_t size, VoxFile& f) {
    if (!bytes) return vt::fail(VT_EINVAL, "vox: null buffer");
    if (size < 8 || memcmp(bytes, "VOX ", 4)) return vt::fail(VT_EINVAL, "vox: not a .vox file (magic)");
    f.version = rd32(bytes + 4);
    const std::string err = walk(bytes + 8, bytes + size, f, 0);
    if (!err.empty()) return vt::fail(VT_EINVAL, "vox: " + err);
    for (const VoxModel& m : f.models)
        if (!m.has_xyzi) return vt::fail(VT_EINVAL, "vox: SIZE chunk without XYZI chunk");
    return VT_OK;
}

int32_t pick(const uint8_t* bytes, uint64_t size, uint32_t model, VoxFile& f) {
    int32_t rc = parse(bytes, size, f);
    if (rc) return rc;
    if (model >= f.models.size()) return vt::fail(VT_ENOTFOUND, "vox: no such model");
    return VT_OK;
}

}  // namespace

extern "C" {

int32_t vt_vox_inspect(const uint8_t* bytes, uint64_t size, vt_vox_info* info) {
    if (!info) return vt::fail(VT_EINVAL, "vt_vox_inspect: null info");
    VoxFile f;
    int32_t rc = parse(bytes, size, f);
    if (rc) return rc;
    info->version = f.version;
    info->models = (uint32_t)f.models.size();
    info->has_palette = f.rgba ? 1u : 0u;
    info->reserved = 0;
    return VT_OK;
}

int32_t vt_vox_model_info(const uint8_t* bytes, uint64_t size, uint32_t model, vt_vox_model* out) {
    if (!out) return vt::fail(VT_EINVAL, "vt_vox_model_info: null output");
    VoxFile f;
    int32_t rc = pick(bytes, size, model, f);
    if (rc) return rc;
    const VoxModel& m = f.models[model];
    out->size[0] = m.sx;
    out->size[1] = m.sy;
    out->size[2] = m.sz;
    out->voxels = m.count;
    return VT_OK;
}

int32_t vt_vox_model_chunk(const uint8_t* bytes, uint64_t size, uint32_t model, uint8_t* rgba,
                           uint64_t capacity_bytes) {
    VoxFile f;
    int32_t rc = pick(bytes, size, model, f);
    if (rc) return rc;
    if (!f.rgba) return vt::fail(VT_EINVAL, "vox: no RGBA chunk (the default palette is not supported)");
    const VoxModel& m = f.models[model];
    const uint64_t need = (uint64_t)m.sx * m.sy * m.sz * 4;
    if (!rgba || capacity_bytes < need) return vt::fail(VT_EINVAL, "vt_vox_model_chunk: output too small");
    memset(rgba, 0, need);  // Color::from_uint(0)
    for (uint32_t k = 0; k < m.count; ++k) {
        const uint8_t* v = m.xyzi + 4 * (size_t)k;
        const uint32_t x = v[0], y = v[1], z = v[2];
        const uint32_t i = v[3] ? v[3] - 1u : 0u;
        // chunk coordinate (x, size.y - z - 1, y)
        if (x >= m.sx || z >= m.sy || y >= m.sz)
            return vt::fail(VT_EINVAL, "vox: voxel " + std::to_string(k) +
                                           " maps outside the model's chunk");
        const uint64_t cx = x, cy = m.sy - z - 1, cz = y;
        memcpy(rgba + 4 * (cz + (uint64_t)m.sz * (cy + (uint64_t)m.sy * cx)), f.rgba + 4 * i, 4);
    }
    return VT_OK;
}

}  // extern "C"
