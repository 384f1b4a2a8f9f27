// vt_gen.cpp — seeded synthetic scenes, rays and palettes (host code of libvtrace).
//
// Deterministic across x86-64 and aarch64: integer hashing plus IEEE binary32 arithmetic built
// with -ffp-contract=off; no libm transcendental calls (sqrt is correctly rounded everywhere).
// Work is split over host threads by z-slabs; each voxel depends only on its coordinates and the
// seed, so the result does not depend on the thread count.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "vt_internal.h"

namespace vt {

// lowbias32 integer finaliser (C. Wellons, "hash-prospector"), a published 32-bit mixer.
static inline uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
static inline uint32_t hash4(uint32_t seed, uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = mix32(seed ^ 0x9E3779B9u);
    h = mix32(h ^ a);
    h = mix32(h ^ (b + 0x85EBCA6Bu));
    h = mix32(h ^ (c + 0xC2B2AE35u));
    return h;
}
static inline float unit24(uint32_t h) { return (float)(h >> 8) * 0x1p-24f; }  // [0,1)

static void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& fn) {
    unsigned hw = std::thread::hardware_concurrency();
    int64_t threads = hw ? (int64_t)hw : 4;
    if (threads > n) threads = n;
    if (threads <= 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    int64_t per = (n + threads - 1) / threads;
    for (int64_t t = 0; t < threads; ++t) {
        int64_t b = t * per, e = std::min(n, b + per);
        if (b >= e) break;
        pool.emplace_back(fn, b, e);
    }
    for (auto& th : pool) th.join();
}

static inline uint8_t voxel_value(uint32_t seed, uint32_t x, uint32_t y, uint32_t z) {
    return (uint8_t)(1u + hash4(seed ^ 0xA5A5A5A5u, x, y, z) % 255u);
}

// ---------------------------------------------------------------- gradient noise
// Perlin-style gradient noise on the integer lattice with the quintic fade 6t^5 - 15t^4 + 10t^3.
static inline float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
static inline float lerpf(float a, float b, float t) { return a + t * (b - a); }

static inline float grad2(uint32_t seed, int32_t ix, int32_t iy, float fx, float fy) {
    uint32_t h = hash4(seed, (uint32_t)ix, (uint32_t)iy, 0x2D2Du) & 7u;
    // eight unit-ish directions
    static const float gx[8] = {1.f, -1.f, 1.f, -1.f, 1.f, -1.f, 0.f, 0.f};
    static const float gy[8] = {1.f, 1.f, -1.f, -1.f, 0.f, 0.f, 1.f, -1.f};
    return gx[h] * fx + gy[h] * fy;
}

static float noise2(uint32_t seed, float x, float y) {
    float flx = floorf(x), fly = floorf(y);
    int32_t ix = (int32_t)flx, iy = (int32_t)fly;
    float fx = x - flx, fy = y - fly;
    float u = fade(fx), v = fade(fy);
    float n00 = grad2(seed, ix, iy, fx, fy);
    float n10 = grad2(seed, ix + 1, iy, fx - 1.f, fy);
    float n01 = grad2(seed, ix, iy + 1, fx, fy - 1.f);
    float n11 = grad2(seed, ix + 1, iy + 1, fx - 1.f, fy - 1.f);
    return lerpf(lerpf(n00, n10, u), lerpf(n01, n11, u), v);  // roughly [-1, 1]
}

static inline float grad3(uint32_t seed, int32_t ix, int32_t iy, int32_t iz, float fx, float fy,
                          float fz) {
    // the 12 cube-edge gradients of improved Perlin noise
    uint32_t h = hash4(seed, (uint32_t)ix, (uint32_t)iy, (uint32_t)iz) % 12u;
    switch (h) {
        case 0: return fx + fy;
        case 1: return -fx + fy;
        case 2: return fx - fy;
        case 3: return -fx - fy;
        case 4: return fx + fz;
        case 5: return -fx + fz;
        case 6: return fx - fz;
        case 7: return -fx - fz;
        case 8: return fy + fz;
        case 9: return -fy + fz;
        case 10: return fy - fz;
        default: return -fy - fz;
    }
}

static float noise3(uint32_t seed, float x, float y, float z) {
    float flx = floorf(x), fly = floorf(y), flz = floorf(z);
    int32_t ix = (int32_t)flx, iy = (int32_t)fly, iz = (int32_t)flz;
    float fx = x - flx, fy = y - fly, fz = z - flz;
    float u = fade(fx), v = fade(fy), w = fade(fz);
    float c[8];
    for (int k = 0; k < 8; ++k) {
        int dx = k & 1, dy = (k >> 1) & 1, dz = (k >> 2) & 1;
        c[k] = grad3(seed, ix + dx, iy + dy, iz + dz, fx - (float)dx, fy - (float)dy,
                     fz - (float)dz);
    }
    float x00 = lerpf(c[0], c[1], u), x10 = lerpf(c[2], c[3], u);
    float x01 = lerpf(c[4], c[5], u), x11 = lerpf(c[6], c[7], u);
    return lerpf(lerpf(x00, x10, v), lerpf(x01, x11, v), w);
}

// ---------------------------------------------------------------- generators

int32_t gen_palette(uint32_t seed, uint32_t* pal) {
    pal[0] = 0u;  // index 0 = empty (alpha 0)
    for (uint32_t i = 1; i < 256; ++i) {
        uint32_t h = hash4(seed, i, 0x7A1Eu, 1u);
        uint32_t a = 1u + hash4(seed, i, 0x7A1Eu, 2u) % 255u;  // alpha >= 1: occupied
        pal[i] = (h & 0x00FFFFFFu) | (a << 24);
    }
    return VT_OK;
}

int32_t gen_terrain(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t octaves,
                    float occupancy, uint8_t* vox) {
    // column heights over the (x, z) plane from fBm; solid from y = 0 up to the height
    std::vector<uint32_t> height((size_t)nx * nz);
    const float base_freq = 4.0f / (float)std::max(nx, nz);  // ~4 features across the grid
    parallel_for(nz, [&](int64_t z0, int64_t z1) {
        for (int64_t z = z0; z < z1; ++z)
            for (uint32_t x = 0; x < nx; ++x) {
                float f = 0.f, amp = 0.5f, freq = base_freq, norm = 0.f;
                for (uint32_t o = 0; o < octaves; ++o) {
                    f = f + amp * noise2(seed + 17u * o, (float)x * freq, (float)z * freq);
                    norm = norm + amp;
                    amp = amp * 0.5f;
                    freq = freq * 2.0f;
                }
                f = f / norm;  // about [-1, 1], mean ~0
                float h = occupancy + 0.9f * f;
                h = h < 0.f ? 0.f : (h > 1.f ? 1.f : h);
                height[(size_t)z * nx + x] = (uint32_t)(h * (float)ny);
            }
    });
    parallel_for(nz, [&](int64_t z0, int64_t z1) {
        for (int64_t z = z0; z < z1; ++z)
            for (uint32_t y = 0; y < ny; ++y) {
                uint8_t* row = vox + (size_t)nx * (y + (size_t)ny * z);
                for (uint32_t x = 0; x < nx; ++x)
                    row[x] = y < height[(size_t)z * nx + x] ? voxel_value(seed, x, y, (uint32_t)z)
                                                             : 0;
            }
    });
    return VT_OK;
}

struct Shape {
    float c[3];
    float h[3];  // box half extents
    float r;     // sphere radius (0 for boxes)
    int32_t lo[3], hi[3];
    uint8_t value;
};

int32_t gen_shapes(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t count,
                   float rmin, float rmax, uint8_t* vox) {
    const uint32_t n[3] = {nx, ny, nz};
    std::vector<Shape> shapes(count);
    for (uint32_t i = 0; i < count; ++i) {
        Shape& s = shapes[i];
        // radius: rmin + (rmax - rmin) * u1*u2*u3 (product of three uniforms: many small shapes,
        // few large ones)
        float p = unit24(hash4(seed, i, 1u, 0u)) * unit24(hash4(seed, i, 2u, 0u)) *
                  unit24(hash4(seed, i, 3u, 0u));
        float r = rmin + (rmax - rmin) * p;
        bool sphere = (hash4(seed, i, 4u, 0u) & 1u) != 0u;
        for (int a = 0; a < 3; ++a) {
            s.c[a] = unit24(hash4(seed, i, 5u, (uint32_t)a)) * (float)n[a];
            s.h[a] = sphere ? r : r * (0.5f + 0.5f * unit24(hash4(seed, i, 6u, (uint32_t)a)));
            float ext = s.h[a] + 1.0f;
            float lo = s.c[a] - ext, hi = s.c[a] + ext;
            s.lo[a] = lo < 0.f ? 0 : (int32_t)lo;
            s.hi[a] = hi >= (float)n[a] ? (int32_t)n[a] - 1 : (int32_t)hi;
        }
        s.r = sphere ? r : 0.f;
        s.value = (uint8_t)(1u + hash4(seed, i, 7u, 0u) % 255u);
    }
    memset(vox, 0, (size_t)nx * ny * nz);
    // each worker owns a z range and rasterises every shape's part inside it (later shapes win)
    parallel_for(nz, [&](int64_t z0, int64_t z1) {
        for (const Shape& s : shapes) {
            int32_t zl = std::max<int32_t>(s.lo[2], (int32_t)z0), zh = std::min<int32_t>(s.hi[2], (int32_t)z1 - 1);
            for (int32_t z = zl; z <= zh; ++z) {
                float dz = ((float)z + 0.5f) - s.c[2];
                for (int32_t y = s.lo[1]; y <= s.hi[1]; ++y) {
                    float dy = ((float)y + 0.5f) - s.c[1];
                    uint8_t* row = vox + (size_t)nx * ((size_t)y + (size_t)ny * z);
                    for (int32_t x = s.lo[0]; x <= s.hi[0]; ++x) {
                        float dx = ((float)x + 0.5f) - s.c[0];
                        bool in;
                        if (s.r > 0.f)
                            in = (dx * dx + dy * dy) + dz * dz <= s.r * s.r;
                        else
                            in = fabsf(dx) <= s.h[0] && fabsf(dy) <= s.h[1] && fabsf(dz) <= s.h[2];
                        if (in) row[x] = s.value;
                    }
                }
            }
        }
    });
    return VT_OK;
}

int32_t gen_cave(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, float occupancy,
                 uint8_t* vox) {
    // two octaves of 3D gradient noise; the threshold is the (1 - occupancy) quantile of a
    // deterministic 64^3 sample of the same field
    const float f0 = 6.0f / (float)std::max(nx, std::max(ny, nz));
    auto field = [&](float x, float y, float z) {
        return noise3(seed, x * f0, y * f0, z * f0) +
               0.5f * noise3(seed + 101u, x * (2.f * f0), y * (2.f * f0), z * (2.f * f0));
    };
    std::vector<float> sample;
    const uint32_t S = 64;
    sample.reserve((size_t)S * S * S);
    for (uint32_t k = 0; k < S; ++k)
        for (uint32_t j = 0; j < S; ++j)
            for (uint32_t i = 0; i < S; ++i)
                sample.push_back(field(((float)i + 0.5f) * (float)nx / (float)S,
                                       ((float)j + 0.5f) * (float)ny / (float)S,
                                       ((float)k + 0.5f) * (float)nz / (float)S));
    size_t q = (size_t)((1.0f - occupancy) * (float)(sample.size() - 1));
    std::nth_element(sample.begin(), sample.begin() + q, sample.end());
    const float thr = sample[q];
    parallel_for(nz, [&](int64_t z0, int64_t z1) {
        for (int64_t z = z0; z < z1; ++z)
            for (uint32_t y = 0; y < ny; ++y) {
                uint8_t* row = vox + (size_t)nx * (y + (size_t)ny * z);
                for (uint32_t x = 0; x < nx; ++x)
                    row[x] = field((float)x, (float)y, (float)z) > thr
                                 ? voxel_value(seed, x, y, (uint32_t)z)
                                 : 0;
            }
    });
    return VT_OK;
}

int32_t gen_rays_uniform(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint64_t n,
                         vt_ray* rays) {
    const float dims[3] = {(float)nx, (float)ny, (float)nz};
    parallel_for((int64_t)((n + 4095) / 4096), [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            uint64_t i0 = (uint64_t)b * 4096, i1 = std::min<uint64_t>(n, i0 + 4096);
            for (uint64_t i = i0; i < i1; ++i) {
                uint32_t lo = (uint32_t)i, hi = (uint32_t)(i >> 32);
                vt_ray& r = rays[i];
                for (int a = 0; a < 3; ++a)
                    r.origin[a] = unit24(hash4(seed, lo, hi, 10u + (uint32_t)a)) * dims[a];
                // direction: rejection-sample the unit ball, then normalise
                for (uint32_t attempt = 0;; ++attempt) {
                    float v[3];
                    for (int a = 0; a < 3; ++a)
                        v[a] = 2.0f * unit24(hash4(seed ^ (attempt * 0x51ED27u), lo, hi,
                                                   20u + (uint32_t)a)) - 1.0f;
                    float q2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
                    if (q2 > 1e-6f && q2 <= 1.0f) {
                        float len = sqrtf(q2);
                        for (int a = 0; a < 3; ++a) r.dir[a] = v[a] / len;
                        break;
                    }
                }
            }
        }
    });
    return VT_OK;
}

}  // namespace vt

extern "C" {

int32_t vt_gen_palette(uint32_t seed, uint32_t* palette256) {
    if (!palette256) return vt::fail(VT_EINVAL, "vt_gen_palette: null palette");
    return vt::gen_palette(seed, palette256);
}

int32_t vt_gen_terrain(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t octaves,
                       float occupancy, uint8_t* voxels) {
    if (!voxels || !nx || !ny || !nz || octaves == 0 || octaves > 16 || !(occupancy >= 0.f) ||
        occupancy > 1.f)
        return vt::fail(VT_EINVAL, "vt_gen_terrain: bad argument");
    return vt::gen_terrain(nx, ny, nz, seed, octaves, occupancy, voxels);
}

int32_t vt_gen_shapes(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t count,
                      float rmin, float rmax, uint8_t* voxels) {
    if (!voxels || !nx || !ny || !nz || !(rmin > 0.f) || !(rmax >= rmin))
        return vt::fail(VT_EINVAL, "vt_gen_shapes: bad argument");
    return vt::gen_shapes(nx, ny, nz, seed, count, rmin, rmax, voxels);
}

int32_t vt_gen_cave(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, float occupancy,
                    uint8_t* voxels) {
    if (!voxels || !nx || !ny || !nz || !(occupancy > 0.f) || !(occupancy < 1.f))
        return vt::fail(VT_EINVAL, "vt_gen_cave: bad argument");
    return vt::gen_cave(nx, ny, nz, seed, occupancy, voxels);
}

int32_t vt_gen_rays_uniform(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint64_t n,
                            vt_ray* rays) {
    if (!rays || !nx || !ny || !nz) return vt::fail(VT_EINVAL, "vt_gen_rays_uniform: bad argument");
    return vt::gen_rays_uniform(nx, ny, nz, seed, n, rays);
}

int32_t vt_camera_look_at(const float eye[3], const float target[3], const float up[3],
                          float vfov_degrees, uint32_t width, uint32_t height, vt_camera* out) {
    if (!eye || !target || !up || !out || !width || !height || !(vfov_degrees > 0.f) ||
        !(vfov_degrees < 180.f))
        return vt::fail(VT_EINVAL, "vt_camera_look_at: bad argument");
    double f[3], u[3], r[3];
    for (int a = 0; a < 3; ++a) {
        f[a] = (double)target[a] - (double)eye[a];
        u[a] = up[a];
    }
    double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0.0)) return vt::fail(VT_EINVAL, "vt_camera_look_at: eye == target");
    for (int a = 0; a < 3; ++a) f[a] /= fl;
    r[0] = f[1] * u[2] - f[2] * u[1];
    r[1] = f[2] * u[0] - f[0] * u[2];
    r[2] = f[0] * u[1] - f[1] * u[0];
    double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (!(rl > 0.0)) return vt::fail(VT_EINVAL, "vt_camera_look_at: up parallel to view");
    for (int a = 0; a < 3; ++a) r[a] /= rl;
    double uu[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2],
                    r[0] * f[1] - r[1] * f[0]};
    const double th = tan(0.5 * (double)vfov_degrees * 3.14159265358979323846 / 180.0);
    const double aspect = (double)width / (double)height;
    for (int a = 0; a < 3; ++a) {
        out->origin[a] = eye[a];
        out->forward[a] = (float)f[a];
        out->right[a] = (float)(r[a] * th * aspect);
        out->up[a] = (float)(uu[a] * th);
    }
    out->width = width;
    out->height = height;
    return VT_OK;
}

}  // extern "C"
