/*
 * vt_oracle.h — CPU restatement of vtrace's voxel traversal (TEST INFRASTRUCTURE ONLY).
 *
 * This oracle is the parity checker for libvtrace's CUDA kernels and the timed CPU baseline.  It
 * is never part of the product path: only the tests, the smoke check and the benchmark's CPU
 * baseline leg load it.
 *
 * Semantics restated (reference paths relative to the vtrace source tree):
 *  - shaders/trace.frag:68-71   DDA set-up: voxel = floor(min(pos, size-1)), step = sign(dir),
 *                               delta = |length(dir)/dir|, side = (sign*(voxel-pos) + sign*0.5
 *                               + 0.5) * delta
 *  - shaders/trace.frag:73-75   loop guard: steps < sx+sy+sz and voxel inside [0,size)
 *  - shaders/trace.frag:76-80   sample the voxel; hit iff alpha > 0 (NEAREST, CLAMP_TO_EDGE,
 *                               lib/descriptor.c:97-117; alpha of an RGBA8 texel is linear)
 *  - shaders/trace.frag:83-86   mask = side <= min(side.yzx, side.zxy); side += mask*delta;
 *                               voxel += mask*step (two or three axes step at once on ties)
 *  - shaders/trace.frag:89      miss; the pixel keeps the clear colour (lib/command.c:57-60)
 * Arithmetic: IEEE binary32, round to nearest, no contraction (-ffp-contract=off), operations in
 * the order the GLSL writes them.  min() is GLSL's `y < x ? y : x`.  `vec3(mask) * delta` is read
 * as a select (mask ? delta : 0), the rewrite GPU shader compilers apply to b2f-multiplies; the
 * literal IEEE product 0 * inf = NaN would freeze rays with a zero direction component.
 *
 * Parity pin: the reference has no golden vectors for this path and its shaders need a graphics
 * API.  oracle/build.py (build_ref) compiles shaders/trace.frag itself as C++ through a
 * GLSL-compatibility header (oracle/glsl_compat.hpp, driven by oracle/ref_harness.cpp); tests compare this restatement against that build where the
 * reference tree is present.  Camera ray generation, the slab entry, face ids, t, shading and
 * shadow rays are this project's own specification (the reference derives rays from rasterised
 * cube faces and has no shading), stated once here and mirrored by the kernels.
 */
#ifndef VT_ORACLE_H
#define VT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vto_hit { /* layout identical to vt_hit */
    uint16_t x, y, z;
    uint8_t palette_index;
    uint8_t face;
    float t;
    uint32_t rgba;
} vto_hit;

typedef struct vto_grid {
    const uint8_t* voxels;    /* u8 palette indices, x-fastest, or NULL */
    const uint32_t* palette;  /* 256 RGBA8 entries (with voxels) */
    const uint32_t* texels;   /* RGBA8 per voxel, x-fastest, or NULL */
    int32_t nx, ny, nz;
    uint8_t* brick_nonempty;  /* filled by vto_grid_prepare: one byte per 8^3 brick */
} vto_grid;

typedef struct vto_camera { /* layout identical to vt_camera */
    float origin[3];
    float forward[3];
    float right[3];
    float up[3];
    uint32_t width, height;
} vto_camera;

typedef struct vto_light { /* layout identical to vt_light */
    float dir[3];
    float ambient;
    uint32_t shadows;
} vto_light;

typedef struct vto_stats { /* layout identical to vt_trace_stats */
    uint64_t rays, shadow_rays, hits, steps;
    uint64_t bricks_entered, nonempty_bricks_entered, voxels_tested, ties;
} vto_stats;

typedef struct vto_dda_out {
    int32_t v[3];       /* final voxel */
    int32_t hit;
    uint32_t steps;     /* loop iterations executed */
    int32_t last_mask;  /* axes stepped on the final iteration (bit a); 0 if none */
    int32_t tie;        /* some iteration stepped two or three axes */
    int32_t step[3];
} vto_dda_out;

typedef struct vto_hit64 {
    int32_t hit;
    int32_t v[3];
    int32_t face;
    int32_t tie;
    double t;
} vto_hit64;

/* sRGB encoding of the reference clear colour (0.53, 0.81, 0.92, 1). */
#define VTO_SKY_RGBA 0xFFF6E8C0u
#define VTO_FLAG_SHADOW_RAY 0x08u
#define VTO_FLAG_INVALID 0x10u
#define VTO_FLAG_SHADOWED 0x20u
#define VTO_FLAG_HIT 0x80u

/* Allocate and fill g->brick_nonempty; vto_grid_release frees it. */
int vto_grid_prepare(vto_grid* g);
void vto_grid_release(vto_grid* g);

/* The reference DDA (shaders/trace.frag:68-87) from grid-space entry point `pos`. */
void vto_dda_f32(const vto_grid* g, const float pos[3], const float dir[3], vto_dda_out* out,
                 vto_stats* stats);

/* The reference shader's own entry form (identity matrices): d = normalize(s[i]),
 * pos = (mp[i] + 0.5) * size, then the DDA.  out[5*i..] = {hit, x, y, z, fetches}, where
 * fetches = loop iterations + hit, the number of texture() calls the shader makes. */
void vto_trace_entry_points(const vto_grid* g, uint64_t n, const float* mp, const float* s,
                            int32_t* out);

/* Ray/box slab entry: 0 = misses the grid, 1 = enters from outside (pos on the entry face),
 * 2 = origin inside the closed box (pos = origin). */
int vto_slab_entry(const vto_grid* g, const float o[3], const float d[3], float pos[3],
                   float* t_entry, int* entry_axis);

/* One ray: validity check, slab entry, DDA, face, t, unshaded colour (0 on a miss). */
void vto_trace_ray_f32(const vto_grid* g, const float o[3], const float d[3], vto_hit* out,
                       vto_stats* stats);
/* The same ray with the DDA recurrence in binary64 (entry point from the binary32 slab test). */
void vto_trace_ray_f64(const vto_grid* g, const float o[3], const float d[3], vto_hit64* out);

/* Camera ray for pixel (px, py) with sub-pixel offset (jx, jy). */
void vto_raygen(const vto_camera* c, uint32_t px, uint32_t py, float jx, float jy, float o[3],
                float d[3]);
/* Philox4x32-10 (Salmon et al., SC'11), the published counter-based generator. */
void vto_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Sub-pixel jitter of sample `s` of pixel (px, py) in view `view`: both in [0,1). */
void vto_jitter(uint32_t seed, uint32_t view, uint32_t px, uint32_t py, uint32_t s, float* jx,
                float* jy);

/* Primary ray + shading + optional shadow ray for one pixel sample. */
void vto_shade_sample(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                      uint32_t px, uint32_t py, float jx, float jy, vto_hit* out,
                      vto_stats* stats);

/* Whole image, one record per pixel (pixel centres), `threads` host threads (0 = all cores). */
void vto_render(const vto_grid* g, const vto_camera* cam, const vto_light* light, vto_hit* hits,
                int threads, vto_stats* stats);
/* Rows [row0, row1) only (for bounded CPU samples of a large image). */
void vto_render_rows(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                     uint32_t row0, uint32_t row1, vto_hit* hits, int threads, vto_stats* stats);
/* Jittered multi-sample view: hits[(py*width + px)*spp + s]. */
void vto_render_view(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                     uint32_t spp, uint32_t seed, uint32_t view, vto_hit* hits, int threads,
                     vto_stats* stats);
/* Ray buffer: rays are 6 floats (origin, dir). */
void vto_trace_rays(const vto_grid* g, const float* rays, uint64_t n, vto_hit* hits, int threads,
                    vto_stats* stats);
/* binary64 traversal of a ray buffer (for t accuracy and tie-divergence statistics). */
void vto_trace_rays_f64(const vto_grid* g, const float* rays, uint64_t n, vto_hit64* hits,
                        int threads);
/* The rays of a rendered frame as ray-buffer entries (6 floats each): the camera ray of every
 * pixel (pixel centres, row-major from the top row) into camera_rays, and, for every record of
 * `hits` (the frame's width * height records) that carries VTO_FLAG_SHADOW_RAY, the shadow ray
 * shade_from_ray traced for it, in pixel order, into shadow_rays (capacity width * height).
 * Returns the number of shadow rays written. */
uint64_t vto_frame_rays(const vto_camera* cam, const vto_light* light, const vto_hit* hits,
                        float* camera_rays, float* shadow_rays);

/* The reference's multi-instance frame as libvtrace's headless render_tick computes it: RGBA8
 * sRGB pixels, row-major from the top row.  instances: n column-major mat4 (texture id in the bits
 * of element [3][3]); grids: the textures by id.  Returns 0, or -1 for singular matrices. */
int vto_compat_render(const vto_grid* grids, uint32_t ngrids, const float* instances,
                      uint32_t ninst, const float P[16], const float C[16], int32_t width,
                      int32_t height, uint8_t* rgba, int threads);

int vto_hardware_threads(void);

/* Path tracing: the library's estimator (vt_path.cu), restated. */
typedef struct vto_path_params { /* layout identical to vt_path_params */
    uint32_t spp, max_bounces, seed, out_format;
    float sky[3], sun_dir[3], sun[3];
} vto_path_params;
void vto_path_pixel(const vto_grid* g, const vto_camera* cam, const vto_path_params* p,
                    uint32_t px, uint32_t py, float out[3], uint64_t* rays);
/* Rows row0..row1-1 of the image into out ((row1 - row0) * width * 4 floats: r, g, b, 1); rays
 * may be NULL. */
void vto_path_trace(const vto_grid* g, const vto_camera* cam, const vto_path_params* params,
                    uint32_t row0, uint32_t row1, float* out, int threads, uint64_t* rays);

#ifdef __cplusplus
}
#endif

#endif
