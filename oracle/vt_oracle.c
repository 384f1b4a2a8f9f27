/*
 * vt_oracle.c — CPU restatement of vtrace's voxel traversal (TEST INFRASTRUCTURE ONLY; see
 * vt_oracle.h for the semantics and the reference lines each part follows).
 *
 * Build with -ffp-contract=off: every float expression below is one IEEE binary32 operation per
 * operator, evaluated in source order.
 */
#define _GNU_SOURCE
#include "vt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* GLSL min(x, y) is defined as (y < x) ? y : x (GLSL 4.60 §8.3). */
static inline float glsl_min(float x, float y) { return (y < x) ? y : x; }
static inline double glsl_min64(double x, double y) { return (y < x) ? y : x; }
/* GLSL sign(): 1.0, 0.0 or -1.0. */
static inline float glsl_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

static inline uint32_t voxel_rgba(const vto_grid* g, int32_t x, int32_t y, int32_t z) {
    uint64_t i = (uint64_t)x + (uint64_t)g->nx * ((uint64_t)y + (uint64_t)g->ny * (uint64_t)z);
    if (g->texels) return g->texels[i];
    return g->palette[g->voxels[i]];
}
static inline uint8_t voxel_index(const vto_grid* g, int32_t x, int32_t y, int32_t z) {
    if (!g->voxels) return 0;
    uint64_t i = (uint64_t)x + (uint64_t)g->nx * ((uint64_t)y + (uint64_t)g->ny * (uint64_t)z);
    return g->voxels[i];
}
/* shaders/trace.frag:78: texSample.w > 0.0; the alpha byte a gives a/255 > 0 iff a != 0. */
static inline int voxel_occupied(const vto_grid* g, int32_t x, int32_t y, int32_t z) {
    return (voxel_rgba(g, x, y, z) >> 24) != 0u;
}

int vto_grid_prepare(vto_grid* g) {
    int32_t bx = (g->nx + 7) / 8, by = (g->ny + 7) / 8, bz = (g->nz + 7) / 8;
    g->brick_nonempty = (uint8_t*)calloc((size_t)bx * by * bz, 1);
    if (!g->brick_nonempty) return -1;
    for (int32_t z = 0; z < g->nz; ++z)
        for (int32_t y = 0; y < g->ny; ++y)
            for (int32_t x = 0; x < g->nx; ++x)
                if (voxel_occupied(g, x, y, z))
                    g->brick_nonempty[(x >> 3) + bx * ((y >> 3) + by * (z >> 3))] = 1;
    return 0;
}

void vto_grid_release(vto_grid* g) {
    free(g->brick_nonempty);
    g->brick_nonempty = NULL;
}

/* shaders/trace.frag:68-87, with the brick visit counters of the brick-grid layout. */
void vto_dda_f32(const vto_grid* g, const float pos[3], const float d[3], vto_dda_out* out,
                 vto_stats* stats) {
    const int32_t isize[3] = {g->nx, g->ny, g->nz};
    const float size[3] = {(float)g->nx, (float)g->ny, (float)g->nz};
    /* length(): sqrt((x*x + y*y) + z*z) */
    const float len = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    int32_t v[3], st[3];
    float delta[3], side[3];
    for (int a = 0; a < 3; ++a) {
        /* trace.frag:68 ivec3(floor(min(model_ray_pos, model_size - 1.0))) */
        float m = glsl_min(pos[a], size[a] - 1.0f);
        v[a] = (int32_t)floorf(m);
        /* trace.frag:69-71 */
        float sg = glsl_sign(d[a]);
        st[a] = (int32_t)sg;
        delta[a] = fabsf(len / d[a]);
        side[a] = ((sg * ((float)v[a] - pos[a]) + sg * 0.5f) + 0.5f) * delta[a];
    }
    const int32_t bxn = (g->nx + 7) / 8, byn = (g->ny + 7) / 8;
    const uint32_t max_steps = (uint32_t)(g->nx + g->ny + g->nz); /* trace.frag:74 */
    uint32_t steps = 0;
    int32_t last = 0, tie = 0, hit = 0;
    int64_t prev_brick = -1;
    while (steps < max_steps && v[0] >= 0 && v[1] >= 0 && v[2] >= 0 && v[0] < isize[0] &&
           v[1] < isize[1] && v[2] < isize[2]) { /* trace.frag:75 */
        int64_t brick = (int64_t)(v[0] >> 3) + bxn * ((int64_t)(v[1] >> 3) + (int64_t)byn * (v[2] >> 3));
        int nonempty = g->brick_nonempty ? g->brick_nonempty[brick] : 1;
        if (stats) {
            if (brick != prev_brick) {
                stats->bricks_entered++;
                if (nonempty) stats->nonempty_bricks_entered++;
            }
            if (nonempty) stats->voxels_tested++;
        }
        prev_brick = brick;
        if (nonempty && voxel_occupied(g, v[0], v[1], v[2])) { /* trace.frag:76-80 */
            hit = 1;
            break;
        }
        /* trace.frag:83-86 */
        float mnx = glsl_min(side[1], side[2]);
        float mny = glsl_min(side[2], side[0]);
        float mnz = glsl_min(side[0], side[1]);
        int bx = side[0] <= mnx, by = side[1] <= mny, bz = side[2] <= mnz;
        if (bx) side[0] = side[0] + delta[0];
        if (by) side[1] = side[1] + delta[1];
        if (bz) side[2] = side[2] + delta[2];
        if (bx) v[0] += st[0];
        if (by) v[1] += st[1];
        if (bz) v[2] += st[2];
        last = bx | (by << 1) | (bz << 2);
        if (bx + by + bz > 1) tie = 1;
        ++steps;
    }
    if (stats) stats->steps += steps;
    for (int a = 0; a < 3; ++a) {
        out->v[a] = v[a];
        out->step[a] = st[a];
    }
    out->hit = hit;
    out->steps = steps;
    out->last_mask = last;
    out->tie = tie;
}

int vto_slab_entry(const vto_grid* g, const float o[3], const float d[3], float pos[3],
                   float* t_entry, int* entry_axis) {
    const float size[3] = {(float)g->nx, (float)g->ny, (float)g->nz};
    float tn = -INFINITY, tf = INFINITY;
    int ax = -1;
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
            if (o[a] < 0.0f || o[a] > size[a]) return 0;
            continue;
        }
        float ta = (0.0f - o[a]) / d[a];
        float tb = (size[a] - o[a]) / d[a];
        float lo = ta < tb ? ta : tb;
        float hi = ta < tb ? tb : ta;
        if (lo > tn) {
            tn = lo;
            ax = a;
        }
        if (hi < tf) tf = hi;
    }
    if (tn > tf || tf < 0.0f) return 0;
    if (tn <= 0.0f) {
        pos[0] = o[0];
        pos[1] = o[1];
        pos[2] = o[2];
        *t_entry = 0.0f;
        *entry_axis = -1;
        return 2;
    }
    for (int b = 0; b < 3; ++b) {
        float p = o[b] + tn * d[b];
        p = p < 0.0f ? 0.0f : p;
        p = p > size[b] ? size[b] : p;
        pos[b] = p;
    }
    pos[ax] = d[ax] > 0.0f ? 0.0f : size[ax];
    *t_entry = tn;
    *entry_axis = ax;
    return 1;
}

static inline uint8_t face_code(int axis, int normal_positive) {
    return (uint8_t)(1 + 2 * axis + (normal_positive ? 0 : 1));
}

static void miss_record(vto_hit* out, uint8_t flags) {
    out->x = out->y = out->z = 0xFFFF;
    out->palette_index = 0;
    out->face = flags;
    out->t = INFINITY;
    out->rgba = 0;
}

static inline int finite3(const float a[3]) {
    return isfinite(a[0]) && isfinite(a[1]) && isfinite(a[2]);
}

void vto_trace_ray_f32(const vto_grid* g, const float o[3], const float d[3], vto_hit* out,
                       vto_stats* stats) {
    if (stats) stats->rays++;
    if (!finite3(o) || !finite3(d)) {
        miss_record(out, VTO_FLAG_INVALID);
        return;
    }
    float pos[3], t_entry;
    int entry_axis;
    int kind = vto_slab_entry(g, o, d, pos, &t_entry, &entry_axis);
    if (kind == 0) {
        miss_record(out, 0);
        return;
    }
    vto_dda_out r;
    vto_dda_f32(g, pos, d, &r, stats);
    const uint8_t flags = 0; /* ties are counted in the statistics, not flagged per record */
    if (stats && r.tie) stats->ties++;
    if (!r.hit) {
        miss_record(out, flags);
        return;
    }
    uint8_t face = 0;
    float t = 0.0f;
    if (r.last_mask != 0) { /* the ray moved: face of the final iteration's step */
        int a = (r.last_mask & 1) ? 0 : ((r.last_mask & 2) ? 1 : 2);
        float plane = (float)(r.step[a] > 0 ? r.v[a] : r.v[a] + 1);
        t = (plane - o[a]) / d[a];
        face = face_code(a, r.step[a] < 0);
    } else if (kind == 1) {
        int a = entry_axis;
        t = t_entry;
        face = face_code(a, d[a] < 0.0f);
    }
    out->x = (uint16_t)r.v[0];
    out->y = (uint16_t)r.v[1];
    out->z = (uint16_t)r.v[2];
    out->palette_index = voxel_index(g, r.v[0], r.v[1], r.v[2]);
    out->face = (uint8_t)(face | flags | VTO_FLAG_HIT);
    out->t = t;
    out->rgba = voxel_rgba(g, r.v[0], r.v[1], r.v[2]);
}

/* The same traversal with the DDA state in binary64; the entry point comes from the binary32 slab
 * test so that only the recurrence differs. */
void vto_trace_ray_f64(const vto_grid* g, const float o[3], const float d[3], vto_hit64* out) {
    memset(out, 0, sizeof(*out));
    out->t = INFINITY;
    if (!finite3(o) || !finite3(d)) return;
    float pos32[3], t_entry;
    int entry_axis;
    int kind = vto_slab_entry(g, o, d, pos32, &t_entry, &entry_axis);
    if (kind == 0) return;
    const int32_t isize[3] = {g->nx, g->ny, g->nz};
    const double size[3] = {(double)g->nx, (double)g->ny, (double)g->nz};
    double dd[3] = {d[0], d[1], d[2]}, pos[3] = {pos32[0], pos32[1], pos32[2]};
    double len = sqrt((dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2]);
    int32_t v[3], st[3];
    double delta[3], side[3];
    for (int a = 0; a < 3; ++a) {
        double m = glsl_min64(pos[a], size[a] - 1.0);
        v[a] = (int32_t)floor(m);
        double sg = dd[a] > 0.0 ? 1.0 : (dd[a] < 0.0 ? -1.0 : 0.0);
        st[a] = (int32_t)sg;
        delta[a] = fabs(len / dd[a]);
        side[a] = ((sg * ((double)v[a] - pos[a]) + sg * 0.5) + 0.5) * delta[a];
    }
    uint32_t max_steps = (uint32_t)(g->nx + g->ny + g->nz), steps = 0;
    int last = 0, tie = 0, hit = 0;
    while (steps < max_steps && v[0] >= 0 && v[1] >= 0 && v[2] >= 0 && v[0] < isize[0] &&
           v[1] < isize[1] && v[2] < isize[2]) {
        if (voxel_occupied(g, v[0], v[1], v[2])) {
            hit = 1;
            break;
        }
        double mnx = glsl_min64(side[1], side[2]);
        double mny = glsl_min64(side[2], side[0]);
        double mnz = glsl_min64(side[0], side[1]);
        int bx = side[0] <= mnx, by = side[1] <= mny, bz = side[2] <= mnz;
        if (bx) side[0] = side[0] + delta[0];
        if (by) side[1] = side[1] + delta[1];
        if (bz) side[2] = side[2] + delta[2];
        if (bx) v[0] += st[0];
        if (by) v[1] += st[1];
        if (bz) v[2] += st[2];
        last = bx | (by << 1) | (bz << 2);
        if (bx + by + bz > 1) tie = 1;
        ++steps;
    }
    out->tie = tie;
    if (!hit) return;
    out->hit = 1;
    out->v[0] = v[0];
    out->v[1] = v[1];
    out->v[2] = v[2];
    if (steps > 0) {
        int a = (last & 1) ? 0 : ((last & 2) ? 1 : 2);
        double plane = (double)(st[a] > 0 ? v[a] : v[a] + 1);
        out->t = (plane - (double)o[a]) / dd[a];
        out->face = face_code(a, st[a] < 0);
    } else if (kind == 1) {
        int a = entry_axis;
        double plane = d[a] > 0.0f ? 0.0 : size[a];
        out->t = (plane - (double)o[a]) / dd[a];
        out->face = face_code(a, d[a] < 0.0f);
    } else {
        out->t = 0.0;
        out->face = 0;
    }
}

void vto_trace_entry_points(const vto_grid* g, uint64_t n, const float* mp, const float* s,
                            int32_t* out) {
    const float size[3] = {(float)g->nx, (float)g->ny, (float)g->nz};
    for (uint64_t i = 0; i < n; ++i) {
        const float* v = s + 3 * i;
        const float len = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
        float d[3], pos[3];
        for (int a = 0; a < 3; ++a) {
            d[a] = v[a] / len;
            pos[a] = (mp[3 * i + a] + 0.5f) * size[a];
        }
        vto_dda_out r;
        vto_dda_f32(g, pos, d, &r, NULL);
        int32_t* o = out + 5 * i;
        o[0] = r.hit;
        o[1] = r.v[0];
        o[2] = r.v[1];
        o[3] = r.v[2];
        o[4] = (int32_t)(r.steps + (r.hit ? 1u : 0u));
    }
}

void vto_raygen(const vto_camera* c, uint32_t px, uint32_t py, float jx, float jy, float o[3],
                float d[3]) {
    const float inv_w2 = 2.0f / (float)c->width;
    const float inv_h2 = 2.0f / (float)c->height;
    const float fx = (float)px + jx;
    const float fy = (float)py + jy;
    const float sx = fx * inv_w2 - 1.0f;
    const float sy = 1.0f - fy * inv_h2;
    float r[3];
    for (int a = 0; a < 3; ++a) r[a] = (c->forward[a] + sx * c->right[a]) + sy * c->up[a];
    const float len = sqrtf((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
    for (int a = 0; a < 3; ++a) {
        d[a] = r[a] / len;
        o[a] = c->origin[a];
    }
}

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void vto_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void vto_jitter(uint32_t seed, uint32_t view, uint32_t px, uint32_t py, uint32_t s, float* jx,
                float* jy) {
    const uint32_t ctr[4] = {px, py, s, view};
    const uint32_t key[2] = {seed, 0x56544752u};
    uint32_t r[4];
    vto_philox4x32_10(ctr, key, r);
    *jx = (float)(r[0] >> 8) * 0x1p-24f;
    *jy = (float)(r[1] >> 8) * 0x1p-24f;
}

static void shade_from_ray(const vto_grid* g, const vto_light* light, const float o[3],
                           const float d[3], vto_hit* out, vto_stats* stats) {
    vto_trace_ray_f32(g, o, d, out, stats);
    if (!(out->face & VTO_FLAG_HIT)) {
        out->rgba = VTO_SKY_RGBA;
        return;
    }
    if (stats) stats->hits++;
    if (!light) return;
    const int face = out->face & 7;
    if (face == 0) return; /* origin inside the hit voxel: no normal, colour unshaded */
    const int a = (face - 1) / 2;
    const int npos = (face & 1) != 0;
    const float ndl = npos ? light->dir[a] : -light->dir[a];
    float vis = 1.0f;
    if (ndl > 0.0f && light->shadows) {
        const int32_t hv[3] = {out->x, out->y, out->z};
        const float plane = (float)(npos ? hv[a] + 1 : hv[a]);
        float so[3];
        for (int b = 0; b < 3; ++b) so[b] = o[b] + out->t * d[b];
        so[a] = npos ? plane + 0.015625f : plane - 0.015625f;
        vto_hit sh;
        vto_trace_ray_f32(g, so, light->dir, &sh, stats);
        if (stats) stats->shadow_rays++;
        out->face |= VTO_FLAG_SHADOW_RAY;
        if (sh.face & VTO_FLAG_HIT) {
            vis = 0.0f;
            out->face |= VTO_FLAG_SHADOWED;
        }
    }
    const float lam = ndl > 0.0f ? ndl : 0.0f;
    const float k = light->ambient + (1.0f - light->ambient) * (lam * vis);
    uint32_t base = out->rgba, res = base & 0xFF000000u;
    for (int c = 0; c < 3; ++c) {
        float v = (float)((base >> (8 * c)) & 0xFFu) * k + 0.5f;
        uint32_t q = v >= 255.0f ? 255u : (v <= 0.0f ? 0u : (uint32_t)v);
        res |= q << (8 * c);
    }
    out->rgba = res;
}

void vto_shade_sample(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                      uint32_t px, uint32_t py, float jx, float jy, vto_hit* out,
                      vto_stats* stats) {
    float o[3], d[3];
    vto_raygen(cam, px, py, jx, jy, o, d);
    shade_from_ray(g, light, o, d, out, stats);
}

/* The shadow-ray origin below is shade_from_ray's, from the record's voxel, face and t. */
uint64_t vto_frame_rays(const vto_camera* cam, const vto_light* light, const vto_hit* hits,
                        float* camera_rays, float* shadow_rays) {
    uint64_t ns = 0;
    for (uint32_t py = 0; py < cam->height; ++py) {
        for (uint32_t px = 0; px < cam->width; ++px) {
            const uint64_t p = (uint64_t)py * cam->width + px;
            float* r = camera_rays + 6 * p;
            vto_raygen(cam, px, py, 0.5f, 0.5f, r, r + 3);
            const vto_hit* h = &hits[p];
            if (!light || !(h->face & VTO_FLAG_SHADOW_RAY)) continue;
            const int face = h->face & 7;
            const int a = (face - 1) / 2;
            const int npos = (face & 1) != 0;
            const int32_t hv[3] = {h->x, h->y, h->z};
            const float plane = (float)(npos ? hv[a] + 1 : hv[a]);
            float* s = shadow_rays + 6 * ns;
            for (int b = 0; b < 3; ++b) s[b] = r[b] + h->t * r[3 + b];
            s[a] = npos ? plane + 0.015625f : plane - 0.015625f;
            for (int b = 0; b < 3; ++b) s[3 + b] = light->dir[b];
            ++ns;
        }
    }
    return ns;
}

/* ------------------------------------------------------------------ path tracing */

/* The library's path-tracing estimator (vt_path.cu's header states it; vtrace itself has none). */
static int sphere_sample(uint32_t seed, uint32_t px, uint32_t py, uint32_t s, uint32_t bounce,
                         float u[3]) {
    for (uint32_t t = 0; t < 16; ++t) {
        const uint32_t ctr[4] = {px, py, s, (bounce << 8) | t};
        const uint32_t key[2] = {seed, 0x50415448u};
        uint32_t r[4];
        vto_philox4x32_10(ctr, key, r);
        float p[3];
        for (int k = 0; k < 3; ++k) p[k] = (float)(r[k] >> 8) * 0x1p-23f - 1.0f;
        const float r2 = (p[0] * p[0] + p[1] * p[1]) + p[2] * p[2];
        if (r2 <= 1.0f && r2 > 0x1p-20f) {
            const float l = sqrtf(r2);
            for (int k = 0; k < 3; ++k) u[k] = p[k] / l;
            return 1;
        }
    }
    return 0;
}

void vto_path_pixel(const vto_grid* g, const vto_camera* cam, const vto_path_params* P,
                    uint32_t px, uint32_t py, float out[3], uint64_t* rays) {
    int sun_on = 0;
    for (int c = 0; c < 3; ++c)
        if (P->sun[c] > 0.0f) sun_on = 1;
    float sum[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t s = 0; s < P->spp; ++s) {
        float jx, jy, o[3], d[3];
        vto_jitter(P->seed, 0u, px, py, s, &jx, &jy);
        vto_raygen(cam, px, py, jx, jy, o, d);
        float T[3] = {1.0f, 1.0f, 1.0f}, L[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t b = 0;; ++b) {
            vto_hit h;
            vto_trace_ray_f32(g, o, d, &h, NULL);
            ++*rays;
            if (!(h.face & VTO_FLAG_HIT)) {
                for (int c = 0; c < 3; ++c) L[c] = L[c] + T[c] * P->sky[c];
                break;
            }
            const int face = h.face & 7;
            if (face == 0) break;
            for (int c = 0; c < 3; ++c) T[c] = T[c] * ((float)((h.rgba >> (8 * c)) & 0xFFu) / 255.0f);
            const int a = (face - 1) / 2;
            const int npos = (face & 1) != 0;
            const int32_t hv[3] = {h.x, h.y, h.z};
            const float plane = (float)(npos ? hv[a] + 1 : hv[a]);
            float so[3];
            for (int k = 0; k < 3; ++k) so[k] = o[k] + h.t * d[k];
            so[a] = npos ? plane + 0.015625f : plane - 0.015625f;
            if (sun_on) {
                const float ndl = npos ? P->sun_dir[a] : -P->sun_dir[a];
                if (ndl > 0.0f) {
                    vto_hit sh;
                    vto_trace_ray_f32(g, so, P->sun_dir, &sh, NULL);
                    ++*rays;
                    if (!(sh.face & VTO_FLAG_HIT))
                        for (int c = 0; c < 3; ++c) L[c] = L[c] + (T[c] * P->sun[c]) * ndl;
                }
            }
            if (b >= P->max_bounces) break;
            float n[3] = {0.0f, 0.0f, 0.0f}, u[3], nd[3];
            n[a] = npos ? 1.0f : -1.0f;
            if (sphere_sample(P->seed, px, py, s, b, u)) {
                for (int k = 0; k < 3; ++k) nd[k] = n[k] + u[k];
                const float l = sqrtf((nd[0] * nd[0] + nd[1] * nd[1]) + nd[2] * nd[2]);
                if (l > 1e-6f)
                    for (int k = 0; k < 3; ++k) nd[k] = nd[k] / l;
                else
                    for (int k = 0; k < 3; ++k) nd[k] = n[k];
            } else {
                for (int k = 0; k < 3; ++k) nd[k] = n[k];
            }
            for (int k = 0; k < 3; ++k) {
                o[k] = so[k];
                d[k] = nd[k];
            }
        }
        for (int c = 0; c < 3; ++c) sum[c] = sum[c] + L[c];
    }
    const float n = (float)P->spp;
    for (int c = 0; c < 3; ++c) out[c] = sum[c] / n;
}

/* ------------------------------------------------------------------ threading */

int vto_hardware_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

typedef struct job {
    int kind; /* 0 render rows, 1 rays f32, 2 rays f64, 3 view */
    const vto_grid* g;
    const vto_camera* cam;
    const vto_light* light;
    const float* rays;
    vto_hit* hits;
    vto_hit64* hits64;
    uint32_t spp, seed, view;
    uint64_t begin, end; /* pixels (kind 0/3) or rays */
    uint32_t row_offset;
    vto_stats stats;
    int want_stats;
    const vto_path_params* path;
    float* path_out; /* width * height * 4 floats */
    uint64_t path_rays;
} job;

static void* run_job(void* arg) {
    job* j = (job*)arg;
    vto_stats* st = j->want_stats ? &j->stats : NULL;
    if (j->kind == 0) { /* begin/end: pixel indices y * width + x */
        const uint32_t w = j->cam->width;
        for (uint64_t p = j->begin; p < j->end; ++p) {
            const uint32_t y = (uint32_t)(p / w), x = (uint32_t)(p % w);
            vto_shade_sample(j->g, j->cam, j->light, x, y, 0.5f, 0.5f,
                             &j->hits[p - (uint64_t)j->row_offset * w], st);
        }
    } else if (j->kind == 1) {
        for (uint64_t i = j->begin; i < j->end; ++i) {
            const float* r = j->rays + 6 * i;
            vto_trace_ray_f32(j->g, r, r + 3, &j->hits[i], st);
        }
    } else if (j->kind == 2) {
        for (uint64_t i = j->begin; i < j->end; ++i) {
            const float* r = j->rays + 6 * i;
            vto_trace_ray_f64(j->g, r, r + 3, &j->hits64[i]);
        }
    } else if (j->kind == 4) { /* path tracing, begin/end: pixel indices */
        const uint32_t w = j->cam->width;
        for (uint64_t p = j->begin; p < j->end; ++p) {
            const uint32_t y = (uint32_t)(p / w), x = (uint32_t)(p % w);
            float* o = j->path_out + 4 * p;
            vto_path_pixel(j->g, j->cam, j->path, x, y, o, &j->path_rays);
            o[3] = 1.0f;
        }
    } else { /* begin/end: pixel indices */
        const uint32_t w = j->cam->width;
        for (uint64_t p = j->begin; p < j->end; ++p) {
            const uint32_t y = (uint32_t)(p / w), x = (uint32_t)(p % w);
            for (uint32_t s = 0; s < j->spp; ++s) {
                float jx, jy;
                vto_jitter(j->seed, j->view, x, y, s, &jx, &jy);
                vto_shade_sample(j->g, j->cam, j->light, x, y, jx, jy, &j->hits[p * j->spp + s],
                                 st);
            }
        }
    }
    return NULL;
}

typedef struct lane {
    job* jobs;
    uint64_t n, first, stride;
} lane;

static void* lane_main(void* arg) {
    lane* l = (lane*)arg;
    for (uint64_t c = l->first; c < l->n; c += l->stride) run_job(&l->jobs[c]);
    return NULL;
}

/* Splits [begin, end) into chunks of ~1/16 of a thread's share, handed out round-robin. */
static void run_parallel(job* proto, uint64_t begin, uint64_t end, int threads, vto_stats* stats) {
    if (end <= begin) return;
    if (threads <= 0) threads = vto_hardware_threads();
    if ((uint64_t)threads > end - begin) threads = (int)(end - begin);
    if (threads < 1) threads = 1;
    const uint64_t total = end - begin;
    uint64_t chunk = total / ((uint64_t)threads * 16);
    if (chunk == 0) chunk = 1;
    const uint64_t nchunks = (total + chunk - 1) / chunk;
    job* jobs = (job*)calloc((size_t)nchunks, sizeof(job));
    pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    lane* lanes = (lane*)calloc((size_t)threads, sizeof(lane));
    for (uint64_t c = 0; c < nchunks; ++c) {
        jobs[c] = *proto;
        memset(&jobs[c].stats, 0, sizeof(vto_stats));
        jobs[c].begin = begin + c * chunk;
        jobs[c].end = jobs[c].begin + chunk < end ? jobs[c].begin + chunk : end;
    }
    for (int t = 0; t < threads; ++t) {
        lanes[t].jobs = jobs;
        lanes[t].n = nchunks;
        lanes[t].first = (uint64_t)t;
        lanes[t].stride = (uint64_t)threads;
    }
    if (threads == 1) {
        lane_main(&lanes[0]);
    } else {
        for (int t = 0; t < threads; ++t) pthread_create(&tids[t], NULL, lane_main, &lanes[t]);
        for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
    }
    if (stats) {
        for (uint64_t c = 0; c < nchunks; ++c) {
            const vto_stats* s = &jobs[c].stats;
            stats->rays += s->rays;
            stats->shadow_rays += s->shadow_rays;
            stats->hits += s->hits;
            stats->steps += s->steps;
            stats->bricks_entered += s->bricks_entered;
            stats->nonempty_bricks_entered += s->nonempty_bricks_entered;
            stats->voxels_tested += s->voxels_tested;
            stats->ties += s->ties;
        }
    }
    free(lanes);
    free(tids);
    proto->path_rays = 0;
    for (uint64_t c = 0; c < nchunks; ++c) proto->path_rays += jobs[c].path_rays;
    free(jobs);
}

void vto_render_rows(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                     uint32_t row0, uint32_t row1, vto_hit* hits, int threads, vto_stats* stats) {
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 0;
    p.g = g;
    p.cam = cam;
    p.light = light;
    p.hits = hits;
    p.row_offset = row0;
    p.want_stats = stats != NULL;
    run_parallel(&p, (uint64_t)row0 * cam->width, (uint64_t)row1 * cam->width, threads, stats);
}

void vto_render(const vto_grid* g, const vto_camera* cam, const vto_light* light, vto_hit* hits,
                int threads, vto_stats* stats) {
    vto_render_rows(g, cam, light, 0, cam->height, hits, threads, stats);
}

void vto_render_view(const vto_grid* g, const vto_camera* cam, const vto_light* light,
                     uint32_t spp, uint32_t seed, uint32_t view, vto_hit* hits, int threads,
                     vto_stats* stats) {
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 3;
    p.g = g;
    p.cam = cam;
    p.light = light;
    p.hits = hits;
    p.spp = spp;
    p.seed = seed;
    p.view = view;
    p.want_stats = stats != NULL;
    run_parallel(&p, 0, (uint64_t)cam->height * cam->width, threads, stats);
}

void vto_trace_rays(const vto_grid* g, const float* rays, uint64_t n, vto_hit* hits, int threads,
                    vto_stats* stats) {
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 1;
    p.g = g;
    p.rays = rays;
    p.hits = hits;
    p.want_stats = stats != NULL;
    run_parallel(&p, 0, n, threads, stats);
}

void vto_trace_rays_f64(const vto_grid* g, const float* rays, uint64_t n, vto_hit64* hits,
                        int threads) {
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 2;
    p.g = g;
    p.rays = rays;
    p.hits64 = hits;
    run_parallel(&p, 0, n, threads, NULL);
}

/* ------------------------------------------------------------------ reference-compatible frame
 *
 * Restates libvtrace's headless render_tick: the reference rasterises one cube per instance and
 * marches from each front-face fragment (trace.frag:41-90), depth-tests LESS on the cube face
 * (lib/pipeline.c:146-152) and blends SRC_ALPHA / ONE_MINUS_SRC_ALPHA into an sRGB target
 * cleared to (0.53, 0.81, 0.92, 1) (lib/command.c:57-60, lib/pipeline.c:129-137).  Per pixel, in
 * draw order: slab entry into [-0.5,0.5]^3 along inverse(model) * view ray (skipped when the
 * camera is inside), DDA from (entry + 0.5) * size, blend on a hit nearer than the depth so far.
 * Matrix preparation is in binary64 with the same cofactor expansion as the library. */

static double srgb_to_linear_d(double c) {
    return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
}

static int invert4d(const double* a, double* inv) {
    double r[16];
    r[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    r[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    r[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    r[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    r[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    r[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    r[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    r[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    r[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    r[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    r[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    r[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    r[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    r[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    r[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    r[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const double det = a[0] * r[0] + a[1] * r[4] + a[2] * r[8] + a[3] * r[12];
    if (!(det != 0.0) || !isfinite(det)) return 0;
    for (int i = 0; i < 16; ++i) inv[i] = r[i] / det;
    return 1;
}

static void mul4d(const double* a, const double* b, double* c) {
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[col * 4 + k];
            c[col * 4 + row] = s;
        }
}

typedef struct compat_inst {
    float minv[12];
    int32_t texture;
} compat_inst;

typedef struct compat_job {
    const vto_grid* grids;
    const compat_inst* inst;
    uint32_t ninst;
    float dirm[12], cam[3];
    int32_t width, height;
    float decode[256], thresh[255];
    uint8_t* out;
    uint64_t begin, end;
} compat_job;

static uint32_t srgb_encode_t(const float* thresh, float v) {
    uint32_t lo = 0, hi = 255;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (thresh[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

static void compat_pixel(const compat_job* f, int32_t px, int32_t py) {
    const float inv_w = 2.0f / (float)f->width;
    const float xn = ((float)px + 0.5f) * inv_w - 1.0f;
    const float yn = ((float)py + 0.5f) * inv_w - 1.0f;
    float dw[3];
    for (int r = 0; r < 3; ++r)
        dw[r] = ((f->dirm[4 * r] * xn + f->dirm[4 * r + 1] * yn) + f->dirm[4 * r + 2]) + f->dirm[4 * r + 3];
    const float len = sqrtf((dw[0] * dw[0] + dw[1] * dw[1]) + dw[2] * dw[2]);
    for (int r = 0; r < 3; ++r) dw[r] = dw[r] / len;
    uint32_t col[3] = {VTO_SKY_RGBA & 0xFFu, (VTO_SKY_RGBA >> 8) & 0xFFu, (VTO_SKY_RGBA >> 16) & 0xFFu};
    uint32_t ca = VTO_SKY_RGBA >> 24;
    float depth = INFINITY;
    for (uint32_t i = 0; i < f->ninst; ++i) {
        const compat_inst* I = &f->inst[i];
        const vto_grid* g = &f->grids[I->texture];
        float om[3], dm[3];
        for (int r = 0; r < 3; ++r) {
            const float* m = I->minv + 4 * r;
            om[r] = ((m[0] * f->cam[0] + m[1] * f->cam[1]) + m[2] * f->cam[2]) + m[3];
            dm[r] = (m[0] * dw[0] + m[1] * dw[1]) + m[2] * dw[2];
        }
        float tn = -INFINITY, tf = INFINITY;
        int ax = -1, miss = 0;
        for (int a = 0; a < 3; ++a) {
            if (dm[a] == 0.0f) {
                if (om[a] < -0.5f || om[a] > 0.5f) miss = 1;
                continue;
            }
            const float ta = (-0.5f - om[a]) / dm[a];
            const float tb = (0.5f - om[a]) / dm[a];
            const float lo = ta < tb ? ta : tb, hi = ta < tb ? tb : ta;
            if (lo > tn) {
                tn = lo;
                ax = a;
            }
            if (hi < tf) tf = hi;
        }
        if (miss || tn > tf || tf < 0.0f || tn <= 0.0f) continue;
        if (!(tn < depth)) continue;
        const float size[3] = {(float)g->nx, (float)g->ny, (float)g->nz};
        float pos[3];
        for (int b = 0; b < 3; ++b) {
            float mp = om[b] + tn * dm[b];
            mp = mp < -0.5f ? -0.5f : (mp > 0.5f ? 0.5f : mp);
            if (b == ax) mp = dm[b] > 0.0f ? -0.5f : 0.5f;
            pos[b] = (mp + 0.5f) * size[b];
        }
        vto_dda_out r;
        vto_dda_f32(g, pos, dm, &r, NULL);
        if (!r.hit) continue;
        const uint32_t tex = voxel_rgba(g, r.v[0], r.v[1], r.v[2]);
        const float a = (float)(tex >> 24) / 255.0f;
        const float ia = 1.0f - a;
        for (int c = 0; c < 3; ++c) {
            const float v = f->decode[(tex >> (8 * c)) & 0xFFu] * a + f->decode[col[c]] * ia;
            col[c] = srgb_encode_t(f->thresh, v);
        }
        ca = tex >> 24;
        depth = tn;
    }
    uint8_t* o = f->out + 4 * ((size_t)py * f->width + px);
    o[0] = (uint8_t)col[0];
    o[1] = (uint8_t)col[1];
    o[2] = (uint8_t)col[2];
    o[3] = (uint8_t)ca;
}

static void* compat_worker(void* arg) {
    compat_job* j = (compat_job*)arg;
    for (uint64_t p = j->begin; p < j->end; ++p)
        compat_pixel(j, (int32_t)(p % (uint64_t)j->width), (int32_t)(p / (uint64_t)j->width));
    return NULL;
}

int vto_compat_render(const vto_grid* grids, uint32_t ngrids, const float* instances,
                      uint32_t ninst, const float P[16], const float C[16], int32_t width,
                      int32_t height, uint8_t* rgba, int threads) {
    double p[16], cm[16], c0[16], ip[16], ic[16], ic0[16], dm[16];
    for (int i = 0; i < 16; ++i) {
        p[i] = P[i];
        cm[i] = C[i];
        c0[i] = C[i];
    }
    c0[12] = c0[13] = c0[14] = 0.0;
    if (!invert4d(p, ip) || !invert4d(cm, ic) || !invert4d(c0, ic0)) return -1;
    mul4d(ic0, ip, dm);
    compat_job f;
    memset(&f, 0, sizeof(f));
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) f.dirm[4 * r + k] = (float)dm[k * 4 + r];
    for (int r = 0; r < 3; ++r) f.cam[r] = (float)ic[12 + r];
    f.width = width;
    f.height = height;
    for (int i = 0; i < 256; ++i) f.decode[i] = (float)srgb_to_linear_d(i / 255.0);
    for (int k = 0; k < 255; ++k) f.thresh[k] = (float)srgb_to_linear_d((k + 0.5) / 255.0);
    compat_inst* inst = (compat_inst*)calloc(ninst ? ninst : 1, sizeof(compat_inst));
    uint32_t n = 0;
    for (uint32_t i = 0; i < ninst; ++i) {
        const float* m = instances + 16 * i;
        int32_t tid;
        memcpy(&tid, &m[15], 4);
        if (tid < 0 || (uint32_t)tid >= ngrids) continue;
        double md[16], mi[16];
        for (int k = 0; k < 16; ++k) md[k] = m[k];
        md[15] = 1.0;
        if (!invert4d(md, mi)) continue;
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 4; ++k) inst[n].minv[4 * r + k] = (float)mi[k * 4 + r];
        inst[n].texture = tid;
        ++n;
    }
    f.grids = grids;
    f.inst = inst;
    f.ninst = n;
    f.out = rgba;
    if (threads <= 0) threads = vto_hardware_threads();
    const uint64_t total = (uint64_t)width * height;
    compat_job* jobs = (compat_job*)calloc((size_t)threads, sizeof(compat_job));
    pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) {
        jobs[t] = f;
        jobs[t].begin = total * (uint64_t)t / (uint64_t)threads;
        jobs[t].end = total * (uint64_t)(t + 1) / (uint64_t)threads;
        pthread_create(&tids[t], NULL, compat_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
    free(tids);
    free(jobs);
    free(inst);
    return 0;
}

void vto_path_trace(const vto_grid* g, const vto_camera* cam, const vto_path_params* params,
                    uint32_t row0, uint32_t row1, float* out, int threads, uint64_t* rays) {
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 4;
    p.g = g;
    p.cam = cam;
    p.path = params;
    p.path_out = out - 4 * (uint64_t)row0 * cam->width; /* out holds rows row0..row1-1 */
    run_parallel(&p, (uint64_t)row0 * cam->width, (uint64_t)row1 * cam->width, threads, NULL);
    if (rays) *rays = p.path_rays;
}
