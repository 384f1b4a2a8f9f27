/* A C host driving libvtrace through the seven entry points vtrace's renderer binds
 * (src/render.rs:110-128), in the order its Rust host calls them (src/render.rs:184-320):
 * entry, add_texture per texture, start/end_update_instances, render_tick per frame, cleanup.
 *
 * Writes to argv[1]: the perspective and camera matrices, the instances and the textures it used
 * and the last frame read back with vt_framebuffer_download, so that a test can check the frame
 * against the reference frame restated on the CPU.  Exit status 0 on success. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vtrace.h"

#define NTEX 2
static const uint32_t dims[NTEX][3] = {{16, 16, 16}, {12, 20, 10}};

static uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

/* glm::perspective and glm::look_at (src/render.rs:208-214), column-major. */
static void perspective(float fov, float aspect, float near, float far, float m[16]) {
    const double f = 1.0 / tan(fov / 2.0);
    memset(m, 0, 16 * sizeof(float));
    m[0] = (float)(f / aspect);
    m[5] = (float)f;
    m[10] = (float)((far + near) / (near - far));
    m[11] = -1.0f;
    m[14] = (float)(2.0 * far * near / (near - far));
}

static void look_at(const double e[3], const double c[3], float m[16]) {
    double f[3] = {c[0] - e[0], c[1] - e[1], c[2] - e[2]};
    double n = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (int i = 0; i < 3; ++i) f[i] /= n;
    double s[3] = {f[1] * 0.0 - f[2] * 1.0, f[2] * 0.0 - f[0] * 0.0, f[0] * 1.0 - f[1] * 0.0};
    n = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (int i = 0; i < 3; ++i) s[i] /= n;
    const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    memset(m, 0, 16 * sizeof(float));
    for (int i = 0; i < 3; ++i) {
        m[4 * i + 0] = (float)s[i];
        m[4 * i + 1] = (float)u[i];
        m[4 * i + 2] = (float)-f[i];
    }
    m[12] = (float)-(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]);
    m[13] = (float)-(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]);
    m[14] = (float)(f[0] * e[0] + f[1] * e[1] + f[2] * e[2]);
    m[15] = 1.0f;
}

/* translate * scale, texture id in the bits of element [3][3] (trace.vert:38-40) */
static void instance(float tx, float ty, float tz, float scale, int32_t tid, float m[16]) {
    memset(m, 0, 16 * sizeof(float));
    m[0] = m[5] = m[10] = scale;
    m[12] = tx;
    m[13] = ty;
    m[14] = tz;
    memcpy(&m[15], &tid, 4);
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: replay OUT\n");
        return 2;
    }
    if (entry() != 0) {
        fprintf(stderr, "entry failed: %s\n", vt_last_error());
        return 1;
    }
    uint8_t* tex[NTEX];
    for (int t = 0; t < NTEX; ++t) {
        const size_t n = (size_t)dims[t][0] * dims[t][1] * dims[t][2];
        tex[t] = (uint8_t*)calloc(n, 4);
        for (size_t i = 0; i < n; ++i) {
            const uint32_t h = hash32((uint32_t)i * 2654435761U + (uint32_t)t);
            if ((h & 15U) < 3U) {
                const uint32_t c = hash32(h) | 0xFF000000U;
                memcpy(tex[t] + 4 * i, &c, 4);
            }
        }
        if (add_texture(tex[t], dims[t][0], dims[t][1], dims[t][2]) != t) {
            fprintf(stderr, "add_texture failed: %s\n", vt_last_error());
            return 1;
        }
    }
    enum { NINST = 5 };
    float inst[NINST][16];
    instance(0.0f, 0.0f, -6.0f, 4.0f, 0, inst[0]);
    instance(3.0f, -1.0f, -9.0f, 3.0f, 1, inst[1]);
    instance(-3.5f, 1.5f, -11.0f, 5.0f, 0, inst[2]);
    instance(0.5f, 2.5f, -14.0f, 6.0f, 1, inst[3]);
    instance(0.0f, 0.0f, 0.0f, 100.0f, 1, inst[4]); /* camera inside: not drawn */
    float* p = start_update_instances(NINST);
    if (!p) return 1;
    memcpy(p, inst, sizeof(inst));
    if (end_update_instances(NINST) != 0) return 1;
    float P[16], C[16];
    perspective(80.0f / 180.0f * 3.1415926f, 1.0f, 0.01f, 10000.0f, P); /* src/render.rs:190 */
    render_tick_info info = {P, C};
    int32_t w = 0, h = 0;
    for (int frame = 0; frame < 3; ++frame) { /* the camera moves between frames */
        const double eye[3] = {0.3 * frame, 0.6, 2.0 - 0.5 * frame}, at[3] = {0.0, 0.0, -8.0};
        look_at(eye, at, C);
        if (render_tick(&w, &h, &info) != 0) {
            fprintf(stderr, "render_tick failed: %s\n", vt_last_error());
            return 1;
        }
    }
    const user_input* in = get_input_data_pointer();
    if (!in || in->keys[0] != 0) return 1;
    uint8_t* fb = (uint8_t*)malloc((size_t)w * h * 4);
    if (vt_framebuffer_download(fb, (uint64_t)w * h * 4) != VT_OK) return 1;
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 1;
    const int32_t hdr[3] = {w, h, NINST};
    fwrite(hdr, sizeof(hdr), 1, f);
    fwrite(P, sizeof(P), 1, f);
    fwrite(C, sizeof(C), 1, f);
    fwrite(inst, sizeof(inst), 1, f);
    for (int t = 0; t < NTEX; ++t)
        fwrite(tex[t], 4, (size_t)dims[t][0] * dims[t][1] * dims[t][2], f);
    fwrite(fb, 4, (size_t)w * h, f);
    fclose(f);
    cleanup();
    if (render_tick(&w, &h, &info) != -1) return 1; /* after cleanup */
    printf("ok %dx%d\n", w, h);
    return 0;
}
