// vt_compat.cu — the seven C entry points vtrace's Rust host binds (src/render.rs:110-128),
// headless on CUDA.
//
// A frame of the reference (lib/entry.c:150-248) rasterises one unit cube per instance
// (lib/command.c:102, trace.vert:32-47) with back-face culling, and the fragment shader marches
// the instance's texture from the front-face point along the view ray (trace.frag:41-90).  The
// depth test (LESS, lib/pipeline.c:146-152) uses the cube-face depth, a discarded fragment writes
// nothing, and colour blends SRC_ALPHA / ONE_MINUS_SRC_ALPHA into an sRGB target cleared to
// (0.53, 0.81, 0.92, 1) (lib/command.c:57-60, lib/pipeline.c:129-137).
//
// render_tick restates that per pixel without rasterisation: for each instance in draw order it
// intersects the pixel's view ray with the instance cube [-0.5,0.5]^3 in model space (the
// front-face entry point, skipped when the camera is inside the cube, as culling would), runs the
// reference DDA from (entry + 0.5) * size along inverse(model) * dir, and, on a hit nearer than
// the depth so far, blends the texel into the 8-bit sRGB pixel.  Depth order along one pixel ray
// is the order of the entry parameter t, so t stands in for the face depth.  The viewport height
// equals the framebuffer width as in lib/command.c:81.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "vt_api_internal.h"
#include "vt_device.cuh"
#include "vt_internal.h"

namespace vt {

constexpr uint32_t kMaxTextures = 65536;  // lib/common.h:35

struct CompatInstance {
    float minv[12];  // inverse(model), rows 0..2 of the 4x4 (row-major)
    int32_t texture;
    int32_t pad[3];
};

struct CompatFrame {
    float dirm[12];  // inverse(centered camera) * inverse(projection), rows 0..2
    float cam[3];
    int32_t width, height;
};

// sRGB transfer tables: decode of the 256 byte values, and the 255 linear thresholds at which the
// encoded byte steps up (linear value of (k + 0.5) / 255 in sRGB), both computed in double.
struct SrgbTables {
    float decode[256];
    float thresh[255];
};

static double srgb_to_linear(double c) {
    return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
}

__constant__ SrgbTables c_srgb;

__device__ __forceinline__ uint32_t srgb_encode(float v) {
    // number of thresholds <= v, by binary search over the 255 sorted thresholds
    uint32_t lo = 0, hi = 255;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (c_srgb.thresh[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) compat_kernel(const GridView* __restrict__ views,
                                                     const CompatInstance* __restrict__ inst,
                                                     int32_t ninst, CompatFrame f,
                                                     uchar4* __restrict__ fb) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int32_t px = (int32_t)(blockIdx.x * 16 + (warp & 1u) * 8u + (lane & 7u));
    const int32_t py = (int32_t)(blockIdx.y * 16 + (warp >> 1) * 4u + (lane >> 3));
    if (px >= f.width || py >= f.height) return;
    const float inv_w = __fdiv_rn(2.0f, __int2float_rn(f.width));
    const float xn = __fsub_rn(__fmul_rn(__fadd_rn(__int2float_rn(px), 0.5f), inv_w), 1.0f);
    const float yn = __fsub_rn(__fmul_rn(__fadd_rn(__int2float_rn(py), 0.5f), inv_w), 1.0f);
    float dw[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        dw[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(f.dirm[4 * r], xn), __fmul_rn(f.dirm[4 * r + 1], yn)),
                                    f.dirm[4 * r + 2]),
                          f.dirm[4 * r + 3]);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dw[0], dw[0]), __fmul_rn(dw[1], dw[1])),
                                           __fmul_rn(dw[2], dw[2])));
#pragma unroll
    for (int r = 0; r < 3; ++r) dw[r] = __fdiv_rn(dw[r], len);
    uint32_t cr = VT_SKY_RGBA & 0xFFu, cg = (VT_SKY_RGBA >> 8) & 0xFFu,
             cb = (VT_SKY_RGBA >> 16) & 0xFFu, ca = VT_SKY_RGBA >> 24;
    float depth = INFINITY;
    for (int32_t i = 0; i < ninst; ++i) {
        const CompatInstance& I = inst[i];
        const GridView g = views[I.texture];
        float om[3], dm[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float* m = I.minv + 4 * r;
            om[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], f.cam[0]), __fmul_rn(m[1], f.cam[1])),
                                        __fmul_rn(m[2], f.cam[2])),
                              m[3]);
            dm[r] = __fadd_rn(__fadd_rn(__fmul_rn(m[0], dw[0]), __fmul_rn(m[1], dw[1])), __fmul_rn(m[2], dw[2]));
        }
        // slab test against the unit cube [-0.5, 0.5]^3
        float tn = -INFINITY, tf = INFINITY;
        int ax = -1;
        bool miss = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (dm[a] == 0.0f) {
                if (om[a] < -0.5f || om[a] > 0.5f) miss = true;
                continue;
            }
            const float ta = __fdiv_rn(__fsub_rn(-0.5f, om[a]), dm[a]);
            const float tb = __fdiv_rn(__fsub_rn(0.5f, om[a]), dm[a]);
            const float lo = ta < tb ? ta : tb, hi = ta < tb ? tb : ta;
            if (lo > tn) {
                tn = lo;
                ax = a;
            }
            if (hi < tf) tf = hi;
        }
        // camera inside the cube: only back faces face it, and those are culled
        if (miss || tn > tf || tf < 0.0f || tn <= 0.0f) continue;
        if (!(tn < depth)) continue;  // depth test LESS against the nearest hit so far
        const float size[3] = {__int2float_rn(g.nx), __int2float_rn(g.ny), __int2float_rn(g.nz)};
        float pos[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float mp = __fadd_rn(om[b], __fmul_rn(tn, dm[b]));
            mp = mp < -0.5f ? -0.5f : (mp > 0.5f ? 0.5f : mp);
            if (b == ax) mp = dm[b] > 0.0f ? -0.5f : 0.5f;
            pos[b] = __fmul_rn(__fadd_rn(mp, 0.5f), size[b]);  // trace.frag:66
        }
        DDAResult r;
        dda_skip(g, pos[0], pos[1], pos[2], dm[0], dm[1], dm[2], r);
        if (!r.hit) continue;  // discard: no colour, no depth
        uint32_t index;
        const uint32_t tex = voxel_value(g, r.slot, r.vx, r.vy, r.vz, index);
        const float a = __fdiv_rn(__uint2float_rn(tex >> 24), 255.0f);
        const float ia = __fsub_rn(1.0f, a);
        const uint32_t src[3] = {tex & 0xFFu, (tex >> 8) & 0xFFu, (tex >> 16) & 0xFFu};
        uint32_t* dst[3] = {&cr, &cg, &cb};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = __fadd_rn(__fmul_rn(c_srgb.decode[src[c]], a), __fmul_rn(c_srgb.decode[*dst[c]], ia));
            *dst[c] = srgb_encode(v);
        }
        ca = tex >> 24;  // alpha: ONE * src + ZERO * dst
        depth = tn;
    }
    fb[(size_t)py * f.width + px] = make_uchar4((unsigned char)cr, (unsigned char)cg,
                                                (unsigned char)cb, (unsigned char)ca);
}

struct Compat {
    std::mutex mu;
    bool inited = false;
    int32_t width = 1000, height = 1000;  // lib/entry.c:64-65
    uchar4* fb = nullptr;
    std::vector<int32_t> textures;  // texture id -> grid id
    float* host_instances = nullptr;  // pinned, capacity * 16 floats
    uint32_t capacity = 0;
    uint32_t count = 0;
    bool mapped = false;
    GridView* d_views = nullptr;
    uint32_t views_capacity = 0;
    CompatInstance* d_inst = nullptr;
    uint32_t inst_capacity = 0;
    user_input input;
};

static Compat& compat() {
    static Compat c;
    return c;
}

static uint32_t round_up_p2(uint32_t x) {
    uint32_t r = 1;
    while (r < x) r *= 2;
    return r;
}

// 4x4 inverse in double (cofactor expansion), column-major in and out.
static bool invert4(const double* m, double* inv) {
    double a[16];
    memcpy(a, m, sizeof(a));
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
    if (!(det != 0.0) || !isfinite(det)) return false;
    for (int i = 0; i < 16; ++i) inv[i] = r[i] / det;
    return true;
}

// column-major product c = a * b
static void mul4(const double* a, const double* b, double* c) {
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[col * 4 + k];
            c[col * 4 + row] = s;
        }
}

static int32_t compat_upload_tables() {
    SrgbTables t;
    for (int i = 0; i < 256; ++i) t.decode[i] = (float)srgb_to_linear(i / 255.0);
    for (int k = 0; k < 255; ++k) t.thresh[k] = (float)srgb_to_linear((k + 0.5) / 255.0);
    cudaError_t e = cudaMemcpyToSymbol(c_srgb, &t, sizeof(t));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyToSymbol(srgb tables)");
    return VT_OK;
}

static void compat_release_locked(Compat& c) {
    if (!c.inited) return;
    cudaStreamSynchronize(state().stream);
    cudaFree(c.fb);
    cudaFree(c.d_views);
    cudaFree(c.d_inst);
    cudaFreeHost(c.host_instances);
    for (int32_t g : c.textures) vt_grid_destroy(g);
    c.textures.clear();
    c.fb = nullptr;
    c.d_views = nullptr;
    c.d_inst = nullptr;
    c.host_instances = nullptr;
    c.capacity = c.count = c.views_capacity = c.inst_capacity = 0;
    c.mapped = false;
    c.inited = false;
}

}  // namespace vt

using namespace vt;

void vt_compat_release() {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    compat_release_locked(c);
}

extern "C" {

uint64_t entry(void) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.inited) return 0;
    int32_t rc = ensure_init();
    if (rc) return ((uint64_t)(uint32_t)cudaGetLastError() << 32) | 1u;
    const char* w = getenv("VTRACE_WIDTH");
    const char* h = getenv("VTRACE_HEIGHT");
    c.width = w ? atoi(w) : 1000;
    c.height = h ? atoi(h) : 1000;
    if (c.width <= 0 || c.height <= 0 || c.width > 16384 || c.height > 16384) return 2u;
    cudaError_t e = cudaMalloc(&c.fb, (size_t)c.width * c.height * sizeof(uchar4));
    if (e != cudaSuccess) return ((uint64_t)(uint32_t)e << 32) | 3u;
    if (compat_upload_tables()) return ((uint64_t)(uint32_t)cudaErrorUnknown << 32) | 4u;
    // one instance of capacity, as create_instance_buffer does with instance_count + 1
    c.capacity = 1;
    e = cudaMallocHost(&c.host_instances, 16 * sizeof(float));
    if (e != cudaSuccess) return ((uint64_t)(uint32_t)e << 32) | 5u;
    memset(&c.input, 0, sizeof(c.input));
    c.count = 0;
    c.inited = true;
    return 0;
}

user_input* get_input_data_pointer(void) { return &compat().input; }

int32_t add_texture(const uint8_t* data, uint32_t width, uint32_t height, uint32_t depth) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.inited || !data) return -1;
    if (c.textures.size() >= kMaxTextures) {
        fail(VT_ELIMIT, "Tried allocating too many textures");
        return -1;
    }
    const int32_t g = vt_grid_create_rgba8(data, width, height, depth);
    if (g < 0) return -1;
    c.textures.push_back(g);
    return (int32_t)c.textures.size() - 1;
}

float* start_update_instances(uint32_t instance_count) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.inited) return nullptr;
    if (instance_count == 0) instance_count = 1;
    if (instance_count > c.capacity) {
        cudaStreamSynchronize(state().stream);
        const uint32_t cap = round_up_p2(instance_count + 1);
        float* p = nullptr;
        if (cudaMallocHost(&p, (size_t)cap * 16 * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cudaFreeHost(c.host_instances);
        c.host_instances = p;
        c.capacity = cap;
    }
    c.mapped = true;
    return c.host_instances;
}

int32_t end_update_instances(uint32_t instance_count) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.inited) return -1;
    if (instance_count == 0) instance_count = 1;
    if (instance_count > c.capacity) return -1;
    c.count = instance_count;
    c.mapped = false;
    return 0;
}

int32_t render_tick(int32_t* window_width, int32_t* window_height, const render_tick_info* info) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.inited || !info || !info->perspective || !info->camera) return -1;
    const float* P = (const float*)info->perspective;
    const float* C = (const float*)info->camera;
    double p[16], cm[16], c0[16], ip[16], ic[16], ic0[16], dm[16];
    for (int i = 0; i < 16; ++i) {
        p[i] = P[i];
        cm[i] = C[i];
        c0[i] = C[i];
    }
    c0[12] = c0[13] = c0[14] = 0.0;  // centered camera (trace.frag:54-57)
    if (!invert4(p, ip) || !invert4(cm, ic) || !invert4(c0, ic0)) return -1;
    mul4(ic0, ip, dm);
    CompatFrame f;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) f.dirm[4 * r + k] = (float)dm[k * 4 + r];
    for (int r = 0; r < 3; ++r) f.cam[r] = (float)ic[12 + r];  // inverse(camera) * (0,0,0,1)
    f.width = c.width;
    f.height = c.height;

    // instances -> device records (texture id in the bits of element [3][3], trace.vert:38-40)
    std::vector<CompatInstance> recs;
    recs.reserve(c.count);
    const uint32_t ntex = (uint32_t)c.textures.size();
    for (uint32_t i = 0; i < c.count; ++i) {
        const float* m = c.host_instances + 16 * i;
        int32_t tid;
        memcpy(&tid, &m[15], 4);
        if (tid < 0 || (uint32_t)tid >= ntex) continue;  // unbound descriptor: nothing drawn
        double md[16], mi[16];
        for (int k = 0; k < 16; ++k) md[k] = m[k];
        md[15] = 1.0;
        if (!invert4(md, mi)) continue;
        CompatInstance ci;
        memset(&ci, 0, sizeof(ci));
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 4; ++k) ci.minv[4 * r + k] = (float)mi[k * 4 + r];
        ci.texture = tid;
        recs.push_back(ci);
    }
    cudaStream_t st = state().stream;
    if (ntex > c.views_capacity) {
        cudaFree(c.d_views);
        c.views_capacity = round_up_p2(ntex);
        if (cudaMalloc(&c.d_views, (size_t)c.views_capacity * sizeof(GridView)) != cudaSuccess) {
            c.views_capacity = 0;
            return -1;
        }
    }
    if (recs.size() > c.inst_capacity) {
        cudaFree(c.d_inst);
        c.inst_capacity = round_up_p2((uint32_t)recs.size());
        if (cudaMalloc(&c.d_inst, (size_t)c.inst_capacity * sizeof(CompatInstance)) != cudaSuccess) {
            c.inst_capacity = 0;
            return -1;
        }
    }
    std::vector<GridView> views(ntex);
    for (uint32_t t = 0; t < ntex; ++t) {
        Grid* g = lookup_grid(c.textures[t]);
        if (!g) return -1;
        views[t] = g->view();
    }
    cudaError_t e = cudaSuccess;
    if (ntex) e = cudaMemcpyAsync(c.d_views, views.data(), ntex * sizeof(GridView), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !recs.empty())
        e = cudaMemcpyAsync(c.d_inst, recs.data(), recs.size() * sizeof(CompatInstance), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return -1;
    dim3 grid((c.width + 15) / 16, (c.height + 15) / 16);
    compat_kernel<<<grid, 256, 0, st>>>(c.d_views, c.d_inst, (int32_t)recs.size(), f, c.fb);
    if (cudaGetLastError() != cudaSuccess) return -1;
    // the host vectors above are staged by the copies: wait before they go out of scope
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (window_width) *window_width = c.width;
    if (window_height) *window_height = c.height;
    return 0;
}

void cleanup(void) { vt_compat_release(); }

int32_t vt_framebuffer_download(uint8_t* rgba, uint64_t capacity_bytes) {
    Compat& c = compat();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.inited) return fail(VT_EINVAL, "vt_framebuffer_download: entry() has not run");
    const size_t bytes = (size_t)c.width * c.height * 4;
    if (!rgba || capacity_bytes < bytes) return fail(VT_EINVAL, "vt_framebuffer_download: buffer too small");
    cudaStream_t st = state().stream;
    cudaError_t e = cudaMemcpyAsync(rgba, c.fb, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_framebuffer_download");
    return VT_OK;
}

}  // extern "C"
