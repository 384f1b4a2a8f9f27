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
    int32_t tx0, ty0, tx1, ty1;  // 16 x 16-pixel tiles its pixels can fall in (inclusive; empty
                                 // when tx0 > tx1)
    float near;  // at most the slab entry parameter tn of any pixel's ray (0: no bound)
    int32_t pad;
};

constexpr int32_t kTile = 16;
// Bitmasks larger than this are not built; every tile then visits every instance.
constexpr size_t kMaxBinBytes = (size_t)256 << 20;

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

// Instance binning: bit i of word w of tile t is set iff instance 32 w + i may cover a pixel of
// tile t.  One warp per instance sets its bit in the word of every tile of its rectangle (the
// masks are cleared beforehand), so the work follows the rectangles' areas (24 tiles per
// instance on average in the pager world) instead of tiles x instances (ballots over every
// word of every tile measured 32 us against the scatter's few).
__global__ void __launch_bounds__(256) compat_scatter_kernel(const CompatInstance* __restrict__ inst,
                                                             int32_t ninst, int32_t words,
                                                             int32_t tiles_x, int32_t tiles_y,
                                                             uint32_t* __restrict__ bins) {
    const int32_t lane = threadIdx.x & 31;
    const int32_t i = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (i >= ninst) return;
    const int32_t x0 = max(inst[i].tx0, 0), y0 = max(inst[i].ty0, 0);
    const int32_t x1 = min(inst[i].tx1, tiles_x - 1), y1 = min(inst[i].ty1, tiles_y - 1);
    if (x0 > x1 || y0 > y1) return;
    const int32_t rw = x1 - x0 + 1, area = rw * (y1 - y0 + 1);
    const uint32_t bit = 1u << (i & 31);
    uint32_t* col = bins + (i >> 5);
    for (int32_t k = lane; k < area; k += 32) {
        const int32_t ty = y0 + k / rw, tx = x0 + k % rw;
        atomicOr(col + (size_t)(ty * tiles_x + tx) * words, bit);
    }
}

// The instances of tile `tile` in draw order (all of them when there are no bins), the same
// sequence for every lane of a warp, whose lanes all lie in one tile and all call next() together:
// the lanes load the tile's mask words 32 at a time (one word each, one ballot of the non-empty
// ones), and each non-empty word is broadcast to the warp when its turn comes, so a tile's words
// cost one load round per 32 instead of one dependent load each.
struct InstanceCursor {
    const uint32_t* bins;
    int32_t ninst, words, base, i, w;
    uint32_t lane, mine, pending, bits;
    __device__ InstanceCursor(const uint32_t* b, int32_t n, int32_t nw, int32_t tile)
        : bins(b ? b + (size_t)tile * nw : nullptr), ninst(n), words(nw), base(-32), i(-1), w(0),
          lane(threadIdx.x & 31u), mine(0), pending(0), bits(0) {}
    // next instance index, or -1
    __device__ __forceinline__ int32_t next() {
        if (!bins) return ++i < ninst ? i : -1;
        while (bits == 0) {
            if (pending == 0) {
                base += 32;
                if (base >= words) return -1;
                mine = base + (int32_t)lane < words ? __ldg(bins + base + lane) : 0u;
                pending = __ballot_sync(0xFFFFFFFFu, mine != 0u);
                continue;
            }
            const int32_t j = __ffs(pending) - 1;
            pending &= pending - 1u;
            bits = __shfl_sync(0xFFFFFFFFu, mine, j);
            w = base + j;
        }
        const int32_t b = __ffs(bits) - 1;
        bits &= bits - 1u;
        return w * 32 + b;
    }
};

// Blocks of 128 threads cover 16 x 8 pixels, two per 16 x 16 binning tile.  8 blocks per SM
// (64 registers instead of 72): 3-7% shorter ticks on the pager world.
__global__ void __launch_bounds__(128, 8) compat_kernel(const GridView* __restrict__ views,
                                                     const CompatInstance* __restrict__ inst,
                                                     int32_t ninst, const uint32_t* __restrict__ bins,
                                                     int32_t words, CompatFrame f,
                                                     uchar4* __restrict__ fb) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int32_t px = (int32_t)(blockIdx.x * 16 + (warp & 1u) * 8u + (lane & 7u));
    const int32_t py = (int32_t)(blockIdx.y * 8 + (warp >> 1) * 4u + (lane >> 3));
    // a warp's 8 x 4 pixels lie in one binning tile; lanes outside the frame stay to the end,
    // since the cursor's loads are shared by the warp
    const bool inside = px < f.width && py < f.height;
    if (__ballot_sync(0xFFFFFFFFu, inside) == 0u) return;
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
    InstanceCursor cur(bins, ninst, words, (int32_t)((blockIdx.y >> 1) * gridDim.x + blockIdx.x));
    for (int32_t i = cur.next(); i >= 0; i = cur.next()) {
        if (!inside) continue;
        const CompatInstance& I = inst[i];
        if (I.texture < 0) continue;  // draws nothing (only reached without bins)
        if (I.near >= depth) continue;  // tn >= near >= depth: fails the depth test below
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
    if (!inside) return;
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
    uint32_t views_count = 0;     // texture views on the device, as of grid-table epoch:
    uint64_t views_epoch = ~0ull;  // re-uploaded only when textures or grids change
    CompatInstance* d_inst = nullptr;
    uint32_t inst_capacity = 0;
    float* d_raw = nullptr;  // device copy of the instance matrices, where pinned memory is not
    uint32_t raw_capacity = 0;  // addressable from the device
    uint32_t* d_bins = nullptr;  // per-tile instance bitmasks
    size_t bins_capacity = 0;
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

// 4x4 inverse in double (cofactor expansion), column-major in and out.  Host and device builds
// evaluate it identically (IEEE binary64, no contraction).
static __host__ __device__ bool invert4(const double* m, double* inv) {
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

// Screen-space culling of instances.  The kernel's view ray of pixel (px, py) runs from the
// camera `cam` along A (xn, yn) + c with xn = (px + 0.5) 2 / width - 1 and yn likewise (the
// viewport is width x width, lib/command.c:81), where A's columns and c come from the direction
// matrix.  A world point X lies on that ray at t > 0 iff B q = X - cam with B = [A c] has q.z > 0
// and (q.x, q.y) / q.z = (xn, yn).  The cube's hit points therefore project into the projection
// of the cube clipped to q.z >= eps, for any eps no larger than the nearest hit's q.z: every hit
// is at least the cube's distance delta from the camera, and q.z = |X - cam| / |A (xn, yn) + c|,
// so eps = delta / (largest ray length over the screen) loses nothing.  delta is bounded below by
// the model-space distance of the camera to the unit cube over the Frobenius norm of the inverse
// model matrix.  The clipped cube's vertices (corners with q.z >= eps, and edge crossings of
// q.z = eps) give a pixel rectangle, widened by two pixels for the FP32 rounding of the kernel's
// rays, in double precision throughout.
struct CullFrame {
    double binv[9];  // inverse of B, row-major
    double cam[3];
    double len_max;
    int32_t width, height;
    bool ok;
};

static bool invert3(const double* m, double* r) {
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8],
                 c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (!(det != 0.0) || !isfinite(det)) return false;
    r[0] = c00 / det;
    r[1] = (m[2] * m[7] - m[1] * m[8]) / det;
    r[2] = (m[1] * m[5] - m[2] * m[4]) / det;
    r[3] = c01 / det;
    r[4] = (m[0] * m[8] - m[2] * m[6]) / det;
    r[5] = (m[2] * m[3] - m[0] * m[5]) / det;
    r[6] = c02 / det;
    r[7] = (m[1] * m[6] - m[0] * m[7]) / det;
    r[8] = (m[0] * m[4] - m[1] * m[3]) / det;
    return true;
}

static CullFrame cull_frame(const double* dm, const double* cam, int32_t width, int32_t height) {
    CullFrame cf;
    cf.width = width;
    cf.height = height;
    double b[9];
    for (int r = 0; r < 3; ++r) {
        b[3 * r + 0] = dm[0 * 4 + r];
        b[3 * r + 1] = dm[1 * 4 + r];
        b[3 * r + 2] = dm[2 * 4 + r] + dm[3 * 4 + r];
    }
    cf.ok = invert3(b, cf.binv);
    for (int r = 0; r < 3; ++r) cf.cam[r] = cam[r];
    // |A (xn, yn) + c| is convex in (xn, yn): its maximum over the screen is at a corner
    const double yn_max = 2.0 * height / width - 1.0;
    cf.len_max = 0.0;
    for (int k = 0; k < 4; ++k) {
        const double xn = (k & 1) ? 1.0 : -1.0, yn = (k & 2) ? yn_max : -1.0;
        double l2 = 0.0;
        for (int r = 0; r < 3; ++r) {
            const double v = b[3 * r] * xn + b[3 * r + 1] * yn + b[3 * r + 2];
            l2 += v * v;
        }
        cf.len_max = fmax(cf.len_max, sqrt(l2));
    }
    cf.ok = cf.ok && isfinite(cf.len_max) && cf.len_max > 0.0;
    return cf;
}

// Tile rectangle of an instance (model matrix md, column-major; its inverse mi).  Returns false
// when no pixel can see it.
// A lower bound of the slab entry parameter tn (the distance along the unit-length pixel ray) of
// every pixel's ray, for rejecting the instance behind a pixel's depth before its slab test: the
// camera's distance to the cube in model space over a bound of the inverse's spectral norm
// (sqrt(|Minv|_1 |Minv|_inf)), less 1%.  The pixel kernel's binary32 tn is within about
// cond(M) 2^-21 of the exact one relative to its size, so the 1% holds it above the bound while
// cond(M) (Frobenius) stays below 1024 and the camera is not within 1/256 of the cube; otherwise 0.
static __host__ __device__ float instance_near(const CullFrame& cf, const double* md,
                                               const double* mi) {
    if (!cf.ok) return 0.0f;
    double d2 = 0.0, fm = 0.0, fi = 0.0, n1 = 0.0, ninf = 0.0;
    for (int r = 0; r < 3; ++r) {
        const double om = mi[0 * 4 + r] * cf.cam[0] + mi[1 * 4 + r] * cf.cam[1] +
                          mi[2 * 4 + r] * cf.cam[2] + mi[3 * 4 + r];
        const double e = fmax(fabs(om) - 0.5, 0.0);
        d2 += e * e;
        double row = 0.0, col = 0.0;
        for (int k = 0; k < 3; ++k) {
            fm += md[k * 4 + r] * md[k * 4 + r];
            fi += mi[k * 4 + r] * mi[k * 4 + r];
            row += fabs(mi[k * 4 + r]);  // row r of the inverse's linear part
            col += fabs(mi[r * 4 + k]);  // column r
        }
        ninf = fmax(ninf, row);
        n1 = fmax(n1, col);
    }
    const double dist = sqrt(d2), cond = sqrt(fm) * sqrt(fi), n2 = sqrt(n1 * ninf);
    if (!(dist > 1.0 / 256.0) || !(cond <= 1024.0) || !(n2 > 0.0) || !isfinite(dist)) return 0.0f;
    const float near = (float)(0.99 * dist / n2);
    return isfinite(near) ? near : 0.0f;
}

static __host__ __device__ bool instance_tiles(const CullFrame& cf, const double* md,
                                               const double* mi, int32_t& tx0, int32_t& ty0,
                                               int32_t& tx1, int32_t& ty1) {
    const int32_t ntx = (cf.width + kTile - 1) / kTile, nty = (cf.height + kTile - 1) / kTile;
    tx0 = 0;
    ty0 = 0;
    tx1 = ntx - 1;
    ty1 = nty - 1;
    if (!cf.ok) return true;
    // camera in model space and its distance to the unit cube
    double om[3], d2 = 0.0, fro = 0.0;
    for (int r = 0; r < 3; ++r) {
        om[r] = mi[0 * 4 + r] * cf.cam[0] + mi[1 * 4 + r] * cf.cam[1] + mi[2 * 4 + r] * cf.cam[2] +
                mi[3 * 4 + r];
        const double e = fmax(fabs(om[r]) - 0.5, 0.0);
        d2 += e * e;
        for (int k = 0; k < 3; ++k) fro += mi[k * 4 + r] * mi[k * 4 + r];
    }
    if (!(d2 > 0.0) || !isfinite(d2) || !(fro > 0.0) || !isfinite(fro)) return true;
    const double eps = 0.5 * sqrt(d2 / fro) / cf.len_max;
    // corners in q space
    double q[8][3];
    for (int k = 0; k < 8; ++k) {
        const double m[3] = {(k & 1) ? 0.5 : -0.5, (k & 2) ? 0.5 : -0.5, (k & 4) ? 0.5 : -0.5};
        double x[3];
        for (int r = 0; r < 3; ++r)
            x[r] = md[0 * 4 + r] * m[0] + md[1 * 4 + r] * m[1] + md[2 * 4 + r] * m[2] +
                   md[3 * 4 + r] - cf.cam[r];
        for (int r = 0; r < 3; ++r)
            q[k][r] = cf.binv[3 * r] * x[0] + cf.binv[3 * r + 1] * x[1] + cf.binv[3 * r + 2] * x[2];
    }
    double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
    int used = 0;
    auto take = [&](const double* p) {
        const double r = 1.0 / p[2], xn = p[0] * r, yn = p[1] * r;
        xmin = fmin(xmin, xn);
        xmax = fmax(xmax, xn);
        ymin = fmin(ymin, yn);
        ymax = fmax(ymax, yn);
        ++used;
    };
    for (int k = 0; k < 8; ++k)
        if (q[k][2] >= eps) take(q[k]);
    for (int k = 0; k < 8; ++k)
        for (int a = 0; a < 3; ++a) {
            const int j = k | (1 << a);
            if (j == k) continue;  // each edge once, from its lower corner
            const double sa = q[k][2] - eps, sb = q[j][2] - eps;
            if ((sa < 0.0) == (sb < 0.0)) continue;
            const double u = sa / (sa - sb);
            double p[3];
            for (int r = 0; r < 3; ++r) p[r] = q[k][r] + u * (q[j][r] - q[k][r]);
            p[2] = eps;
            take(p);
        }
    if (used == 0) return false;  // the whole cube is behind the camera
    if (!(isfinite(xmin) && isfinite(xmax) && isfinite(ymin) && isfinite(ymax))) return true;
    // xn -> px: px = (xn + 1) width / 2 - 0.5, and yn -> py with the same width
    const double hw = 0.5 * cf.width;
    const double px0 = floor((xmin + 1.0) * hw - 0.5) - 2.0, px1 = ceil((xmax + 1.0) * hw - 0.5) + 2.0;
    const double py0 = floor((ymin + 1.0) * hw - 0.5) - 2.0, py1 = ceil((ymax + 1.0) * hw - 0.5) + 2.0;
    if (px1 < 0.0 || py1 < 0.0 || px0 > cf.width - 1 || py0 > cf.height - 1) return false;
    tx0 = (int32_t)(fmax(px0, 0.0) / kTile);
    tx1 = (int32_t)(fmin(px1, cf.width - 1.0) / kTile);
    ty0 = (int32_t)(fmax(py0, 0.0) / kTile);
    ty1 = (int32_t)(fmin(py1, cf.height - 1.0) / kTile);
    return true;
}

// Device records of the instances (trace.vert:38-40: the texture id in the bits of element
// [3][3], which reads as 1): inverse model matrix and tile rectangle, one thread per instance,
// in draw order.  Instances with an unbound texture id or a singular matrix draw nothing
// (texture -1, empty rectangle).
__global__ void __launch_bounds__(128) compat_prepare_kernel(const float* __restrict__ insts,
                                                             uint32_t n, uint32_t ntex, CullFrame cf,
                                                             CompatInstance* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* m4 = reinterpret_cast<const float4*>(insts + 16 * (size_t)i);
    float m[16];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float4 v = m4[k];
        m[4 * k] = v.x;
        m[4 * k + 1] = v.y;
        m[4 * k + 2] = v.z;
        m[4 * k + 3] = v.w;
    }
    const int32_t tid = __float_as_int(m[15]);
    CompatInstance ci;
#pragma unroll
    for (int k = 0; k < 12; ++k) ci.minv[k] = 0.0f;
    ci.texture = -1;
    ci.tx0 = ci.ty0 = 1;  // empty rectangle: in no tile
    ci.tx1 = ci.ty1 = 0;
    ci.near = 0.0f;
    ci.pad = 0;
    if (tid >= 0 && (uint32_t)tid < ntex) {
        double md[16], mi[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) md[k] = m[k];
        md[15] = 1.0;
        if (invert4(md, mi)) {
            for (int r = 0; r < 3; ++r)
                for (int k = 0; k < 4; ++k) ci.minv[4 * r + k] = (float)mi[k * 4 + r];
            ci.texture = tid;
            ci.near = instance_near(cf, md, mi);
            if (!instance_tiles(cf, md, mi, ci.tx0, ci.ty0, ci.tx1, ci.ty1)) {
                ci.tx0 = ci.ty0 = 1;
                ci.tx1 = ci.ty1 = 0;
            }
        }
    }
    out[i] = ci;
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
    cudaFree(c.d_raw);
    cudaFree(c.d_bins);
    cudaFreeHost(c.host_instances);
    for (int32_t g : c.textures) vt_grid_destroy(g);
    c.textures.clear();
    c.fb = nullptr;
    c.d_views = nullptr;
    c.d_inst = nullptr;
    c.d_raw = nullptr;
    c.raw_capacity = 0;
    c.d_bins = nullptr;
    c.bins_capacity = 0;
    c.host_instances = nullptr;
    c.capacity = c.count = c.views_capacity = c.inst_capacity = 0;
    c.views_count = 0;
    c.views_epoch = ~0ull;
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
    const CullFrame cf = cull_frame(dm, ic + 12, c.width, c.height);

    cudaStream_t st = state().stream;
    const uint32_t ntex = (uint32_t)c.textures.size();
    const uint64_t epoch = state().grid_epoch.load();
    if (ntex != c.views_count || epoch != c.views_epoch) {  // texture views, when they changed
        if (ntex > c.views_capacity) {
            cudaFree(c.d_views);
            c.views_capacity = round_up_p2(ntex);
            if (cudaMalloc(&c.d_views, (size_t)c.views_capacity * sizeof(GridView)) != cudaSuccess) {
                c.views_capacity = 0;
                return -1;
            }
        }
        std::vector<GridView> views(ntex);
        for (uint32_t t = 0; t < ntex; ++t) {
            Grid* g = lookup_grid(c.textures[t]);
            if (!g) return -1;
            views[t] = g->view();
        }
        if (ntex && (cudaMemcpyAsync(c.d_views, views.data(), ntex * sizeof(GridView),
                                     cudaMemcpyHostToDevice, st) != cudaSuccess ||
                     cudaStreamSynchronize(st) != cudaSuccess))
            return -1;
        c.views_count = ntex;
        c.views_epoch = epoch;
    }
    // instance records on the device, from the pinned instance buffer the GPU reads directly
    const uint32_t n = c.count;
    if (n > c.inst_capacity) {
        cudaFree(c.d_inst);
        c.inst_capacity = round_up_p2(n);
        if (cudaMalloc(&c.d_inst, (size_t)c.inst_capacity * sizeof(CompatInstance)) != cudaSuccess) {
            c.inst_capacity = 0;
            return -1;
        }
    }
    const float* d_src = (const float*)host_mapped(c.host_instances);
    if (n && !d_src) {  // not addressable from the device here: copy the matrices over
        if (n > c.raw_capacity) {
            cudaFree(c.d_raw);
            c.raw_capacity = round_up_p2(n);
            if (cudaMalloc(&c.d_raw, (size_t)c.raw_capacity * 16 * sizeof(float)) != cudaSuccess) {
                c.raw_capacity = 0;
                return -1;
            }
        }
        if (cudaMemcpyAsync(c.d_raw, c.host_instances, (size_t)n * 16 * sizeof(float),
                            cudaMemcpyHostToDevice, st) != cudaSuccess)
            return -1;
        d_src = c.d_raw;
    }
    if (n)
        // 32 threads per block spread the binary64 work of a few thousand instances over all SMs
        compat_prepare_kernel<<<(n + 31) / 32, 32, 0, st>>>(d_src, n, ntex, cf, c.d_inst);
    dim3 grid((c.width + kTile - 1) / kTile, (c.height + kTile - 1) / kTile);
    const int32_t ninst = (int32_t)n;
    const int32_t words = (ninst + 31) / 32, ntiles = (int32_t)(grid.x * grid.y);
    const size_t bin_bytes = (size_t)ntiles * words * 4;
    uint32_t* bins = nullptr;
    if (ninst > 0 && bin_bytes <= kMaxBinBytes) {
        if (bin_bytes > c.bins_capacity) {
            cudaFree(c.d_bins);
            c.d_bins = nullptr;
            c.bins_capacity = 0;
            if (cudaMalloc(&c.d_bins, bin_bytes) != cudaSuccess) return -1;
            c.bins_capacity = bin_bytes;
        }
        bins = c.d_bins;
        if (cudaMemsetAsync(bins, 0, bin_bytes, st) != cudaSuccess) return -1;
        compat_scatter_kernel<<<(ninst + 7) / 8, 256, 0, st>>>(c.d_inst, ninst, words,
                                                               (int32_t)grid.x, (int32_t)grid.y, bins);
    }
    const dim3 pgrid(grid.x, (c.height + 7) / 8);
    compat_kernel<<<pgrid, 128, 0, st>>>(c.d_views, c.d_inst, ninst, bins, words, f, c.fb);
    if (cudaGetLastError() != cudaSuccess) return -1;
    // the frame is complete when render_tick returns (the instance buffer may then change)
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
