// vt_trace.cu — traversal kernels of libvtrace: per-pixel render and ray-buffer trace.
#include <cuda_runtime.h>

#include <algorithm>

#include "vt_device.cuh"
#include "vt_kernels.h"

namespace vt {

// Image tile of one warp: 8 x 4 pixels by default, so that a warp's rays start together and stay
// coherent.  A 128-thread block covers 16 x 8 pixels (2 x 2 warps): small blocks free their slots
// soon after their slowest ray ends (6% faster than 256-thread blocks on the 1080p frame).  The
// fused render launch takes other warp tiles and block sizes from its tuning (the autotuner's
// search space); the two-pass form keeps the default.
constexpr int kTileW = 16, kTileH = 8, kTileThreads = 128;

// Warp tile and block arrangement of a render launch: warp tiles of (1 << wx_log) x
// (32 >> wx_log) pixels, bx x by of them per block.
struct RenderShape {
    uint32_t wx_log, bx, by;
    uint32_t block_w() const { return bx << wx_log; }
    uint32_t block_h() const { return by * (32u >> wx_log); }
};

static RenderShape render_shape(const TraceTuning* tune) {
    static const uint32_t kLog[4] = {3, 2, 4, 5};  // VT_TILE_8X4, 4X8, 16X2, 32X1
    const uint32_t wx_log = tune && tune->tile_shape < 4 ? kLog[tune->tile_shape] : 3u;
    uint32_t warps = tune ? tune->block_warps : 4u;
    if (warps != 1 && warps != 2 && warps != 8) warps = 4;
    // warps along x: the power of two that brings the block closest to twice as wide as high
    RenderShape best{wx_log, 1, warps};
    double best_err = 1e30;
    for (uint32_t bx = 1; bx <= warps; bx <<= 1) {
        const RenderShape r{wx_log, bx, warps / bx};
        const double aspect = (double)r.block_w() / (double)r.block_h();
        const double err = aspect > 2.0 ? aspect / 2.0 : 2.0 / aspect;
        if (err < best_err) {
            best_err = err;
            best = r;
        }
    }
    return best;
}

// Rows row0 .. row1 - 1 of the image (a band; the whole image when 0 .. height).
template <bool STATS>
__global__ void __launch_bounds__(256) render_kernel(GridView g, vt_camera cam, LightView light,
                                                     uint4* __restrict__ out,
                                                     Counters* __restrict__ counters,
                                                     uint32_t row0, uint32_t row1,
                                                     RenderShape shape) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t wx = 1u << shape.wx_log, wy = 32u >> shape.wx_log;
    const uint32_t px = blockIdx.x * (shape.bx * wx) + (warp % shape.bx) * wx + (lane & (wx - 1u));
    const uint32_t py = row0 + blockIdx.y * (shape.by * wy) + (warp / shape.bx) * wy + (lane >> shape.wx_log);
    const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, px < cam.width && py < row1);
    if (px >= cam.width || py >= row1) return;
    Tally<STATS> tl;
    tl.bind(counters, g.bricks);
    const HitRec h = render_pixel<STATS>(g, cam, light, px, py, vmask, tl);
    out[(size_t)py * cam.width + px] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    tl.flush(counters);
}

template <bool STATS>
__global__ void __launch_bounds__(256) trace_rays_kernel(GridView g,
                                                         const float2* __restrict__ rays,
                                                         uint64_t n, uint4* __restrict__ out,
                                                         Counters* __restrict__ counters,
                                                         const unsigned int* __restrict__ n_dev) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = min((uint64_t)*n_dev, n);
    if (i >= n) return;
    Tally<STATS> tl;
    tl.bind(counters, g.bricks);
    // 24-byte rays: three 8-byte loads
    const float2 a = __ldg(rays + 3 * i), b = __ldg(rays + 3 * i + 1), c = __ldg(rays + 3 * i + 2);
    const float o[3] = {a.x, a.y, b.x}, d[3] = {b.y, c.x, c.y};
    const HitRec h = trace_ray<STATS>(g, o, d, tl);
    out[i] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    tl.flush(counters);
}

cudaError_t launch_render(const GridView& g, const vt_camera& cam, const LightView& light,
                          uint4* out, Counters* counters, cudaStream_t stream, uint32_t row0,
                          uint32_t row1, const TraceTuning* tune) {
    if (row1 == 0 || row1 > cam.height) row1 = cam.height;
    if (row0 >= row1) return cudaSuccess;
    const RenderShape sh = render_shape(tune);
    const unsigned threads = 32u * sh.bx * sh.by;
    dim3 grid((cam.width + sh.block_w() - 1) / sh.block_w(),
              (row1 - row0 + sh.block_h() - 1) / sh.block_h());
    if (counters)
        render_kernel<true><<<grid, threads, 0, stream>>>(g, cam, light, out, counters, row0, row1, sh);
    else
        render_kernel<false><<<grid, threads, 0, stream>>>(g, cam, light, out, nullptr, row0, row1, sh);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const GridView& g, const vt_ray* rays, uint64_t n, uint4* out,
                              Counters* counters, cudaStream_t stream, const unsigned int* n_dev) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = (n + 255) / 256;
    const float2* r2 = reinterpret_cast<const float2*>(rays);
    if (counters)
        trace_rays_kernel<true><<<(unsigned)blocks, 256, 0, stream>>>(g, r2, n, out, counters, n_dev);
    else
        trace_rays_kernel<false><<<(unsigned)blocks, 256, 0, stream>>>(g, r2, n, out, nullptr, n_dev);
    return cudaGetLastError();
}

}  // namespace vt

// ---------------------------------------------------------------------------------------------
// Persistent tracers with live-ray compaction.
//
// One launch of sm_count x (resident blocks per SM) blocks.  Every warp keeps a ray per lane and
// loops: when at least `refill_min` lanes are idle, the warp fetches that many work items with
// one atomic on `counter` and starts their rays; then every live lane advances its ray by one
// unit (vt_lane.cuh).  Lanes whose rays end are refilled between units, so the warp stays full
// while the image's rays have very different lengths.  Items are numbered in 8 x 4 pixel tiles
// (render) or by ray index (ray buffers), so a refill hands a warp neighbouring rays.
// ---------------------------------------------------------------------------------------------
#include "vt_lane.cuh"

namespace vt {

__device__ __forceinline__ bool item_pixel(uint64_t item, uint32_t tiles_x, const vt_camera& cam,
                                           uint32_t& px, uint32_t& py) {
    const uint64_t tile = item >> 5;
    const uint32_t l = (uint32_t)item & 31u;
    px = (uint32_t)(tile % tiles_x) * 8u + (l & 7u);
    py = (uint32_t)(tile / tiles_x) * 4u + (l >> 3);
    return px < cam.width && py < cam.height;
}

// Render state of one lane: kind 0 idle, 1 primary ray, 2 shadow ray of `prim`; pend 1 or 2
// when that ray is queued but not started.
struct RenderLane {
    LaneRay R;
    int kind, pend;
    uint32_t pix;
    HitRec prim;
    float ndl;
    float so[3];  // origin of the queued shadow ray
};

constexpr int kRayQueued = 3;  // the lane's next ray is queued in RenderLane::pend

// A ray of the lane ended with `st`: write the pixel, or queue the shadow ray.
__device__ __forceinline__ void render_finish(const GridView& g, const LightView& L, RenderLane& s,
                                              int st, uint4* out) {
    if (s.kind == 1) {
        HitRec h = ray_record(g, s.R, st, VT_SKY_RGBA);
        float nd;
        if (st != kRayHit || !L.enabled || !face_lit(h, L, nd)) {
            out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
            s.kind = 0;
            return;
        }
        if (nd > 0.0f && L.shadows) {
            shadow_origin(h, s.R.o, s.R.d, s.so);
            s.prim = h;
            s.ndl = nd;
            s.kind = 2;
            s.pend = 2;
            return;
        }
        h.w3 = shade_rgba(h.w3, nd, 1.0f, L.ambient);
        out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
        s.kind = 0;
        return;
    }
    // shadow ray
    const bool shadowed = st == kRayHit;
    HitRec h = s.prim;
    h.w3 = shade_rgba(h.w3, s.ndl, shadowed ? 0.0f : 1.0f, L.ambient);
    h.w1 |= (VT_HIT_FLAG_SHADOW_RAY | (shadowed ? VT_HIT_FLAG_SHADOWED : 0u)) << 24;
    out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    s.kind = 0;
}

// ray_begin, render_finish and ray_unit each have one call site (lanes starting rays do so
// together; small code).
__global__ void __launch_bounds__(256) render_persistent_kernel(
    GridView g, vt_camera cam, LightView L, uint4* __restrict__ out,
    unsigned long long* __restrict__ counter, uint32_t tiles_x, uint64_t total,
    uint32_t refill_min) {
    const uint32_t lane = threadIdx.x & 31u;
    RenderLane s;
    s.kind = 0;
    s.pend = 0;
    s.pix = 0;
    s.ndl = 0.0f;
    int st = kRayMiss;
    bool more = true;  // warp-uniform
    for (;;) {
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, s.kind == 0);
        while (more && __popc(idle) >= (int)refill_min) {
            uint64_t item;
            const uint64_t base = warp_fetch(counter, idle, lane, item);
            if (base + __popc(idle) >= total) more = false;
            if (s.kind == 0 && item < total) {
                uint32_t px, py;
                if (item_pixel(item, tiles_x, cam, px, py)) {
                    s.pix = py * cam.width + px;
                    s.kind = 1;
                    s.pend = 1;
                    st = kRayQueued;
                }
            }
            idle = __ballot_sync(0xFFFFFFFFu, s.kind == 0);
        }
        if (!more && idle == 0xFFFFFFFFu) break;
        while (s.kind != 0 && st != kRayRunning) {
            if (s.pend != 0) {
                float o[3], d[3];
                if (s.pend == 1) {
                    raygen(cam, s.pix % cam.width, s.pix / cam.width, 0.5f, 0.5f, o, d);
                } else {
#pragma unroll
                    for (int k = 0; k < 3; ++k) o[k] = s.so[k];
                    d[0] = L.dx;
                    d[1] = L.dy;
                    d[2] = L.dz;
                }
                s.pend = 0;
                st = ray_begin(g, o, d, s.R);
            } else {
                render_finish(g, L, s, st, out);
                st = kRayQueued;
            }
        }
        if (s.kind != 0) st = ray_unit(g, s.R);
    }
}

constexpr int kUnitWait = 4;

// n_dev: nullptr, or the device-side ray count (at most n), read at the start (ray queues whose
// length the host does not know).  Held to 48 registers (a few bytes of spills) so that five
// blocks fit an SM instead of four: the short rays of dense grids wait on their mask and directory
// loads, and the fifth block hides more of that (16.7M cave rays 2.29 -> 2.17 ms; six blocks at
// 40 registers spill more and lose).
__global__ void __launch_bounds__(256, 5) trace_rays_persistent_kernel(
    GridView g, const float2* __restrict__ rays, uint64_t n, uint4* __restrict__ out,
    unsigned long long* __restrict__ counter, uint32_t refill_min,
    const unsigned int* __restrict__ n_dev) {
    if (n_dev) n = min((uint64_t)*n_dev, n);
    const uint32_t lane = threadIdx.x & 31u;
    LaneRay R;
    bool busy = false;
    uint64_t idx = 0;
    bool more = true;
    int wait_w = 0, wait_c = 0;  // warp-uniform: iterations a unit kind was passed over
    for (;;) {
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, !busy);
        while (more && __popc(idle) >= (int)refill_min) {
            uint64_t item;
            const uint64_t base = warp_fetch(counter, idle, lane, item);
            if (base + __popc(idle) >= n) more = false;
            if (!busy && item < n) {
                const float2 a = __ldg(rays + 3 * item), b = __ldg(rays + 3 * item + 1),
                             c = __ldg(rays + 3 * item + 2);
                const float o[3] = {a.x, a.y, b.x}, d[3] = {b.y, c.x, c.y};
                const int st = ray_begin(g, o, d, R);
                if (st == kRayRunning) {
                    busy = true;
                    idx = item;
                } else {
                    const HitRec h = ray_record(g, R, st, 0u);
                    out[item] = make_uint4(h.w0, h.w1, h.w2, h.w3);
                }
            }
            idle = __ballot_sync(0xFFFFFFFFu, !busy);
        }
        if (!more && idle == 0xFFFFFFFFu) break;
        // One kind of unit per pass: the lanes whose next unit is the more common kind (walk or
        // crossing) run it, the others wait, unless their kind has already waited kUnitWait
        // passes.  A warp then issues one kind's instructions per pass instead of both; every
        // pass with busy lanes runs at least one unit.  2% faster on the 16M incoherent rays.
        const uint32_t e = busy ? ray_entry(g, R) : kEmptyBit;
        const bool walk = busy && !brick_empty(e);
        const uint32_t wb = __ballot_sync(0xFFFFFFFFu, walk);
        const uint32_t cb = __ballot_sync(0xFFFFFFFFu, busy && !walk);
        bool run_walk = __popc(wb) >= __popc(cb);
        if (run_walk ? (cb && wait_c >= kUnitWait) : (wb && wait_w >= kUnitWait)) run_walk = !run_walk;
        if (run_walk) {
            wait_w = 0;
            wait_c = cb ? wait_c + 1 : 0;
        } else {
            wait_c = 0;
            wait_w = wb ? wait_w + 1 : 0;
        }
        if (busy && walk == run_walk) {
            const int st = ray_unit(g, R, e);
            if (st != kRayRunning) {
                const HitRec h = ray_record(g, R, st, 0u);
                out[idx] = make_uint4(h.w0, h.w1, h.w2, h.w3);
                busy = false;
            }
        }
    }
}

static int resident_blocks(const void* kernel) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, 256, 0) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    return n < 1 ? 1 : n;
}

cudaError_t launch_render_persistent(const GridView& g, const vt_camera& cam,
                                     const LightView& light, uint4* out,
                                     unsigned long long* counter, const TraceTuning& tune,
                                     int sm_count, cudaStream_t stream) {
    static int per_sm = resident_blocks((const void*)render_persistent_kernel);
    const uint32_t tiles_x = (cam.width + 7) / 8, tiles_y = (cam.height + 3) / 4;
    const uint64_t total = (uint64_t)tiles_x * tiles_y * 32;
    const int bps = tune.blocks_per_sm > 0 ? min(tune.blocks_per_sm, per_sm) : per_sm;
    const uint64_t need = (total + 255) / 256;
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)sm_count * bps, need);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    render_persistent_kernel<<<blocks, 256, 0, stream>>>(g, cam, light, out, counter, tiles_x,
                                                         total, tune.refill_min);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays_persistent(const GridView& g, const vt_ray* rays, uint64_t n,
                                         uint4* out, unsigned long long* counter,
                                         const TraceTuning& tune, int sm_count,
                                         cudaStream_t stream, const unsigned int* n_dev) {
    if (n == 0) return cudaSuccess;
    static int per_sm = resident_blocks((const void*)trace_rays_persistent_kernel);
    const int bps = tune.blocks_per_sm > 0 ? min(tune.blocks_per_sm, per_sm) : per_sm;
    const uint64_t need = (n + 255) / 256;
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)sm_count * bps, need);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    trace_rays_persistent_kernel<<<blocks, 256, 0, stream>>>(
        g, reinterpret_cast<const float2*>(rays), n, out, counter, tune.refill_min, n_dev);
    return cudaGetLastError();
}

}  // namespace vt

// ---------------------------------------------------------------------------------------------
// Two-pass render ("wavefront"): the primary pass shades what it can and appends every needed
// shadow ray to a compacted queue (one warp-aggregated atomic per warp, queue order = tile
// order, so neighbouring queue entries are neighbouring pixels); the shadow pass traces full warps
// of shadow rays, all parallel to the light, and finishes those pixels.  Same records as the
// fused render_kernel.
// ---------------------------------------------------------------------------------------------
namespace vt {

struct ShadowJob {
    uint32_t pix;
    float so[3];
};

__global__ void __launch_bounds__(kTileThreads) render_primary_kernel(GridView g, vt_camera cam,
                                                             LightView L,
                                                             uint4* __restrict__ out,
                                                             ShadowJob* __restrict__ queue,
                                                             unsigned int* __restrict__ count) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t px = blockIdx.x * kTileW + (warp & 1u) * 8u + (lane & 7u);
    const uint32_t py = blockIdx.y * kTileH + (warp >> 1) * 4u + (lane >> 3);
    const bool inside = px < cam.width && py < cam.height;
    bool need = false;
    ShadowJob job;
    if (inside) {
        Tally<false> tl;
        float o[3], d[3];
        raygen(cam, px, py, 0.5f, 0.5f, o, d);
        HitRec h = trace_ray<false>(g, o, d, tl);
        const uint32_t flags = h.w1 >> 24;
        float ndl;
        if (!(flags & VT_HIT_FLAG_HIT)) {
            h.w3 = VT_SKY_RGBA;
        } else if (L.enabled && face_lit(h, L, ndl)) {
            if (ndl > 0.0f && L.shadows) {
                need = true;
                job.pix = py * cam.width + px;
                shadow_origin(h, o, d, job.so);
            } else {
                h.w3 = shade_rgba(h.w3, ndl, 1.0f, L.ambient);
            }
        }
        out[(size_t)py * cam.width + px] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    }
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, need);
    if (ballot) {
        const int leader = __ffs(ballot) - 1;
        unsigned int base = 0;
        if ((int)lane == leader) base = atomicAdd(count, (unsigned int)__popc(ballot));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (need) queue[base + __popc(ballot & ((1u << lane) - 1u))] = job;
    }
}

__global__ void __launch_bounds__(256) render_shadow_kernel(GridView g, LightView L,
                                                            uint4* __restrict__ out,
                                                            const ShadowJob* __restrict__ queue,
                                                            const unsigned int* __restrict__ count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *count) return;
    const ShadowJob job = queue[i];
    Tally<false> tl;
    const float ld[3] = {L.dx, L.dy, L.dz};
    const HitRec s = trace_ray<false>(g, job.so, ld, tl);
    const bool shadowed = ((s.w1 >> 24) & VT_HIT_FLAG_HIT) != 0u;
    uint4 h = out[job.pix];
    HitRec r;
    r.w0 = h.x;
    r.w1 = h.y;
    r.w2 = h.z;
    r.w3 = h.w;
    float ndl = 0.0f;
    face_lit(r, L, ndl);
    r.w3 = shade_rgba(r.w3, ndl, shadowed ? 0.0f : 1.0f, L.ambient);
    r.w1 |= (VT_HIT_FLAG_SHADOW_RAY | (shadowed ? VT_HIT_FLAG_SHADOWED : 0u)) << 24;
    out[job.pix] = make_uint4(r.w0, r.w1, r.w2, r.w3);
}

cudaError_t launch_render_wavefront(const GridView& g, const vt_camera& cam,
                                    const LightView& light, uint4* out, cudaStream_t stream) {
    const uint64_t npx = (uint64_t)cam.width * cam.height;
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, 256 + npx * sizeof(ShadowJob), stream);
    if (e != cudaSuccess) return e;
    unsigned int* count = (unsigned int*)scratch;
    ShadowJob* queue = (ShadowJob*)((char*)scratch + 256);
    e = cudaMemsetAsync(count, 0, sizeof(unsigned int), stream);
    if (e == cudaSuccess) {
        dim3 grid((cam.width + kTileW - 1) / kTileW, (cam.height + kTileH - 1) / kTileH);
        render_primary_kernel<<<grid, kTileThreads, 0, stream>>>(g, cam, light, out, queue, count);
        if (light.enabled && light.shadows)
            render_shadow_kernel<<<(unsigned)((npx + 255) / 256), 256, 0, stream>>>(g, light, out,
                                                                                   queue, count);
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(scratch, stream);
    return e != cudaSuccess ? e : f;
}

}  // namespace vt

// ---------------------------------------------------------------------------------------------
// Queued-shadow render: resident warps take whole 8 x 4 pixel tiles from a work counter and trace
// their camera rays to the end, one per lane, as the tile launch does; a pixel that needs a shadow
// ray queues it (its primary record and the ray's origin) in its warp's queue in shared memory
// instead of tracing it in the lane, and the warp traces queued shadow rays 32 at a time,
// whenever 32 are waiting, so that shadow rays run in full warps.  No barrier and no per-lane
// state machine: a warp only ever waits for its own lanes.  The remainder of each queue is traced
// when the counter runs dry.  Same records as the fused render.
// ---------------------------------------------------------------------------------------------
namespace vt {

constexpr int kQueueWarps = 4;     // 128-thread blocks
constexpr uint32_t kQueueCap = 64;  // entries per warp: up to 31 left over + 32 from one tile

struct QueuedShadow {
    HitRec prim;  // the unshaded primary record
    float so[3];  // shadow ray origin
    uint32_t pix;
};

// One traversal call site serves both kinds of unit (a tile of camera rays, or up to 32 queued
// shadow rays), so that the kernel holds the traversal's registers once.
__global__ void __launch_bounds__(kQueueWarps * 32, 10) render_queue_kernel(
    GridView g, vt_camera cam, LightView L, uint4* __restrict__ out,
    unsigned long long* __restrict__ counter, uint32_t tiles_x, uint64_t tiles) {
    __shared__ QueuedShadow queue[kQueueWarps][kQueueCap];
    const uint32_t lane = threadIdx.x & 31u;
    QueuedShadow* q = queue[threadIdx.x >> 5];
    uint32_t qn = 0;     // warp-uniform: queued shadow rays
    bool tiles_left = true;  // warp-uniform
    for (;;) {
        // warp-uniform choice of the unit: 32 queued shadow rays, else a tile, else the rest of
        // the queue
        bool shadow_unit = qn >= 32u;
        uint64_t u = 0;
        if (!shadow_unit && tiles_left) {
            unsigned long long v = 0;
            if (lane == 0) v = atomicAdd(counter, 1ull);
            u = __shfl_sync(0xFFFFFFFFu, v, 0);
            if (u >= tiles) tiles_left = false;
        }
        if (!shadow_unit && !tiles_left) {
            if (qn == 0) break;
            shadow_unit = true;
        }
        const uint32_t n = shadow_unit ? min(qn, 32u) : 32u;
        uint32_t px = 0, py = 0;
        bool active;
        float o[3], d[3];
        if (shadow_unit) {
            active = lane < n;
            if (active) {
                o[0] = q[lane].so[0];
                o[1] = q[lane].so[1];
                o[2] = q[lane].so[2];
            }
            d[0] = L.dx;
            d[1] = L.dy;
            d[2] = L.dz;
        } else {
            px = (uint32_t)(u % tiles_x) * 8u + (lane & 7u);
            py = (uint32_t)(u / tiles_x) * 4u + (lane >> 3);
            active = px < cam.width && py < cam.height;
            if (active) raygen(cam, px, py, 0.5f, 0.5f, o, d);
        }
        HitRec h;
        if (active) {
            Tally<false> tl;
            h = trace_ray<false>(g, o, d, tl);
        }
        __syncwarp();
        if (shadow_unit) {
            if (active) {
                const bool shadowed = ((h.w1 >> 24) & VT_HIT_FLAG_HIT) != 0u;
                HitRec p = q[lane].prim;
                float ndl = 0.0f;
                face_lit(p, L, ndl);
                p.w3 = shade_rgba(p.w3, ndl, shadowed ? 0.0f : 1.0f, L.ambient);
                p.w1 |= (VT_HIT_FLAG_SHADOW_RAY | (shadowed ? VT_HIT_FLAG_SHADOWED : 0u)) << 24;
                out[q[lane].pix] = make_uint4(p.w0, p.w1, p.w2, p.w3);
            }
            // move the rest (at most 31 entries) down to the front
            QueuedShadow rest;
            const bool mv = lane + n < qn;
            if (mv) rest = q[lane + n];
            __syncwarp();
            if (mv) q[lane] = rest;
            __syncwarp();
            qn -= n;
            continue;
        }
        bool need = false;
        if (active) {
            const uint32_t pix = py * cam.width + px;
            float ndl;
            if (!((h.w1 >> 24) & VT_HIT_FLAG_HIT)) {
                h.w3 = VT_SKY_RGBA;
            } else if (L.enabled && face_lit(h, L, ndl)) {
                if (ndl > 0.0f && L.shadows) {
                    need = true;
                } else {
                    h.w3 = shade_rgba(h.w3, ndl, 1.0f, L.ambient);
                }
            }
            if (!need) out[pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
        }
        const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, need);
        if (need) {
            QueuedShadow& e = q[qn + __popc(ballot & ((1u << lane) - 1u))];
            e.prim = h;
            e.pix = py * cam.width + px;
            shadow_origin(h, o, d, e.so);
        }
        __syncwarp();
        qn += __popc(ballot);
    }
}

cudaError_t launch_render_queued(const GridView& g, const vt_camera& cam, const LightView& light,
                                 uint4* out, unsigned long long* counter, const TraceTuning& tune,
                                 int sm_count, cudaStream_t stream) {
    static int per_sm = [] {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, (const void*)render_queue_kernel,
                                                          kQueueWarps * 32, 0) != cudaSuccess) {
            cudaGetLastError();
            n = 1;
        }
        return n < 1 ? 1 : n;
    }();
    const uint32_t tiles_x = (cam.width + 7) / 8, tiles_y = (cam.height + 3) / 4;
    const uint64_t tiles = (uint64_t)tiles_x * tiles_y;
    const int bps = tune.blocks_per_sm > 0 ? min(tune.blocks_per_sm, per_sm) : per_sm;
    const uint64_t need = (tiles + kQueueWarps - 1) / kQueueWarps;
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)sm_count * bps, need);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    render_queue_kernel<<<blocks, kQueueWarps * 32, 0, stream>>>(g, cam, light, out, counter,
                                                                 tiles_x, tiles);
    return cudaGetLastError();
}

}  // namespace vt
