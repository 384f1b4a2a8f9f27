// vt_path.cu — multi-bounce diffuse path tracing on the traversal kernel (vtrace's stated goal,
// README.md:2; the reference has no path tracer, so the estimator is this library's own
// specification, restated operation for operation by the oracle's vto_path_pixel).
//
// Per pixel, for each of `spp` samples: a jittered camera ray (Philox4x32-10, as the batched
// renderer), then up to max_bounces + 1 path vertices.  At a vertex the throughput takes the
// voxel's colour (byte / 255 per channel); with a sun, a Lambert next-event ray from the hit point
// (1/64 voxel off the entered face) toward the sun adds throughput x sun x n.l when it leaves the
// grid unblocked; the path continues along n + u, u uniform on the unit sphere (rejection
// sampling in the cube, 16 tries, Philox counters (px, py, sample, bounce << 8 | try)), which is
// cosine-weighted about n, so that the Lambert BRDF and the sampling density cancel.  A ray that
// leaves the grid adds throughput x sky.  A hit without a face (origin inside an occupied voxel)
// ends the path.  The samples' radiances are summed in order and divided by spp; the output is
// float RGBA (alpha 1) or RGBA8 (clamped to [0, 1], x 255, rounded half up, alpha 255).
//
// All arithmetic is IEEE binary32 round-to-nearest without contraction (explicit intrinsics), so
// the result is bit-identical to the oracle.  One thread traces one pixel's samples in 8 x 4
// pixel tiles.
#include <cuda_runtime.h>

#include <algorithm>

#include "vt_api_internal.h"
#include "vt_device.cuh"
#include "vt_internal.h"
#include "vt_lane.cuh"

namespace vt {

struct PathParams {
    uint32_t spp, max_bounces, seed, out_format;
    float sky[3], sun_dir[3], sun[3];
    bool sun_on;
};

constexpr uint32_t kPathKey = 0x50415448u;  // "PATH"
constexpr int kSphereTries = 16;

// A unit vector uniform on the sphere, or false after kSphereTries rejected cube samples.
__device__ __forceinline__ bool sphere_sample(uint32_t seed, uint32_t px, uint32_t py, uint32_t s,
                                              uint32_t bounce, float u[3]) {
    for (int t = 0; t < kSphereTries; ++t) {
        uint32_t r[4];
        philox4x32_10(px, py, s, (bounce << 8) | (uint32_t)t, seed, kPathKey, r);
        float p[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)  // (r >> 8) 2^-23 - 1: exact, in [-1, 1)
            p[k] = __fsub_rn(__fmul_rn(__uint2float_rn(r[k] >> 8), 0x1p-23f), 1.0f);
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(p[0], p[0]), __fmul_rn(p[1], p[1])),
                                   __fmul_rn(p[2], p[2]));
        if (r2 <= 1.0f && r2 > 0x1p-20f) {
            const float l = __fsqrt_rn(r2);
#pragma unroll
            for (int k = 0; k < 3; ++k) u[k] = __fdiv_rn(p[k], l);
            return true;
        }
    }
    return false;
}

__device__ __forceinline__ void path_pixel(const GridView& g, const vt_camera& cam,
                                           const PathParams& P, uint32_t px, uint32_t py,
                                           float sum[3], uint32_t& rays) {
    Tally<false> tl;
    sum[0] = sum[1] = sum[2] = 0.0f;
    for (uint32_t s = 0; s < P.spp; ++s) {
        float jx, jy, o[3], d[3];
        jitter(P.seed, 0u, px, py, s, jx, jy);
        raygen(cam, px, py, jx, jy, o, d);
        float T[3] = {1.0f, 1.0f, 1.0f}, L[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t b = 0;; ++b) {
            const HitRec h = trace_ray<false>(g, o, d, tl);
            ++rays;
            const uint32_t flags = h.w1 >> 24;
            if (!(flags & VT_HIT_FLAG_HIT)) {
#pragma unroll
                for (int c = 0; c < 3; ++c) L[c] = __fadd_rn(L[c], __fmul_rn(T[c], P.sky[c]));
                break;
            }
            const uint32_t face = flags & VT_FACE_MASK;
            if (face == 0) break;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                T[c] = __fmul_rn(T[c], __fdiv_rn(__uint2float_rn((h.w3 >> (8 * c)) & 0xFFu), 255.0f));
            const int a = (int)(face - 1) / 2;
            const bool npos = (face & 1u) != 0u;
            float so[3];
            shadow_origin(h, o, d, so);
            if (P.sun_on) {
                const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
                const float ndl = npos ? la : -la;
                if (ndl > 0.0f) {
                    const HitRec sh = trace_ray<false>(g, so, P.sun_dir, tl);
                    ++rays;
                    if (!((sh.w1 >> 24) & VT_HIT_FLAG_HIT)) {
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            L[c] = __fadd_rn(L[c], __fmul_rn(__fmul_rn(T[c], P.sun[c]), ndl));
                    }
                }
            }
            if (b >= P.max_bounces) break;
            float n[3] = {0.0f, 0.0f, 0.0f};
            n[a] = npos ? 1.0f : -1.0f;
            float u[3], nd[3];
            if (sphere_sample(P.seed, px, py, s, b, u)) {
#pragma unroll
                for (int k = 0; k < 3; ++k) nd[k] = __fadd_rn(n[k], u[k]);
                const float l = __fsqrt_rn(__fadd_rn(
                    __fadd_rn(__fmul_rn(nd[0], nd[0]), __fmul_rn(nd[1], nd[1])), __fmul_rn(nd[2], nd[2])));
                if (l > 1e-6f) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) nd[k] = __fdiv_rn(nd[k], l);
                } else {
#pragma unroll
                    for (int k = 0; k < 3; ++k) nd[k] = n[k];
                }
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) nd[k] = n[k];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                o[k] = so[k];
                d[k] = nd[k];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[c] = __fadd_rn(sum[c], L[c]);
    }
    const float n = __uint2float_rn(P.spp);
#pragma unroll
    for (int c = 0; c < 3; ++c) sum[c] = __fdiv_rn(sum[c], n);
}

__global__ void __launch_bounds__(256) path_kernel(GridView g, vt_camera cam, PathParams P,
                                                   void* __restrict__ out,
                                                   unsigned long long* __restrict__ rays_out) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t px = blockIdx.x * 16 + (warp & 1u) * 8u + (lane & 7u);
    const uint32_t py = blockIdx.y * 16 + (warp >> 1) * 4u + (lane >> 3);
    uint32_t rays = 0;
    if (px < cam.width && py < cam.height) {
        float v[3];
        path_pixel(g, cam, P, px, py, v, rays);
        const size_t i = (size_t)py * cam.width + px;
        if (P.out_format == VT_PATH_OUT_F32X4) {
            ((float4*)out)[i] = make_float4(v[0], v[1], v[2], 1.0f);
        } else {
            uint32_t q = 0xFF000000u;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float x = v[c] > 1.0f ? 1.0f : (v[c] > 0.0f ? v[c] : 0.0f);
                q |= __float2uint_rz(__fadd_rn(__fmul_rn(x, 255.0f), 0.5f)) << (8 * c);
            }
            ((uint32_t*)out)[i] = q;
        }
    }
    if (rays_out) {
        // one atomic per warp
        unsigned long long r = rays;
#pragma unroll
        for (int k = 16; k > 0; k >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, k);
        if (lane == 0 && r) atomicAdd(rays_out, r);
    }
}


// ---------------------------------------------------------------------------------------------
// Persistent form: paths end after very different numbers of rays (escape at the first hit, or
// bounces plus sun rays), so one thread per pixel leaves most lanes idle.  Here resident warps
// hold one path per lane and advance every live lane by one traversal unit (vt_lane.cuh); a lane
// whose path ended takes the next path from a work counter (warp-aggregated).  Paths are numbered
// tile by tile (8 x 4 pixels), sample-major inside a tile, so a refill hands a warp one tile's
// rays for one sample.  Each path's radiance goes to a per-sample buffer; the resolve sums the
// samples of a pixel in sample order, so the image is identical to path_kernel's.
// ---------------------------------------------------------------------------------------------

struct PathLane {
    LaneRay R;
    float T[3], L[3];
    float so[3];      // origin of the next ray (hit point off the face)
    float nd[3];      // direction of a pending bounce ray
    uint32_t item;    // path index
    uint32_t px, py, s;
    uint32_t b;       // vertex index
    uint32_t face;    // face of the current vertex (for the bounce after a sun ray)
    int mode;         // 0 idle, 1 path ray, 2 sun ray
    int pend;         // ray to start: 0 none, 1 camera, 2 sun, 3 bounce
};

// A path vertex after the sun ray (or with none): queue the bounce ray, or end the path.
__device__ __forceinline__ void path_continue(const PathParams& P, PathLane& s,
                                              float4* __restrict__ samples) {
    if (s.b >= P.max_bounces) {
        samples[s.item] = make_float4(s.L[0], s.L[1], s.L[2], 0.0f);
        s.mode = 0;
        return;
    }
    const int a = (int)(s.face - 1) / 2;
    const bool npos = (s.face & 1u) != 0u;
    float n[3] = {0.0f, 0.0f, 0.0f};
    n[a] = npos ? 1.0f : -1.0f;
    float u[3];
    if (sphere_sample(P.seed, s.px, s.py, s.s, s.b, u)) {
#pragma unroll
        for (int k = 0; k < 3; ++k) s.nd[k] = __fadd_rn(n[k], u[k]);
        const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(s.nd[0], s.nd[0]),
                                                       __fmul_rn(s.nd[1], s.nd[1])),
                                             __fmul_rn(s.nd[2], s.nd[2])));
        if (l > 1e-6f) {
#pragma unroll
            for (int k = 0; k < 3; ++k) s.nd[k] = __fdiv_rn(s.nd[k], l);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) s.nd[k] = n[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) s.nd[k] = n[k];
    }
    ++s.b;
    s.mode = 1;
    s.pend = 3;
}

// The lane's ray ended with status `st`: shade the vertex and queue the next ray, or end the
// path.  Same arithmetic, in the same order, as path_pixel.
__device__ __forceinline__ void path_finish(const GridView& g, const PathParams& P, PathLane& s,
                                            int st, float4* __restrict__ samples) {
    if (s.mode == 2) {  // sun ray of vertex b
        if (st != kRayHit) {
            const int a = (int)(s.face - 1) / 2;
            const bool npos = (s.face & 1u) != 0u;
            const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
            const float ndl = npos ? la : -la;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                s.L[c] = __fadd_rn(s.L[c], __fmul_rn(__fmul_rn(s.T[c], P.sun[c]), ndl));
        }
        path_continue(P, s, samples);
        return;
    }
    // path ray of vertex b
    const HitRec h = ray_record(g, s.R, st, 0u);
    const uint32_t flags = h.w1 >> 24;
    const uint32_t face = flags & VT_FACE_MASK;
    if (!(flags & VT_HIT_FLAG_HIT) || face == 0) {
        if (!(flags & VT_HIT_FLAG_HIT)) {
#pragma unroll
            for (int c = 0; c < 3; ++c) s.L[c] = __fadd_rn(s.L[c], __fmul_rn(s.T[c], P.sky[c]));
        }
        samples[s.item] = make_float4(s.L[0], s.L[1], s.L[2], 0.0f);
        s.mode = 0;
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
        s.T[c] = __fmul_rn(s.T[c], __fdiv_rn(__uint2float_rn((h.w3 >> (8 * c)) & 0xFFu), 255.0f));
    s.face = face;
    shadow_origin(h, s.R.o, s.R.d, s.so);
    if (P.sun_on) {
        const int a = (int)(face - 1) / 2;
        const bool npos = (face & 1u) != 0u;
        const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
        if ((npos ? la : -la) > 0.0f) {
            s.mode = 2;
            s.pend = 2;
            return;
        }
    }
    path_continue(P, s, samples);
}

constexpr int kRayPending = 3;  // the lane has a ray queued in PathLane::pend

// ray_begin, the vertex shading and ray_unit each have one call site: lanes that start rays do so
// together, and the kernel stays small.  Four blocks of 256 per SM (64 registers; a few bytes of
// spill) measured faster than three without spill.

__global__ void __launch_bounds__(256, 4) path_persistent_kernel(
    GridView g, vt_camera cam, PathParams P, uint32_t s0, uint32_t sn, float4* __restrict__ samples,
    unsigned long long* __restrict__ counter, uint32_t tiles_x, uint64_t total,
    uint32_t refill_min, unsigned long long* __restrict__ rays_out) {
    const uint32_t lane = threadIdx.x & 31u;
    PathLane s;
    s.mode = 0;
    s.pend = 0;
    int st = kRayMiss;
    uint32_t rays = 0;
    bool more = true;  // warp-uniform
    for (;;) {
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, s.mode == 0);
        while (more && __popc(idle) >= (int)refill_min) {
            uint64_t item;
            const uint64_t base = warp_fetch(counter, idle, lane, item);
            if (base + __popc(idle) >= total) more = false;
            if (s.mode == 0 && item < total) {
                // item = (tile * sn + sample) * 32 + pixel of the tile
                const uint32_t l = (uint32_t)(item & 31u);
                const uint64_t ts = item >> 5;
                const uint32_t smp = (uint32_t)(ts % sn);
                const uint64_t tile = ts / sn;
                const uint32_t px = (uint32_t)(tile % tiles_x) * 8u + (l & 7u);
                const uint32_t py = (uint32_t)(tile / tiles_x) * 4u + (l >> 3);
                if (px < cam.width && py < cam.height) {
                    s.px = px;
                    s.py = py;
                    s.s = s0 + smp;
                    s.item = (uint32_t)(((size_t)py * cam.width + px) * sn + smp);
                    s.b = 0;
                    s.T[0] = s.T[1] = s.T[2] = 1.0f;
                    s.L[0] = s.L[1] = s.L[2] = 0.0f;
                    s.mode = 1;
                    s.pend = 1;
                    st = kRayPending;
                }
            }
            idle = __ballot_sync(0xFFFFFFFFu, s.mode == 0);
        }
        if (!more && idle == 0xFFFFFFFFu) break;
        // start queued rays and shade ended ones until every live lane has a running ray
        while (s.mode != 0 && st != kRayRunning) {
            if (s.pend != 0) {
                float o[3], d[3];
                if (s.pend == 1) {
                    float jx, jy;
                    jitter(P.seed, 0u, s.px, s.py, s.s, jx, jy);
                    raygen(cam, s.px, s.py, jx, jy, o, d);
                } else {
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        o[k] = s.so[k];
                        d[k] = s.pend == 2 ? P.sun_dir[k] : s.nd[k];
                    }
                }
                s.pend = 0;
                ++rays;
                st = ray_begin(g, o, d, s.R);
            } else {
                path_finish(g, P, s, st, samples);
                st = kRayPending;
            }
        }
        if (s.mode != 0) st = ray_unit(g, s.R);
    }
    if (rays_out) {
        unsigned long long r = rays;
#pragma unroll
        for (int k = 16; k > 0; k >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, k);
        if (lane == 0 && r) atomicAdd(rays_out, r);
    }
}

// Adds samples s0 .. s0 + sn - 1 of every pixel to its running sum in sample order; the last
// chunk divides by spp and writes the pixel.
__global__ void __launch_bounds__(256) path_resolve_kernel(const float4* __restrict__ samples,
                                                           float4* __restrict__ sums, uint32_t npx,
                                                           uint32_t sn, bool first, bool last,
                                                           uint32_t spp, uint32_t out_format,
                                                           void* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    float v[3] = {0.0f, 0.0f, 0.0f};
    if (!first) {
        const float4 q = sums[i];
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
    }
    for (uint32_t k = 0; k < sn; ++k) {
        const float4 q = samples[(size_t)i * sn + k];
        v[0] = __fadd_rn(v[0], q.x);
        v[1] = __fadd_rn(v[1], q.y);
        v[2] = __fadd_rn(v[2], q.z);
    }
    if (!last) {
        sums[i] = make_float4(v[0], v[1], v[2], 0.0f);
        return;
    }
    const float n = __uint2float_rn(spp);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = __fdiv_rn(v[c], n);
    if (out_format == VT_PATH_OUT_F32X4) {
        ((float4*)out)[i] = make_float4(v[0], v[1], v[2], 1.0f);
    } else {
        uint32_t q = 0xFF000000u;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float x = v[c] > 1.0f ? 1.0f : (v[c] > 0.0f ? v[c] : 0.0f);
            q |= __float2uint_rz(__fadd_rn(__fmul_rn(x, 255.0f), 0.5f)) << (8 * c);
        }
        ((uint32_t*)out)[i] = q;
    }
}

// Sample buffer of one chunk of samples: at most 16 samples per pixel and 64 Mi entries (1 GiB).
constexpr uint32_t kPathChunkSamples = 64u << 20, kPathChunkSpp = 16;

static int path_resident_blocks() {
    static int n = -1;
    if (n < 0) {
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, (const void*)path_persistent_kernel,
                                                          256, 0) != cudaSuccess) {
            cudaGetLastError();
            k = 1;
        }
        n = k < 1 ? 1 : k;
    }
    return n;
}

static cudaError_t launch_path_persistent(const GridView& g, const vt_camera& cam,
                                          const PathParams& P, void* out,
                                          unsigned long long* rays, const TraceTuning& tune,
                                          int sm_count, cudaStream_t st) {
    const uint32_t npx = cam.width * cam.height;
    const uint32_t tiles_x = (cam.width + 7) / 8, tiles_y = (cam.height + 3) / 4;
    // samples per chunk: as many as fit the sample buffer
    uint32_t sn = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>(std::min(P.spp, kPathChunkSpp), kPathChunkSamples / npx));
    const size_t sbytes = (size_t)npx * sn * sizeof(float4);
    const size_t sums_off = (sbytes + 255) / 256 * 256;
    const size_t total_bytes = sums_off + (size_t)npx * sizeof(float4) + 256;
    char* buf = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&buf, total_bytes, st);
    if (e != cudaSuccess) return e;
    float4* samples = (float4*)buf;
    float4* sums = (float4*)(buf + sums_off);
    const int bps = tune.blocks_per_sm > 0 ? min(tune.blocks_per_sm, path_resident_blocks())
                                           : path_resident_blocks();
    for (uint32_t s0 = 0; s0 < P.spp && e == cudaSuccess; s0 += sn) {
        const uint32_t n = std::min(sn, P.spp - s0);
        const uint64_t total = (uint64_t)tiles_x * tiles_y * n * 32;
        unsigned long long* counter = next_counter();
        e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) break;
        const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)sm_count * bps, (total + 255) / 256);
        path_persistent_kernel<<<blocks, 256, 0, st>>>(g, cam, P, s0, n, samples, counter, tiles_x,
                                                       total, tune.refill_min, rays);
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        path_resolve_kernel<<<(npx + 255) / 256, 256, 0, st>>>(samples, sums, npx, n, s0 == 0,
                                                               s0 + n >= P.spp, P.spp,
                                                               P.out_format, out);
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(buf, st);
    return e != cudaSuccess ? e : f;
}


// ---------------------------------------------------------------------------------------------
// Wavefront form: the paths of a chunk of samples advance one vertex at a time through ray
// queues.  Vertex 0 (camera ray, shading, sun ray) runs a thread per path in 8 x 4 pixel tiles;
// per vertex after that: trace the path rays, shade (sky on a miss; throughput, sun ray and
// bounce ray otherwise), trace the sun rays and add their light, the two ray queues traced by the
// persistent ray-buffer kernel.  Queues keep append order, which follows the pixel tiles:
// neighbouring entries start at neighbouring surface points (bucketing the bounce rays by
// direction octant and origin cell measured 9% slower in all).  Every path's radiance sees the
// same operations in the same order as path_pixel; queue order only changes speed.  Queue
// lengths stay on the device.
// ---------------------------------------------------------------------------------------------

struct WaveState {
    float T[3], L[3], so[3];
    uint32_t face;
    uint32_t pad[2];
};

constexpr uint64_t kWaveChunkPaths = 16u << 20;
constexpr uint32_t kWaveCounters = 256;  // 2 x 128 queue lengths: max_bounces <= 64

// Appends the lanes with `want` to a queue: one atomic per warp; every lane of the warp calls it.
__device__ __forceinline__ uint32_t wave_append(unsigned int* count, bool want) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, want);
    if (!ballot) return 0;
    const int leader = __ffs(ballot) - 1;
    unsigned int base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned int)__popc(ballot));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + __popc(ballot & ((1u << lane) - 1u));
}

__device__ __forceinline__ void wave_path_pixel(uint32_t p, uint32_t sn, uint32_t s0, uint32_t w,
                                                uint32_t& px, uint32_t& py, uint32_t& s) {
    const uint32_t i = p / sn;
    s = s0 + (p - i * sn);
    px = i % w;
    py = i / w;
}

// Direction of the bounce at vertex b of sample s of pixel (px, py), off the face with axis `a`
// and sign `npos`: the normalised sum of the normal and a unit vector uniform on the sphere (the
// normal itself when the sphere sample is rejected or the sum degenerates).  Same operations as
// path_pixel.
__device__ __forceinline__ void bounce_dir(const PathParams& P, uint32_t px, uint32_t py,
                                           uint32_t s, uint32_t b, int a, bool npos, float nd[3]) {
    float n3[3] = {0.0f, 0.0f, 0.0f}, u[3];
    n3[a] = npos ? 1.0f : -1.0f;
    if (sphere_sample(P.seed, px, py, s, b, u)) {
#pragma unroll
        for (int k = 0; k < 3; ++k) nd[k] = __fadd_rn(n3[k], u[k]);
        const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nd[0], nd[0]),
                                                       __fmul_rn(nd[1], nd[1])),
                                             __fmul_rn(nd[2], nd[2])));
        if (l > 1e-6f) {
#pragma unroll
            for (int k = 0; k < 3; ++k) nd[k] = __fdiv_rn(nd[k], l);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) nd[k] = n3[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) nd[k] = n3[k];
    }
}

// Vertex 0 of the chunk's paths, one thread per path in 8 x 4 pixel tiles (the render kernel's
// launch shape: the rays of a warp start together and stay coherent): camera ray, traversal,
// shading, the sun ray traced in the same thread (as the render kernel traces its shadow rays),
// and the bounce ray appended to the queue of vertex 1.
// Held to 48 registers: ten blocks per SM (0.4% shorter path frames than nine at 54).
__global__ void __launch_bounds__(128, 10) wave_primary_kernel(
    GridView g, vt_camera cam, PathParams P, uint32_t s0, uint32_t sn, uint32_t tiles_x,
    uint64_t total, vt_ray* __restrict__ nq, uint32_t* __restrict__ nqid,
    unsigned int* __restrict__ nqn, WaveState* __restrict__ st, float4* __restrict__ samples,
    unsigned long long* __restrict__ rays_out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false;
    uint32_t px = 0, py = 0, smp = 0;
    if (t < total) {  // t = (tile * sn + sample) * 32 + pixel of the 8 x 4 tile
        const uint32_t l = (uint32_t)(t & 31u);
        const uint64_t ts = t >> 5;
        smp = (uint32_t)(ts % sn);
        const uint64_t tile = ts / sn;
        px = (uint32_t)(tile % tiles_x) * 8u + (l & 7u);
        py = (uint32_t)(tile / tiles_x) * 4u + (l >> 3);
        valid = px < cam.width && py < cam.height;
    }
    bool bounce = false;
    uint32_t p = 0, nrays = 0;
    float so[3] = {0.0f, 0.0f, 0.0f}, nd[3] = {0.0f, 0.0f, 0.0f};
    float o[3], d[3];
    HitRec h;
    Tally<false> tl;
    if (valid) {
        p = (py * cam.width + px) * sn + smp;
        float jx, jy;
        jitter(P.seed, 0u, px, py, s0 + smp, jx, jy);
        raygen(cam, px, py, jx, jy, o, d);
        h = trace_ray<false>(g, o, d, tl);
    }
    __syncwarp();  // the warp's sun rays start together (fuller traversal passes)
    if (valid) {
        nrays = 1;
        float T[3] = {1.0f, 1.0f, 1.0f}, L[3] = {0.0f, 0.0f, 0.0f};
        const uint32_t flags = h.w1 >> 24;
        const uint32_t face = flags & VT_FACE_MASK;
        if (!(flags & VT_HIT_FLAG_HIT)) {
#pragma unroll
            for (int c = 0; c < 3; ++c) L[c] = __fadd_rn(L[c], __fmul_rn(T[c], P.sky[c]));
        } else if (face != 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                T[c] = __fmul_rn(T[c], __fdiv_rn(__uint2float_rn((h.w3 >> (8 * c)) & 0xFFu), 255.0f));
            shadow_origin(h, o, d, so);
            const int a = (int)(face - 1) / 2;
            const bool npos = (face & 1u) != 0u;
            if (P.sun_on) {
                const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
                const float ndl = npos ? la : -la;
                if (ndl > 0.0f) {
                    const HitRec sh = trace_ray<false>(g, so, P.sun_dir, tl);
                    ++nrays;
                    if (!((sh.w1 >> 24) & VT_HIT_FLAG_HIT)) {
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            L[c] = __fadd_rn(L[c], __fmul_rn(__fmul_rn(T[c], P.sun[c]), ndl));
                    }
                }
            }
            if (P.max_bounces > 0) {
                bounce = true;
                bounce_dir(P, px, py, s0 + smp, 0u, a, npos, nd);
            }
        }
        if (bounce) {
            WaveState& S = st[p];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                S.T[c] = T[c];
                S.L[c] = L[c];
            }
        } else {
            samples[p] = make_float4(L[0], L[1], L[2], 0.0f);
        }
    }
    const uint32_t kb = wave_append(nqn, bounce);
    if (bounce) {
        nq[kb] = vt_ray{{so[0], so[1], so[2]}, {nd[0], nd[1], nd[2]}};
        nqid[kb] = p;
    }
    if (rays_out) {
        const uint32_t wr = __reduce_add_sync(0xFFFFFFFFu, nrays);
        if ((threadIdx.x & 31u) == 0 && wr) atomicAdd(rays_out, (unsigned long long)wr);
    }
}

// Vertex b of every queued path: its ray ended with record h.
__global__ void __launch_bounds__(256) wave_shade_kernel(
    GridView g, PathParams P, uint32_t b, uint32_t s0, uint32_t sn, uint32_t w,
    const vt_ray* __restrict__ q, const uint32_t* __restrict__ qid,
    const unsigned int* __restrict__ qn, const uint4* __restrict__ hits,
    WaveState* __restrict__ st, float4* __restrict__ samples, vt_ray* __restrict__ sq,
    uint32_t* __restrict__ sid, unsigned int* __restrict__ sqn, vt_ray* __restrict__ nq,
    uint32_t* __restrict__ nqid, unsigned int* __restrict__ nqn,
    unsigned long long* __restrict__ rays_out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *qn;
    if (rays_out && j == 0) atomicAdd(rays_out, (unsigned long long)n);
    bool sun = false, bounce = false;
    uint32_t p = 0;
    float so[3] = {0.0f, 0.0f, 0.0f}, nd[3] = {0.0f, 0.0f, 0.0f};
    if (j < n) {
        p = qid[j];
        const uint4 hv = hits[j];
        HitRec h;
        h.w0 = hv.x;
        h.w1 = hv.y;
        h.w2 = hv.z;
        h.w3 = hv.w;
        WaveState& S = st[p];
        const uint32_t flags = h.w1 >> 24;
        const uint32_t face = flags & VT_FACE_MASK;
        if (!(flags & VT_HIT_FLAG_HIT) || face == 0) {
            if (!(flags & VT_HIT_FLAG_HIT)) {
#pragma unroll
                for (int c = 0; c < 3; ++c) S.L[c] = __fadd_rn(S.L[c], __fmul_rn(S.T[c], P.sky[c]));
            }
            samples[p] = make_float4(S.L[0], S.L[1], S.L[2], 0.0f);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                S.T[c] = __fmul_rn(S.T[c], __fdiv_rn(__uint2float_rn((h.w3 >> (8 * c)) & 0xFFu), 255.0f));
            const vt_ray r = q[j];
            shadow_origin(h, r.origin, r.dir, so);
#pragma unroll
            for (int c = 0; c < 3; ++c) S.so[c] = so[c];
            S.face = face;
            const int a = (int)(face - 1) / 2;
            const bool npos = (face & 1u) != 0u;
            if (P.sun_on) {
                const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
                sun = (npos ? la : -la) > 0.0f;
            }
            if (b < P.max_bounces) {
                bounce = true;
                uint32_t px, py, s;
                wave_path_pixel(p, sn, s0, w, px, py, s);
                bounce_dir(P, px, py, s, b, a, npos, nd);
            } else if (!sun) {
                samples[p] = make_float4(S.L[0], S.L[1], S.L[2], 0.0f);  // the path ends here
            }
        }
    }
    const uint32_t ks = wave_append(sqn, sun);
    if (sun) {
        sq[ks] = vt_ray{{so[0], so[1], so[2]}, {P.sun_dir[0], P.sun_dir[1], P.sun_dir[2]}};
        sid[ks] = p;
    }
    const uint32_t kb = wave_append(nqn, bounce);
    if (bounce) {
        nq[kb] = vt_ray{{so[0], so[1], so[2]}, {nd[0], nd[1], nd[2]}};
        nqid[kb] = p;
    }
}

// The sun rays of vertex b: light of the unblocked ones; paths ending at this vertex are done.
__global__ void __launch_bounds__(256) wave_sun_kernel(PathParams P, bool last,
                                                       const uint32_t* __restrict__ sid,
                                                       const unsigned int* __restrict__ sqn,
                                                       const uint4* __restrict__ hits,
                                                       WaveState* __restrict__ st,
                                                       float4* __restrict__ samples,
                                                       unsigned long long* __restrict__ rays_out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *sqn;
    if (rays_out && j == 0) atomicAdd(rays_out, (unsigned long long)n);
    if (j >= n) return;
    const uint32_t p = sid[j];
    WaveState& S = st[p];
    if (!((hits[j].y >> 24) & VT_HIT_FLAG_HIT)) {
        const int a = (int)(S.face - 1) / 2;
        const bool npos = (S.face & 1u) != 0u;
        const float la = a == 0 ? P.sun_dir[0] : (a == 1 ? P.sun_dir[1] : P.sun_dir[2]);
        const float ndl = npos ? la : -la;
#pragma unroll
        for (int c = 0; c < 3; ++c) S.L[c] = __fadd_rn(S.L[c], __fmul_rn(__fmul_rn(S.T[c], P.sun[c]), ndl));
    }
    if (last) samples[p] = make_float4(S.L[0], S.L[1], S.L[2], 0.0f);
}

static cudaError_t launch_path_wave(const GridView& g, const vt_camera& cam, const PathParams& P,
                                    void* out, unsigned long long* rays, int sm_count,
                                    cudaStream_t st) {
    const State& S = state();
    const uint32_t npx = cam.width * cam.height;
    const uint32_t tiles_x = (cam.width + 7) / 8, tiles_y = (cam.height + 3) / 4;
    const uint32_t sn = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>(std::min(P.spp, kPathChunkSpp), kWaveChunkPaths / npx));
    const uint64_t cap = (uint64_t)npx * sn;
    auto al = [](uint64_t v) { return (v + 255) / 256 * 256; };
    // q, nq, sq (rays); qid, nqid, sid; hits; state; samples; sums; counts
    const uint64_t o_q = 0, o_nq = al(cap * 24), o_sq = o_nq + al(cap * 24), o_qid = o_sq + al(cap * 24);
    const uint64_t o_nqid = o_qid + al(cap * 4), o_sid = o_nqid + al(cap * 4), o_hit = o_sid + al(cap * 4);
    const uint64_t o_st = o_hit + al(cap * 16), o_smp = o_st + al(cap * sizeof(WaveState));
    const uint64_t o_sum = o_smp + al(cap * 16), o_cnt = o_sum + al((uint64_t)npx * 16);
    const uint64_t total_bytes = o_cnt + kWaveCounters * 4;
    char* buf = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&buf, total_bytes, st);
    if (e != cudaSuccess) return e;
    vt_ray* q = (vt_ray*)(buf + o_q);
    vt_ray* nq = (vt_ray*)(buf + o_nq);
    vt_ray* sq = (vt_ray*)(buf + o_sq);
    uint32_t* qid = (uint32_t*)(buf + o_qid);
    uint32_t* nqid = (uint32_t*)(buf + o_nqid);
    uint32_t* sid = (uint32_t*)(buf + o_sid);
    uint4* hits = (uint4*)(buf + o_hit);
    WaveState* wst = (WaveState*)(buf + o_st);
    float4* samples = (float4*)(buf + o_smp);
    float4* sums = (float4*)(buf + o_sum);
    // lengths of the path queue of each vertex (one counter per vertex, so that the bounce queue
    // built at vertex b is the path queue of vertex b + 1 without a copy) and of the sun queues
    unsigned int* qn = (unsigned int*)(buf + o_cnt);
    unsigned int* sqn = qn + kWaveCounters / 2;
    const unsigned blocks = (unsigned)((cap + 255) / 256);
    for (uint32_t s0 = 0; s0 < P.spp && e == cudaSuccess; s0 += sn) {
        const uint32_t n = std::min(sn, P.spp - s0);
        const uint64_t items = (uint64_t)tiles_x * tiles_y * n * 32;
        e = cudaMemsetAsync(qn, 0, kWaveCounters * 4, st);
        if (e != cudaSuccess) break;
        wave_primary_kernel<<<(unsigned)((items + 127) / 128), 128, 0, st>>>(
            g, cam, P, s0, n, tiles_x, items, q, qid, qn + 1, wst, samples, rays);
        e = cudaGetLastError();
        for (uint32_t b = 1; b <= P.max_bounces && e == cudaSuccess; ++b) {
            // queue lengths: qn[b] paths at vertex b, qn[b + 1] bounce rays, sqn[b] sun rays
            unsigned int* cq = qn + b;
            unsigned int* cs = sqn + b;
            e = launch_trace_rays_persistent(g, q, cap, hits, next_counter(), S.tune_rays,
                                             sm_count, st, cq);
            if (e != cudaSuccess) break;
            wave_shade_kernel<<<blocks, 256, 0, st>>>(g, P, b, s0, n, cam.width, q, qid, cq, hits,
                                                      wst, samples, sq, sid, cs, nq, nqid, cq + 1,
                                                      rays);
            e = launch_trace_rays_persistent(g, sq, cap, hits, next_counter(), S.tune_rays,
                                             sm_count, st, cs);
            if (e != cudaSuccess) break;
            wave_sun_kernel<<<blocks, 256, 0, st>>>(P, b >= P.max_bounces, sid, cs, hits, wst,
                                                    samples, rays);
            // the bounce rays stay in the order the shading appended them, which follows the
            // path queue: neighbouring entries leave neighbouring surface points
            std::swap(q, nq);
            std::swap(qid, nqid);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        path_resolve_kernel<<<(npx + 255) / 256, 256, 0, st>>>(samples, sums, npx, n, s0 == 0,
                                                               s0 + n >= P.spp, P.spp,
                                                               P.out_format, out);
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(buf, st);
    return e != cudaSuccess ? e : f;
}

static int32_t path_params(const vt_path_params* in, PathParams& P) {
    if (!in) return fail(VT_EINVAL, "vt_path_trace: null params");
    if (in->spp < 1 || in->spp > 65536) return fail(VT_EINVAL, "vt_path_trace: spp must be 1..65536");
    if (in->max_bounces > 64) return fail(VT_EINVAL, "vt_path_trace: max_bounces must be 0..64");
    if (in->out_format != VT_PATH_OUT_F32X4 && in->out_format != VT_PATH_OUT_RGBA8)
        return fail(VT_EINVAL, "vt_path_trace: bad out_format");
    P.spp = in->spp;
    P.max_bounces = in->max_bounces;
    P.seed = in->seed;
    P.out_format = in->out_format;
    P.sun_on = false;
    for (int c = 0; c < 3; ++c) {
        if (!isfinite(in->sky[c]) || !isfinite(in->sun[c]) || !isfinite(in->sun_dir[c]))
            return fail(VT_EINVAL, "vt_path_trace: non-finite sky, sun or sun direction");
        P.sky[c] = in->sky[c];
        P.sun[c] = in->sun[c];
        P.sun_dir[c] = in->sun_dir[c];
        if (in->sun[c] > 0.0f) P.sun_on = true;
    }
    return VT_OK;
}

static cudaError_t launch_path(const GridView& g, const vt_camera& cam, const PathParams& P,
                               void* out, unsigned long long* rays, cudaStream_t st) {
    State& S = state();
    if (S.tune_path.wavefront) return launch_path_wave(g, cam, P, out, rays, S.sm_count, st);
    if (S.tune_path.persistent)
        return launch_path_persistent(g, cam, P, out, rays, S.tune_path, S.sm_count, st);
    const dim3 grid((cam.width + 15) / 16, (cam.height + 15) / 16);
    path_kernel<<<grid, 256, 0, st>>>(g, cam, P, out, rays);
    return cudaGetLastError();
}

// Pixel counts are 32-bit in the path kernels: a 65536 x 65536 image is refused.
static int32_t check_path_camera(const vt_camera* cam) {
    int32_t rc = check_camera(cam);
    if (rc) return rc;
    if ((uint64_t)cam->width * cam->height >= (1ull << 32))
        return fail(VT_ELIMIT, "vt_path_trace: 2^32 or more pixels");
    return VT_OK;
}

static size_t out_bytes(const vt_camera& cam, uint32_t fmt) {
    return (size_t)cam.width * cam.height * (fmt == VT_PATH_OUT_F32X4 ? 16 : 4);
}

}  // namespace vt

using namespace vt;

extern "C" {

int32_t vt_path_trace(int32_t grid, const vt_camera* camera, const vt_path_params* params,
                      void* d_out, uint64_t* d_rays_traced, void* stream) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_path_trace: unknown grid");
    int32_t rc = check_path_camera(camera);
    if (rc) return rc;
    PathParams P;
    if ((rc = path_params(params, P))) return rc;
    if (!d_out || ((uintptr_t)d_out & 15u)) return fail(VT_EINVAL, "vt_path_trace: output must be 16-byte aligned");
    if ((uintptr_t)d_rays_traced & 7u) return fail(VT_EINVAL, "vt_path_trace: misaligned ray counter");
    cudaError_t e = launch_path(g->view(), *camera, P, d_out, (unsigned long long*)d_rays_traced,
                                pick_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "vt_path_trace launch");
    return VT_OK;
}

int32_t vt_path_trace_host(int32_t grid, const vt_camera* camera, const vt_path_params* params,
                           void* out, uint64_t* rays_traced) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_path_trace_host: unknown grid");
    int32_t rc = check_path_camera(camera);
    if (rc) return rc;
    PathParams P;
    if ((rc = path_params(params, P))) return rc;
    if (!out) return fail(VT_EINVAL, "vt_path_trace_host: null output");
    const size_t bytes = out_bytes(*camera, P.out_format);
    State& s = state();
    cudaStream_t st = s.stream;
    void* mapped = host_mapped(out);  // page-locked output: the resolve kernel writes it directly
    const size_t dbytes = mapped ? 0 : bytes;
    void* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, dbytes + 256, st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_path_trace_host: cudaMallocAsync");
    unsigned long long* dr = (unsigned long long*)((char*)d + ((dbytes + 15) / 16) * 16);
    unsigned long long hr = 0;
    e = cudaMemsetAsync(dr, 0, 8, st);
    if (e == cudaSuccess) e = launch_path(g->view(), *camera, P, mapped ? mapped : d, dr, st);
    if (e == cudaSuccess && !mapped) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hr, dr, 8, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_path_trace_host");
    if (rays_traced) *rays_traced = hr;
    return VT_OK;
}

}  // extern "C"
