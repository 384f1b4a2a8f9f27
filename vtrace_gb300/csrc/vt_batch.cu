// vt_batch.cu — batched multi-view rendering: many cameras over many grids, uneven image sizes
// and sample counts, in one persistent work-stealing launch replayed from a captured CUDA graph.
//
// A batch flattens all its views into one item space: view v owns items [begin_v, begin_v +
// tiles_v * spp_v * 32), item = ((tile * spp + sample) * 32 + lane-in-tile), so a warp refill
// hands out neighbouring pixels of one tile and one sample (tiles of 8 x 4 pixels, or the tile
// shape the VT_KERNEL_BATCH tuning names).  Resident warps fetch items with one
// atomic per refill — whole 32-item units in the default tile form, per idle lane in the lane
// form (vt_lane.cuh) — find the item's view by binary search over the view table (held in shared
// memory), and trace it with the view's grid, camera and light.  Samples are
// jittered with Philox4x32-10 keyed by (seed, view id, pixel, sample), the same jitter the
// oracle uses.  The launch — counter reset plus kernel — is captured once into a CUDA graph at
// vt_batch_create and replayed by vt_batch_run.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "vt_api_internal.h"
#include "vt_batch.h"
#include "vt_device.cuh"
#include "vt_internal.h"
#include "vt_lane.cuh"

namespace vt {

// Lane state: kind 0 idle, 1 camera sample, 2 shadow ray of `prim`; pend 1 or 2 when that ray is
// queued but not started (ray_begin, batch_finish and ray_unit each have one call site, so lanes
// starting rays do so together).
struct BatchLane {
    LaneRay R;
    int kind, pend;
    uint32_t pix;     // sample record index in the view's output
    uint32_t px, py, sample;
    HitRec prim;
    float ndl;
    float so[3];      // origin of the queued shadow ray
    uint32_t view;
};

constexpr int kRayQueued = 3;

// A ray of the lane ended with `st`: write the sample record, or queue the shadow ray.
__device__ __forceinline__ void batch_finish(const BatchView& V, BatchLane& s, int st) {
    if (s.kind == 1) {
        HitRec h = ray_record(V.g, s.R, st, VT_SKY_RGBA);
        float nd;
        if (st != kRayHit || !V.light.enabled || !face_lit(h, V.light, nd)) {
            V.out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
            s.kind = 0;
            return;
        }
        if (nd > 0.0f && V.light.shadows) {
            shadow_origin(h, s.R.o, s.R.d, s.so);
            s.prim = h;
            s.ndl = nd;
            s.kind = 2;
            s.pend = 2;
            return;
        }
        h.w3 = shade_rgba(h.w3, nd, 1.0f, V.light.ambient);
        V.out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
        s.kind = 0;
        return;
    }
    const bool shadowed = st == kRayHit;
    HitRec h = s.prim;
    h.w3 = shade_rgba(h.w3, s.ndl, shadowed ? 0.0f : 1.0f, V.light.ambient);
    h.w1 |= (VT_HIT_FLAG_SHADOW_RAY | (shadowed ? VT_HIT_FLAG_SHADOWED : 0u)) << 24;
    V.out[s.pix] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    s.kind = 0;
}

__global__ void __launch_bounds__(256, 4) batch_kernel(const BatchView* __restrict__ table,
                                                    uint32_t nviews, uint64_t total,
                                                    unsigned long long* __restrict__ counter,
                                                    uint32_t refill_min) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchView* views = reinterpret_cast<BatchView*>(smem_raw);
    {
        const uint32_t words = nviews * (uint32_t)(sizeof(BatchView) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(table);
        uint32_t* dst = reinterpret_cast<uint32_t*>(smem_raw);
        for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u;
    BatchLane s;
    s.kind = 0;
    s.pend = 0;
    s.pix = 0;
    s.ndl = 0.0f;
    s.view = 0;
    int st = kRayMiss;
    bool more = true;
    for (;;) {
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, s.kind == 0);
        while (more && __popc(idle) >= (int)refill_min) {
            uint64_t item;
            const uint64_t base = warp_fetch(counter, idle, lane, item);
            if (base + __popc(idle) >= total) more = false;
            if (s.kind == 0 && item < total) {
                // the view owning the item: last view with begin <= item
                uint32_t lo = 0, hi = nviews - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (views[mid].begin <= item)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                const BatchView& V = views[lo];
                const uint64_t local = item - V.begin + V.first_item;
                const uint64_t ts = local >> 5;
                const uint32_t l = (uint32_t)local & 31u;
                const uint64_t tile = ts / V.spp;
                const uint32_t sample = (uint32_t)(ts - tile * V.spp);
                const uint32_t px = ((uint32_t)(tile % V.tiles_x) << V.wx_log) + (l & ((1u << V.wx_log) - 1u));
                const uint32_t py = (uint32_t)(tile / V.tiles_x) * (32u >> V.wx_log) + (l >> V.wx_log);
                if (px < V.cam.width && py < V.cam.height) {
                    s.view = lo;
                    s.px = px;
                    s.py = py;
                    s.sample = sample;
                    s.pix = ((py * V.cam.width) + px) * V.spp + sample - V.rec_offset;
                    s.kind = 1;
                    s.pend = 1;
                    st = kRayQueued;
                }
            }
            idle = __ballot_sync(0xFFFFFFFFu, s.kind == 0);
        }
        if (!more && idle == 0xFFFFFFFFu) break;
        while (s.kind != 0 && st != kRayRunning) {
            const BatchView& V = views[s.view];
            if (s.pend != 0) {
                float o[3], d[3];
                if (s.pend == 1) {
                    float jx, jy;
                    jitter(V.seed, V.view_id, s.px, s.py, s.sample, jx, jy);
                    raygen(V.cam, s.px, s.py, jx, jy, o, d);
                } else {
#pragma unroll
                    for (int k = 0; k < 3; ++k) o[k] = s.so[k];
                    d[0] = V.light.dx;
                    d[1] = V.light.dy;
                    d[2] = V.light.dz;
                }
                s.pend = 0;
                st = ray_begin(V.g, o, d, s.R);
            } else {
                batch_finish(V, s, st);
                st = kRayQueued;
            }
        }
        if (s.kind != 0) st = ray_unit(views[s.view].g, s.R);
    }
}

// Tile form (refill_min 32, the default): resident warps take whole (pixel tile, sample) units —
// 32 items of one view; 8 x 4 pixels unless the VT_KERNEL_BATCH tuning names another tile shape
// when the batch is created — from the counter, one atomic per unit, and trace each lane's camera ray
// and shadow ray to the end in the lane (the render kernel's traversal), so that a warp's rays
// start together and no lane state is kept between units.  Same item order and records as the
// lane form with whole-warp refills, 23% faster on the 64-view workload.
constexpr int kBatchTileThreads = 128;

// STATS: the counting build (every reference iteration walked, traversal counters gathered into
// `counters`; same records), for the roofline's algorithmic bytes.
template <bool STATS>
__global__ void __launch_bounds__(kBatchTileThreads) batch_tile_kernel(const BatchView* __restrict__ table,
                                                         uint32_t nviews, uint64_t units,
                                                         unsigned long long* __restrict__ counter,
                                                         Counters* __restrict__ counters) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchView* views = reinterpret_cast<BatchView*>(smem_raw);
    {
        const uint32_t words = nviews * (uint32_t)(sizeof(BatchView) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(table);
        uint32_t* dst = reinterpret_cast<uint32_t*>(smem_raw);
        for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u;
    Tally<STATS> tl;
    for (;;) {
        unsigned long long u = 0;
        if (lane == 0) u = atomicAdd(counter, 1ull);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        if (u >= units) break;
        const uint64_t item = u * 32u + lane;  // views begin at multiples of 32 items
        uint32_t lo = 0, hi = nviews - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (views[mid].begin <= item)
                lo = mid;
            else
                hi = mid - 1;
        }
        const BatchView& V = views[lo];
        const uint64_t local = item - V.begin + V.first_item;
        const uint64_t ts = local >> 5;
        const uint64_t tile = ts / V.spp;
        const uint32_t sample = (uint32_t)(ts - tile * V.spp);
        const uint32_t px = ((uint32_t)(tile % V.tiles_x) << V.wx_log) + (lane & ((1u << V.wx_log) - 1u));
        const uint32_t py = (uint32_t)(tile / V.tiles_x) * (32u >> V.wx_log) + (lane >> V.wx_log);
        if (px < V.cam.width && py < V.cam.height) {
            float jx, jy, o[3], d[3];
            jitter(V.seed, V.view_id, px, py, sample, jx, jy);
            raygen(V.cam, px, py, jx, jy, o, d);
            const HitRec h = shade_ray<STATS>(V.g, V.light, o, d, tl);
            V.out[((py * V.cam.width) + px) * V.spp + sample - V.rec_offset] =
                make_uint4(h.w0, h.w1, h.w2, h.w3);
        }
    }
    if (STATS) tl.flush(counters);
}

static bool batch_tile_form(const TraceTuning& tune) { return tune.refill_min >= 32; }

struct Batch {
    std::vector<int32_t> grids;  // referenced grid ids (refcounted while the batch lives)
    BatchView* d_table = nullptr;
    unsigned long long* d_counter = nullptr;
    uint32_t nviews = 0;
    uint64_t total = 0;
    uint64_t rays_primary = 0;
    TraceTuning tune;
    unsigned blocks = 0;
    size_t smem = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static std::mutex g_batch_mu;
static std::vector<std::unique_ptr<Batch>> g_batches;

static void batch_free(Batch& b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    cudaFree(b.d_table);
    cudaFree(b.d_counter);
    for (int32_t id : b.grids) {
        Grid* g = lookup_grid(id);
        if (g) g->refs.fetch_sub(1);
    }
    b.exec = nullptr;
    b.graph = nullptr;
    b.d_table = nullptr;
    b.d_counter = nullptr;
    b.grids.clear();
}

uint32_t tile_wx_log(uint32_t tile_shape) {
    static const uint32_t kLog[4] = {3, 2, 4, 5};  // VT_TILE_8X4, 4X8, 16X2, 32X1
    return tile_shape < 4 ? kLog[tile_shape] : 3u;
}

uint64_t batch_view_items(const vt_camera& cam, uint32_t spp, uint32_t wx_log) {
    return batch_rows_items(cam, spp, 0, cam.height, wx_log);
}

uint64_t batch_rows_items(const vt_camera& cam, uint32_t spp, uint32_t row0, uint32_t row1,
                          uint32_t wx_log) {
    const uint32_t th = 32u >> wx_log, tw = 1u << wx_log;
    const uint64_t tile_rows = (uint64_t)((row1 + th - 1) / th) - row0 / th;
    return tile_rows * ((cam.width + tw - 1) / tw) * spp * 32;
}

BatchView make_batch_view(const Grid& g, const vt_camera& cam, const vt_light* light,
                          uint32_t spp, uint32_t seed, uint32_t view_id, void* out,
                          uint64_t begin, uint32_t row0, uint32_t wx_log) {
    BatchView T;
    memset(&T, 0, sizeof(T));
    T.g = g.view();
    T.cam = cam;
    T.light = light_view(light);
    T.out = (uint4*)out;
    T.begin = begin;
    T.first_item = batch_rows_items(cam, spp, 0, row0, wx_log);
    T.rec_offset = row0 * cam.width * spp;
    T.wx_log = wx_log;
    T.tiles_x = (cam.width + (1u << wx_log) - 1) >> wx_log;
    T.spp = spp;
    T.seed = seed;
    T.view_id = view_id;
    return T;
}

unsigned batch_blocks(uint32_t n, uint64_t total, const TraceTuning& tune) {
    const size_t smem = (size_t)n * sizeof(BatchView);
    // a full table (256 views x 208 B) is above the 48 KiB of dynamic shared memory a launch
    // gets without opting in; set on every call (cheap), so that a re-created context has it too
    const int table_max = (int)(kMaxBatchViews * sizeof(BatchView));
    if (cudaFuncSetAttribute((const void*)batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             table_max) != cudaSuccess ||
        cudaFuncSetAttribute((const void*)batch_tile_kernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, table_max) != cudaSuccess ||
        cudaFuncSetAttribute((const void*)batch_tile_kernel<true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, table_max) != cudaSuccess)
        cudaGetLastError();
    int per_sm = 0;
    const void* kernel =
        batch_tile_form(tune) ? (const void*)batch_tile_kernel<false> : (const void*)batch_kernel;
    const int threads = batch_tile_form(tune) ? kBatchTileThreads : 256;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    if (tune.blocks_per_sm > 0) per_sm = std::min(per_sm, tune.blocks_per_sm);
    const uint64_t need = (total + threads - 1) / threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)state().sm_count * per_sm, need));
}

cudaError_t launch_batch(const BatchView* d_table, uint32_t n, uint64_t total,
                         unsigned long long* counter, const TraceTuning& tune, unsigned blocks,
                         cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    if (batch_tile_form(tune))
        batch_tile_kernel<false><<<blocks, kBatchTileThreads, (size_t)n * sizeof(BatchView), stream>>>(
            d_table, n, total / 32, counter, nullptr);
    else
        batch_kernel<<<blocks, 256, (size_t)n * sizeof(BatchView), stream>>>(d_table, n, total,
                                                                             counter, tune.refill_min);
    return cudaGetLastError();
}

static cudaError_t batch_launch(const Batch& b, cudaStream_t stream) {
    return launch_batch(b.d_table, b.nviews, b.total, b.d_counter, b.tune, b.blocks, stream);
}

}  // namespace vt

using namespace vt;

void vt_batch_release_all() {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    for (auto& b : g_batches)
        if (b) batch_free(*b);
    g_batches.clear();
}

extern "C" {

int32_t vt_batch_create(const vt_view* views, uint32_t n, int32_t* batch_out) {
    if (!views || !batch_out || n == 0) return fail(VT_EINVAL, "vt_batch_create: no views");
    if (n > kMaxBatchViews) return fail(VT_ELIMIT, "vt_batch_create: more than 256 views");
    int32_t rc = ensure_init();
    if (rc) return rc;
    State& st = state();
    std::unique_ptr<Batch> b(new Batch());
    std::vector<BatchView> table(n);
    uint64_t begin = 0;
    const uint32_t wx_log = tile_wx_log(st.tune_batch.tile_shape);
    for (uint32_t i = 0; i < n; ++i) {
        const vt_view& v = views[i];
        Grid* g = lookup_grid(v.grid);
        if (!g) {
            batch_free(*b);
            return fail(VT_ENOTFOUND, "vt_batch_create: unknown grid in view " + std::to_string(i));
        }
        if ((rc = check_camera(&v.camera))) {
            batch_free(*b);
            return rc;
        }
        if (v.spp == 0 || v.spp > 64 || !v.d_out || ((uintptr_t)v.d_out & 15u)) {
            batch_free(*b);
            return fail(VT_EINVAL, "vt_batch_create: view " + std::to_string(i) +
                                       " needs spp in 1..64 and a 16-byte aligned output");
        }
        if ((uint64_t)v.camera.width * v.camera.height * v.spp >= (1ull << 32)) {
            batch_free(*b);  // sample records are indexed with 32 bits
            return fail(VT_ELIMIT, "vt_batch_create: view " + std::to_string(i) +
                                       " has 2^32 or more samples");
        }
        // device memory as given; page-locked host memory through its device address (the
        // kernel writes the records over the host link); anything else is refused rather than
        // handed to a kernel that could not reach it
        void* out = device_address(v.d_out);
        if (!out) {
            batch_free(*b);
            return fail(VT_EINVAL, "vt_batch_create: view " + std::to_string(i) +
                                       " output is neither device nor page-locked host memory");
        }
        g->refs.fetch_add(1);
        b->grids.push_back(v.grid);
        table[i] = make_batch_view(*g, v.camera, (v.flags & VT_VIEW_LIGHT) ? &v.light : nullptr,
                                   v.spp, v.seed, v.view_id, out, begin, 0, wx_log);
        begin += batch_view_items(v.camera, v.spp, wx_log);
        b->rays_primary += (uint64_t)v.camera.width * v.camera.height * v.spp;
    }
    b->nviews = n;
    b->total = begin;
    b->tune = st.tune_batch;
    b->smem = (size_t)n * sizeof(BatchView);
    b->blocks = batch_blocks(n, b->total, b->tune);
    cudaError_t e;
    if (cudaMalloc(&b->d_table, b->smem) != cudaSuccess ||
        cudaMalloc(&b->d_counter, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        batch_free(*b);
        return fail(VT_ENOMEM, "vt_batch_create: cudaMalloc failed");
    }
    e = cudaMemcpy(b->d_table, table.data(), b->smem, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        batch_free(*b);
        return cuda_fail(e, "vt_batch_create: table upload");
    }
    // capture counter reset + kernel into a graph on a private stream
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t le = batch_launch(*b, cs);
            e = cudaStreamEndCapture(cs, &b->graph);
            if (e == cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        cudaStreamDestroy(cs);
    }
    if (e != cudaSuccess) {
        batch_free(*b);
        return cuda_fail(e, "vt_batch_create: graph capture");
    }
    std::lock_guard<std::mutex> lk(g_batch_mu);
    for (size_t i = 0; i < g_batches.size(); ++i)
        if (!g_batches[i]) {
            g_batches[i] = std::move(b);
            *batch_out = (int32_t)i;
            return VT_OK;
        }
    g_batches.push_back(std::move(b));
    *batch_out = (int32_t)(g_batches.size() - 1);
    return VT_OK;
}

static Batch* lookup_batch(int32_t id) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (id < 0 || (size_t)id >= g_batches.size() || !g_batches[id]) return nullptr;
    return g_batches[id].get();
}

int32_t vt_batch_run(int32_t batch, void* stream) {
    Batch* b = lookup_batch(batch);
    if (!b) return fail(VT_ENOTFOUND, "vt_batch_run: unknown batch");
    cudaError_t e = cudaGraphLaunch(b->exec, pick_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "vt_batch_run: graph launch");
    return VT_OK;
}

int32_t vt_batch_run_direct(int32_t batch, void* stream) {
    Batch* b = lookup_batch(batch);
    if (!b) return fail(VT_ENOTFOUND, "vt_batch_run_direct: unknown batch");
    cudaError_t e = batch_launch(*b, pick_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "vt_batch_run_direct: launch");
    return VT_OK;
}

int32_t vt_batch_stats(int32_t batch, vt_trace_stats* stats) {
    Batch* b = lookup_batch(batch);
    if (!b) return fail(VT_ENOTFOUND, "vt_batch_stats: unknown batch");
    if (!stats) return fail(VT_EINVAL, "vt_batch_stats: null output");
    cudaStream_t st = state().stream;
    void* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(Counters) + sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "vt_batch_stats: cudaMalloc(counters)");
    }
    Counters* dc = (Counters*)buf;
    unsigned long long* cursor = (unsigned long long*)((char*)buf + sizeof(Counters));
    Counters hc;
    cudaError_t e = cudaMemsetAsync(buf, 0, sizeof(Counters) + sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        // the counting build always runs in the tile form (same records as either form)
        TraceTuning tile = b->tune;
        tile.refill_min = 32;
        const unsigned blocks = batch_blocks(b->nviews, b->total, tile);
        batch_tile_kernel<true><<<blocks, kBatchTileThreads, b->smem, st>>>(
            b->d_table, b->nviews, b->total / 32, cursor, dc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "vt_batch_stats");
    stats_from(hc, stats);
    return VT_OK;
}

int32_t vt_batch_info(int32_t batch, uint64_t* primary_rays, uint64_t* work_items) {
    Batch* b = lookup_batch(batch);
    if (!b) return fail(VT_ENOTFOUND, "vt_batch_info: unknown batch");
    if (primary_rays) *primary_rays = b->rays_primary;
    if (work_items) *work_items = b->total;
    return VT_OK;
}

int32_t vt_batch_destroy(int32_t batch) {
    std::unique_ptr<Batch> b;
    {
        std::lock_guard<std::mutex> lk(g_batch_mu);
        if (batch < 0 || (size_t)batch >= g_batches.size() || !g_batches[batch])
            return fail(VT_ENOTFOUND, "vt_batch_destroy: unknown batch");
        b = std::move(g_batches[batch]);
    }
    cudaStreamSynchronize(state().stream);
    cudaDeviceSynchronize();
    batch_free(*b);
    return VT_OK;
}

}  // extern "C"
