// vt_api.cu — C ABI of libvtrace: library state, grid table, tracing and rendering calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdio.h>
#include <string.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "vt_api_internal.h"
#include "vt_device.cuh"
#include "vt_internal.h"
#include "vt_kernels.h"

namespace vt {

static thread_local std::string g_last_error;

int32_t fail(int32_t code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
void clear_error() { g_last_error.clear(); }

int32_t cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(VT_ECUDA, m);
}

State& state() {
    static State s;
    return s;
}

int32_t ensure_init_locked(int32_t device) {
    State& s = state();
    if (s.inited) return VT_OK;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    for (int k = 0; k < State::kAux; ++k) {
        e = cudaStreamCreateWithFlags(&s.aux[k], cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate(aux)");
    }
    e = cudaEventCreateWithFlags(&s.aux_start, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    e = cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    e = cudaMalloc(&s.counters, kCounterRing * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(work counters)");
    // stream-ordered temporaries (build scratch, uploads, path-tracing queues) come from the
    // device's default pool; keep up to 4 GiB of freed pool memory for the next call instead
    // of returning it at every synchronisation (a process-local setting of this context)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = 4ull << 30;
        if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess)
            cudaGetLastError();
    } else {
        cudaGetLastError();
    }
    s.device = device;
    s.inited = true;
    return VT_OK;
}

int32_t ensure_init() {
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    return ensure_init_locked(0);
}

unsigned long long* next_counter() {
    State& s = state();
    return s.counters + (s.counter_next.fetch_add(1) % kCounterRing);
}

cudaError_t launch_frame(const GridView& g, const vt_camera& cam, const LightView& light,
                         uint4* out, cudaStream_t stream) {
    State& s = state();
    if (s.tune_render.persistent && s.tune_render.wavefront)
        return launch_render_queued(g, cam, light, out, next_counter(), s.tune_render, s.sm_count,
                                    stream);
    if (s.tune_render.persistent)
        return launch_render_persistent(g, cam, light, out, next_counter(), s.tune_render,
                                        s.sm_count, stream);
    if (s.tune_render.wavefront) return launch_render_wavefront(g, cam, light, out, stream);
    return launch_render(g, cam, light, out, nullptr, stream, 0, 0, &s.tune_render);
}

cudaError_t launch_rays(const GridView& g, const vt_ray* rays, uint64_t n, uint4* out,
                        cudaStream_t stream) {
    State& s = state();
    if (s.tune_rays.persistent)
        return launch_trace_rays_persistent(g, rays, n, out, next_counter(), s.tune_rays,
                                            s.sm_count, stream);
    return launch_trace_rays(g, rays, n, out, nullptr, stream);
}

cudaStream_t pick_stream(void* stream) {
    return stream ? (cudaStream_t)stream : state().stream;
}

GridView Grid::view() const {
    GridView v;
    v.dir = dir;
    v.oct = oct;
    v.lng = lng;
    v.bricks = (uint32_t)bricks;
    v.masks = masks;
    v.payload8 = format == VT_PAYLOAD_U8 ? (const uint8_t*)payload : nullptr;
    v.payload32 = format == VT_PAYLOAD_RGBA8 ? (const uint32_t*)payload : nullptr;
    v.palette = palette;
    v.nx = (int32_t)nx;
    v.ny = (int32_t)ny;
    v.nz = (int32_t)nz;
    v.bx = (int32_t)bx;
    v.by = (int32_t)by;
    v.bz = (int32_t)bz;
    v.max_steps = nx + ny + nz;
    v.format = format;
    return v;
}

bool Grid::in_block(const void* p) const {
    return block && p >= block && (const char*)p < (const char*)block + block_bytes;
}

void Grid::free_slot_arrays() {
    if (!in_block(masks)) cudaFree(masks);
    if (!in_block(payload)) cudaFree(payload);
    masks = nullptr;
    payload = nullptr;
}

void Grid::release() {
    free_slot_arrays();
    // directory, octant and long-box words, palette (and the first slot arrays)
    if (block && pooled) {
        cudaDeviceSynchronize();
        cudaFreeAsync(block, state().stream);
    } else {
        cudaFree(block);
    }
    pooled = false;
    block = nullptr;
    block_bytes = 0;
    dir = nullptr;
    oct = nullptr;
    lng = nullptr;
    palette = nullptr;
}

int32_t check_dims(uint32_t nx, uint32_t ny, uint32_t nz) {
    if (nx == 0 || ny == 0 || nz == 0)
        return fail(VT_EINVAL, "grid dimensions must be nonzero");
    if (nx > kMaxDim || ny > kMaxDim || nz > kMaxDim)
        return fail(VT_EINVAL, "grid dimension above 65535 (hit records hold 16-bit coordinates)");
    const uint64_t bricks = (uint64_t)((nx + 7) / 8) * ((ny + 7) / 8) * ((nz + 7) / 8);
    if (bricks > 0x7FFFFFF0ull) return fail(VT_EINVAL, "grid has more than 2^31 bricks");
    return VT_OK;
}

// One device allocation per grid: directory, octant words, long-box words, palette, masks and
// payloads of `slots` slots, each part 256-byte aligned.
struct BlockLayout {
    size_t oct, lng, pal, msk, pay, total;
};

static BlockLayout block_layout(uint64_t bricks, uint64_t slots, uint32_t format) {
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    const size_t psize = format == VT_PAYLOAD_U8 ? 512 : 2048;
    BlockLayout L;
    L.oct = al(bricks * 4);
    L.lng = L.oct + al(bricks * 4);
    L.pal = L.lng + al(bricks * 12);
    L.msk = L.pal + 1024;
    L.pay = L.msk + al(slots * 64);
    L.total = L.pay + al(slots * psize);
    return L;
}

uint64_t grid_bytes_bound(uint64_t bricks, uint32_t format) {
    return block_layout(bricks, bricks, format).total;
}

static void point_into_block(Grid& g, void* block, const BlockLayout& L, uint64_t slots) {
    char* b = (char*)block;
    g.block = block;
    g.block_bytes = L.total;
    g.dir = (uint32_t*)b;
    g.oct = (uint32_t*)(b + L.oct);
    g.lng = (uint32_t*)(b + L.lng);
    g.palette = g.format == VT_PAYLOAD_U8 ? (uint32_t*)(b + L.pal) : nullptr;
    g.masks = (uint64_t*)(b + L.msk);
    g.payload = b + L.pay;
    g.slot_capacity = slots;
}

// The brick build's launches on `stream` (captured or not): occupancy words, slot scan, compaction
// into dir / masks / payload, distance field, octant words, long-box words.
static cudaError_t build_launches(const void* d_src, uint32_t format, const uint32_t* d_palette,
                                  bool nonzero, const Grid& g, const BuildScratch& s,
                                  cudaStream_t stream) {
    const int32_t nx = (int32_t)g.nx, ny = (int32_t)g.ny, nz = (int32_t)g.nz;
    cudaError_t e = launch_brick_words(d_src, format, d_palette, nx, ny, nz, s, stream, nonzero);
    if (e == cudaSuccess) e = launch_brick_scan(s, g.bricks, stream);
    if (e == cudaSuccess)
        e = launch_brick_compact(d_src, format, nx, ny, nz, s, g.dir, g.masks, g.payload, stream);
    // the occupancy words are no longer needed: their scratch (16 words per brick) holds the
    // occupancy bitmask of the passes along x (words 13 on), the octant passes, and then the
    // long-box runs and window minima (words 0-12)
    uint32_t* occ = (uint32_t*)s.words + 13 * g.bricks;
    if (e == cudaSuccess)
        e = launch_brick_xmask(g.dir, occ, (int32_t)g.bx, (int32_t)g.by, (int32_t)g.bz, stream);
    if (e == cudaSuccess)
        e = launch_brick_distance(s, g.dir, (int32_t)g.bx, (int32_t)g.by, (int32_t)g.bz, stream,
                                  nullptr, occ);
    if (e == cudaSuccess)
        e = launch_brick_octants(g.dir, (uint8_t*)s.words,
                                 (uint16_t*)((uint8_t*)s.words + ((g.bricks + 255) / 256) * 256),
                                 g.oct, (int32_t)g.bx, (int32_t)g.by, (int32_t)g.bz, stream,
                                 nullptr, occ);
    if (e == cudaSuccess)
        e = launch_brick_long(g.dir, g.oct, (uint32_t*)s.words, g.lng, (int32_t)g.bx,
                              (int32_t)g.by, (int32_t)g.bz, stream, nullptr, occ);
    return e;
}

// ---------------------------------------------------------------------------------------------
// Small grids (vtrace's 16^3 chunk textures, .vox models): the build's twenty-odd launches cost
// more than their work, so they are captured once per grid shape into a CUDA graph that reads a
// fixed input buffer and builds into a fixed template of the grid's allocation (every brick has a
// slot).  A build copies its voxels in, replays the graph, and copies the template into the new
// grid's allocation.  Builds of small grids are serialised by g_small_mu.
// ---------------------------------------------------------------------------------------------
constexpr uint64_t kSmallGridBricks = 512;  // 64^3 voxels: at most 1 MiB of unused slots
constexpr size_t kSmallGraphs = 64;

struct SmallBuild {
    uint32_t nx = 0, ny = 0, nz = 0, format = 0;
    bool nonzero = false;
    void* in = nullptr;          // the shape's dense voxels
    void* tmpl = nullptr;        // block layout with a slot per brick
    void* scratch = nullptr;
    uint32_t* counts = nullptr;  // last slot offset, last flag, occupied voxels (u64)
    cudaGraphExec_t exec = nullptr;
    uint64_t last_use = 0;
};

static std::mutex g_small_mu;
static std::vector<SmallBuild> g_small;
static uint64_t g_small_clock = 0;

static void small_free(SmallBuild& b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    cudaFree(b.in);
    cudaFree(b.tmpl);
    cudaFree(b.scratch);
    cudaFree(b.counts);
    b = SmallBuild();
}

void release_small_builds() {
    std::lock_guard<std::mutex> lk(g_small_mu);
    for (SmallBuild& b : g_small) small_free(b);
    g_small.clear();
}

static int32_t small_entry(const Grid& shape, bool nonzero, SmallBuild*& out) {
    for (SmallBuild& b : g_small)
        if (b.nx == shape.nx && b.ny == shape.ny && b.nz == shape.nz && b.format == shape.format &&
            b.nonzero == nonzero) {
            out = &b;
            return VT_OK;
        }
    if (g_small.size() >= kSmallGraphs) {  // drop the least recently used shape
        size_t old = 0;
        for (size_t i = 1; i < g_small.size(); ++i)
            if (g_small[i].last_use < g_small[old].last_use) old = i;
        small_free(g_small[old]);
        g_small.erase(g_small.begin() + (long)old);
    }
    SmallBuild b;
    b.nx = shape.nx;
    b.ny = shape.ny;
    b.nz = shape.nz;
    b.format = shape.format;
    b.nonzero = nonzero;
    const size_t elem = shape.format == VT_PAYLOAD_U8 ? 1 : 4;
    const BlockLayout L = block_layout(shape.bricks, shape.bricks, shape.format);
    if (cudaMalloc(&b.in, (size_t)shape.nx * shape.ny * shape.nz * elem) != cudaSuccess ||
        cudaMalloc(&b.tmpl, L.total) != cudaSuccess ||
        cudaMalloc(&b.scratch, build_scratch_bytes(shape.bricks)) != cudaSuccess ||
        cudaMalloc(&b.counts, 16) != cudaSuccess) {
        cudaGetLastError();
        small_free(b);
        return fail(VT_ENOMEM, "cudaMalloc(small grid build) failed");
    }
    Grid t;  // the template's view of the layout
    t.nx = shape.nx;
    t.ny = shape.ny;
    t.nz = shape.nz;
    t.bx = shape.bx;
    t.by = shape.by;
    t.bz = shape.bz;
    t.bricks = shape.bricks;
    t.format = shape.format;
    point_into_block(t, b.tmpl, L, shape.bricks);
    const BuildScratch s = carve_build_scratch(b.scratch, shape.bricks);
    cudaStream_t cs;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t le = build_launches(b.in, shape.format, t.palette, nonzero, t, s, cs);
            if (le == cudaSuccess)
                le = cudaMemcpyAsync(b.counts, s.offsets + (shape.bricks - 1), 4,
                                     cudaMemcpyDeviceToDevice, cs);
            if (le == cudaSuccess)
                le = cudaMemcpyAsync(b.counts + 1, s.flags + (shape.bricks - 1), 4,
                                     cudaMemcpyDeviceToDevice, cs);
            if (le == cudaSuccess)
                le = cudaMemcpyAsync(b.counts + 2, s.occupied, 8, cudaMemcpyDeviceToDevice, cs);
            e = cudaStreamEndCapture(cs, &graph);
            if (e == cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
    }
    t.block = nullptr;  // the template belongs to the cache entry
    if (e != cudaSuccess) {
        small_free(b);
        return cuda_fail(e, "small grid build graph");
    }
    g_small.push_back(b);
    out = &g_small.back();
    return VT_OK;
}

// `src`: the dense voxels, in device memory, or in host memory when `src_host`.
static int32_t build_small(const void* src, bool src_host, const uint32_t* palette_host,
                           bool nonzero, std::unique_ptr<Grid>& g, cudaStream_t stream) {
    std::lock_guard<std::mutex> lk(g_small_mu);
    SmallBuild* b = nullptr;
    int32_t rc = small_entry(*g, nonzero, b);
    if (rc) return rc;
    b->last_use = ++g_small_clock;
    const size_t elem = g->format == VT_PAYLOAD_U8 ? 1 : 4;
    const BlockLayout L = block_layout(g->bricks, g->bricks, g->format);
    // small blocks come from the stream-ordered pool (freed after a device synchronisation, like
    // cudaFree, so that no launch on another stream can still be reading them)
    void* block = nullptr;
    if (cudaMallocAsync(&block, L.total, stream) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMallocAsync(brick grid) failed");
    }
    point_into_block(*g, block, L, g->bricks);
    g->pooled = true;
    uint32_t hc[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(b->in, src, (size_t)g->nx * g->ny * g->nz * elem,
                                    src_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                    stream);
    if (e == cudaSuccess && g->format == VT_PAYLOAD_U8)
        e = cudaMemcpyAsync((char*)b->tmpl + L.pal, palette_host, 1024, cudaMemcpyHostToDevice,
                            stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(block, b->tmpl, L.total, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, b->counts, 16, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "small grid build");
    g->nonempty = (uint64_t)hc[0] + hc[1];
    g->occupied = (uint64_t)hc[2] | ((uint64_t)hc[3] << 32);
    g->bytes = g->block_bytes;
    g->slots_used = g->nonempty;
    return VT_OK;
}

static std::unique_ptr<Grid> grid_shell(uint32_t format, uint32_t nx, uint32_t ny, uint32_t nz) {
    std::unique_ptr<Grid> g(new Grid());
    g->nx = nx;
    g->ny = ny;
    g->nz = nz;
    g->bx = (nx + 7) / 8;
    g->by = (ny + 7) / 8;
    g->bz = (nz + 7) / 8;
    g->bricks = (uint64_t)g->bx * g->by * g->bz;
    g->format = format;
    return g;
}

// u8 palettes whose only transparent entry is index 0: occupancy is "index != 0"
static bool nonzero_palette(uint32_t format, const uint32_t* palette_host) {
    bool nonzero = format == VT_PAYLOAD_U8 && (palette_host[0] >> 24) == 0u;
    for (int i = 1; nonzero && i < 256; ++i) nonzero = (palette_host[i] >> 24) != 0u;
    return nonzero;
}

static bool small_grid(uint32_t nx, uint32_t ny, uint32_t nz) {
    return (uint64_t)((nx + 7) / 8) * ((ny + 7) / 8) * ((nz + 7) / 8) <= kSmallGridBricks;
}

static int32_t build_small_from_host(const void* voxels, uint32_t format,
                                     const uint32_t* palette_host, uint32_t nx, uint32_t ny,
                                     uint32_t nz, cudaStream_t stream, std::unique_ptr<Grid>& out) {
    std::unique_ptr<Grid> g = grid_shell(format, nx, ny, nz);
    const int32_t rc = build_small(voxels, true, palette_host, nonzero_palette(format, palette_host),
                                   g, stream);
    if (rc) {
        g->release();
        return rc;
    }
    out = std::move(g);
    return VT_OK;
}

// Builds the brick layout of a dense device grid on `stream` and waits for it.
int32_t build_grid(const void* d_src, uint32_t format, const uint32_t* palette_host,
                   uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t stream,
                   std::unique_ptr<Grid>& out) {
    std::unique_ptr<Grid> g = grid_shell(format, nx, ny, nz);
    const bool nonzero = nonzero_palette(format, palette_host);
    int32_t rc = VT_OK;
    if (g->bricks <= kSmallGridBricks) {
        if ((rc = build_small(d_src, false, palette_host, nonzero, g, stream))) {
            g->release();
            return rc;
        }
        out = std::move(g);
        return VT_OK;
    }
    // the words kernel reads the palette from device memory (scratch tail) before the grid's
    // allocation exists: its size needs the count of occupied bricks
    // The scratch is followed by the palette and, when it fits, the staging buffer that lets the
    // compaction copy whole brick blocks instead of re-reading the dense grid (as large again as
    // the padded grid, for the duration of the build; without it the build is the same, slower).
    void* scratch = nullptr;
    const size_t sbytes = build_scratch_bytes(g->bricks);
    const size_t staged_at = sbytes + 1024;  // 256-aligned: sbytes is
    cudaError_t e = cudaMallocAsync(&scratch, staged_at + build_staging_bytes(g->bricks, format), stream);
    bool staging = e == cudaSuccess;
    if (!staging) {
        cudaGetLastError();
        e = cudaMallocAsync(&scratch, staged_at, stream);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMallocAsync(brick build scratch) failed");
    }
    BuildScratch s = carve_build_scratch(scratch, g->bricks);
    if (staging) s.staged = (char*)scratch + staged_at;
    uint32_t* d_palette = (uint32_t*)((char*)scratch + sbytes);
    uint32_t counts[2] = {0, 0};
    unsigned long long occ = 0;
    do {
        if (format == VT_PAYLOAD_U8) {
            e = cudaMemcpyAsync(d_palette, palette_host, 1024, cudaMemcpyHostToDevice, stream);
            if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpy(palette)"); break; }
        }
        e = launch_brick_words(d_src, format, d_palette, (int32_t)nx, (int32_t)ny, (int32_t)nz, s,
                               stream, nonzero);
        if (e == cudaSuccess) e = launch_brick_scan(s, g->bricks, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&counts[0], s.offsets + (g->bricks - 1), 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&counts[1], s.flags + (g->bricks - 1), 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&occ, s.occupied, 8, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) { rc = cuda_fail(e, "brick count"); break; }
        g->nonempty = (uint64_t)counts[0] + counts[1];
        g->occupied = occ;
        const uint64_t slots = g->nonempty ? g->nonempty : 1;
        const BlockLayout L = block_layout(g->bricks, slots, format);
        void* block = nullptr;
        if (cudaMalloc(&block, L.total) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(VT_ENOMEM, "cudaMalloc(brick grid) failed");
            break;
        }
        point_into_block(*g, block, L, slots);
        if (g->palette) {
            e = cudaMemcpyAsync(g->palette, d_palette, 1024, cudaMemcpyDeviceToDevice, stream);
            if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpy(palette)"); break; }
        }
        // compaction (from the words and slot offsets in the scratch), then the distance,
        // octant and long-box passes: build_launches' sequence after its scan
        e = launch_brick_compact(d_src, format, (int32_t)nx, (int32_t)ny, (int32_t)nz, s, g->dir,
                                 g->masks, g->payload, stream);
        uint32_t* occ = (uint32_t*)s.words + 13 * g->bricks;  // as in build_launches
        if (e == cudaSuccess)
            e = launch_brick_xmask(g->dir, occ, (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz, stream);
        if (e == cudaSuccess)
            e = launch_brick_distance(s, g->dir, (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz,
                                      stream, nullptr, occ);
        if (e == cudaSuccess)
            e = launch_brick_octants(g->dir, (uint8_t*)s.words,
                                     (uint16_t*)((uint8_t*)s.words + ((g->bricks + 255) / 256) * 256),
                                     g->oct, (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz, stream,
                                     nullptr, occ);
        if (e == cudaSuccess)
            e = launch_brick_long(g->dir, g->oct, (uint32_t*)s.words, g->lng, (int32_t)g->bx,
                                  (int32_t)g->by, (int32_t)g->bz, stream, nullptr, occ);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) { rc = cuda_fail(e, "brick build"); break; }
        g->bytes = g->block_bytes;
        g->slots_used = g->nonempty;
    } while (0);
    const cudaError_t f = cudaFreeAsync(scratch, stream);
    if (rc == VT_OK && f != cudaSuccess) rc = cuda_fail(f, "cudaFreeAsync(brick build scratch)");
    if (rc != VT_OK) {
        cudaStreamSynchronize(stream);
        g->release();
        return rc;
    }
    out = std::move(g);
    return VT_OK;
}

int32_t register_grid(std::unique_ptr<Grid> g) {
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    s.grid_epoch.fetch_add(1);
    for (size_t i = 0; i < s.grids.size(); ++i)
        if (!s.grids[i]) {
            s.grids[i] = std::move(g);
            return (int32_t)i;
        }
    if (s.grids.size() >= kMaxGrids) {
        g->release();
        return fail(VT_ELIMIT, "too many grids");
    }
    s.grids.push_back(std::move(g));
    return (int32_t)(s.grids.size() - 1);
}

Grid* lookup_grid(int32_t id) {
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    if (id < 0 || (size_t)id >= s.grids.size() || !s.grids[id]) return nullptr;
    return s.grids[id].get();
}

LightView light_view(const vt_light* light) {
    LightView L;
    memset(&L, 0, sizeof(L));
    if (light) {
        L.dx = light->dir[0];
        L.dy = light->dir[1];
        L.dz = light->dir[2];
        L.ambient = light->ambient;
        L.enabled = 1;
        L.shadows = light->shadows ? 1u : 0u;
    }
    return L;
}

int32_t check_camera(const vt_camera* cam) {
    if (!cam) return fail(VT_EINVAL, "null camera");
    if (cam->width == 0 || cam->height == 0 || cam->width > 65536 || cam->height > 65536)
        return fail(VT_EINVAL, "camera size must be in 1..65536");
    return VT_OK;
}

// Device staging for the *_host calls (grown on demand, guarded by State::host_mu).
// Outputs in page-locked host memory (cudaHostAlloc / cudaHostRegister) are written by the
// kernels themselves, over the host link, instead of staged in device memory and copied.
void* host_mapped(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((uintptr_t)a.devicePointer & 15u))
        return nullptr;
    return a.devicePointer;
}

void* device_address(void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    return nullptr;
}

int32_t staging(size_t bytes, void** out) {
    State& s = state();
    if (s.staging_bytes < bytes) {
        cudaFree(s.staging);
        s.staging = nullptr;
        s.staging_bytes = 0;
        if (cudaMalloc(&s.staging, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(VT_ENOMEM, "cudaMalloc(staging) failed");
        }
        s.staging_bytes = bytes;
    }
    *out = s.staging;
    return VT_OK;
}

void stats_from(const Counters& c, vt_trace_stats* st) {
    st->rays = c.rays;
    st->shadow_rays = c.shadow_rays;
    st->hits = c.hits;
    st->steps = c.steps;
    st->bricks_entered = c.bricks;
    st->nonempty_bricks_entered = c.nonempty;
    st->voxels_tested = c.tested;
    st->ties = c.ties;
}

}  // namespace vt

using namespace vt;

extern "C" {

int32_t vt_init(int32_t device) {
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    if (s.inited) {
        if (s.device != device) return fail(VT_EINVAL, "vt_init: already initialised on another device");
        return VT_OK;
    }
    return ensure_init_locked(device);
}

void vt_shutdown(void) {
    vt_serve_release_all();
    vt::noalloc_forget_addresses();
    vt_compat_release();
    vt_batch_release_all();
    vt::release_small_builds();
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.inited) return;
    cudaStreamSynchronize(s.stream);
    for (auto& g : s.grids)
        if (g) g->release();
    s.grids.clear();
    cudaFree(s.staging);
    s.staging = nullptr;
    s.staging_bytes = 0;
    cudaFree(s.counters);
    s.counters = nullptr;
    for (int k = 0; k < State::kAux; ++k) {
        cudaStreamSynchronize(s.aux[k]);
        cudaStreamDestroy(s.aux[k]);
        s.aux[k] = nullptr;
    }
    cudaEventDestroy(s.aux_start);
    s.aux_start = nullptr;
    for (cudaEvent_t ev : s.chunk_events) cudaEventDestroy(ev);
    s.chunk_events.clear();
    cudaStreamDestroy(s.stream);
    s.stream = nullptr;
    s.inited = false;
}

const char* vt_last_error(void) { return g_last_error.c_str(); }

uint32_t vt_version(void) { return (1u << 16) | 3u; }

void* vt_get_stream(void) {
    if (ensure_init()) return nullptr;
    return (void*)state().stream;
}

int32_t vt_device_info(int32_t* device, int32_t* sm_count, uint64_t* free_bytes,
                       uint64_t* total_bytes) {
    int32_t rc = ensure_init();
    if (rc) return rc;
    State& s = state();
    if (device) *device = s.device;
    if (sm_count) *sm_count = s.sm_count;
    size_t f = 0, t = 0;
    cudaError_t e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return VT_OK;
}

static TraceTuning* tuning_of(int32_t kernel) {
    State& s = state();
    switch (kernel) {
        case VT_KERNEL_RENDER: return &s.tune_render;
        case VT_KERNEL_TRACE_RAYS: return &s.tune_rays;
        case VT_KERNEL_BATCH: return &s.tune_batch;
        case VT_KERNEL_PATH: return &s.tune_path;
        default: return nullptr;
    }
}

int32_t vt_get_tuning(int32_t kernel, vt_tuning* out) {
    TraceTuning* t = tuning_of(kernel);
    if (!t || !out) return fail(VT_EINVAL, "vt_get_tuning: bad kernel or null output");
    out->refill_min = t->refill_min;
    out->blocks_per_sm = t->blocks_per_sm;
    out->persistent = t->persistent;
    out->wavefront = t->wavefront;
    out->tile_shape = t->tile_shape;
    out->block_warps = t->block_warps;
    return VT_OK;
}

int32_t vt_set_tuning(int32_t kernel, const vt_tuning* in) {
    TraceTuning* t = tuning_of(kernel);
    if (!t || !in) return fail(VT_EINVAL, "vt_set_tuning: bad kernel or null input");
    if (in->refill_min < 1 || in->refill_min > 32 || in->blocks_per_sm < 0 || in->blocks_per_sm > 64)
        return fail(VT_EINVAL, "vt_set_tuning: refill_min must be 1..32, blocks_per_sm 0..64");
    if (in->tile_shape > VT_TILE_32X1 ||
        (in->block_warps != 0 && in->block_warps != 1 && in->block_warps != 2 &&
         in->block_warps != 4 && in->block_warps != 8))
        return fail(VT_EINVAL, "vt_set_tuning: tile_shape must be a VT_TILE_* value, block_warps "
                               "0, 1, 2, 4 or 8");
    t->refill_min = in->refill_min;
    t->blocks_per_sm = in->blocks_per_sm;
    t->persistent = in->persistent ? 1u : 0u;
    t->wavefront = in->wavefront ? 1u : 0u;
    t->tile_shape = in->tile_shape;
    t->block_warps = in->block_warps ? in->block_warps : 4u;
    return VT_OK;
}

int32_t vt_grid_create_u8_device(const uint8_t* d_voxels, const uint32_t* palette, uint32_t nx,
                                 uint32_t ny, uint32_t nz, void* stream) {
    if (!d_voxels || !palette) return fail(VT_EINVAL, "vt_grid_create_u8_device: null pointer");
    int32_t rc = check_dims(nx, ny, nz);
    if (rc) return rc;
    if ((rc = ensure_init())) return rc;
    std::unique_ptr<Grid> g;
    rc = build_grid(d_voxels, VT_PAYLOAD_U8, palette, nx, ny, nz, pick_stream(stream), g);
    if (rc) return rc;
    return register_grid(std::move(g));
}

static int32_t create_from_host(const void* data, size_t elem, uint32_t format, uint32_t order,
                                const uint32_t* palette, uint32_t nx, uint32_t ny, uint32_t nz) {
    int32_t rc = check_dims(nx, ny, nz);
    if (rc) return rc;
    if ((rc = ensure_init())) return rc;
    const size_t bytes = (size_t)nx * ny * nz * elem;
    const int nbuf = order == VT_ORDER_Z_FASTEST ? 2 : 1;
    cudaStream_t st = state().stream;
    if (order == VT_ORDER_X_FASTEST && small_grid(nx, ny, nz)) {  // straight into the build graph's input
        std::unique_ptr<Grid> g;
        if ((rc = build_small_from_host(data, format, palette, nx, ny, nz, st, g))) return rc;
        return register_grid(std::move(g));
    }
    void* d = nullptr;
    if (cudaMallocAsync(&d, bytes * nbuf, st) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMallocAsync(dense grid upload) failed");
    }
    // z-fastest input lands in the second half and is transposed into the first
    void* up = (char*)d + bytes * (nbuf - 1);
    cudaError_t e = cudaMemcpyAsync(up, data, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nbuf == 2)
        e = launch_transpose_xz(up, d, elem, (int32_t)nx, (int32_t)ny, (int32_t)nz, st);
    std::unique_ptr<Grid> g;
    if (e != cudaSuccess)
        rc = cuda_fail(e, "dense grid upload");
    else
        rc = build_grid(d, format, palette, nx, ny, nz, st, g);
    cudaFreeAsync(d, st);
    cudaStreamSynchronize(st);  // the caller's buffer is read by then
    if (rc) return rc;
    return register_grid(std::move(g));
}

int32_t vt_grid_create(const void* voxels, uint32_t format, uint32_t order,
                       const uint32_t* palette, uint32_t nx, uint32_t ny, uint32_t nz) {
    if (!voxels) return fail(VT_EINVAL, "vt_grid_create: null voxels");
    if (format != VT_PAYLOAD_U8 && format != VT_PAYLOAD_RGBA8)
        return fail(VT_EINVAL, "vt_grid_create: format must be VT_PAYLOAD_U8 or VT_PAYLOAD_RGBA8");
    if (order != VT_ORDER_X_FASTEST && order != VT_ORDER_Z_FASTEST)
        return fail(VT_EINVAL, "vt_grid_create: order must be VT_ORDER_X_FASTEST or VT_ORDER_Z_FASTEST");
    if (format == VT_PAYLOAD_U8 && !palette)
        return fail(VT_EINVAL, "vt_grid_create: a u8 grid needs a palette");
    return create_from_host(voxels, format == VT_PAYLOAD_U8 ? 1 : 4, format, order,
                            format == VT_PAYLOAD_U8 ? palette : nullptr, nx, ny, nz);
}

int32_t vt_grid_create_u8(const uint8_t* voxels, const uint32_t* palette, uint32_t nx,
                          uint32_t ny, uint32_t nz) {
    if (!voxels || !palette) return fail(VT_EINVAL, "vt_grid_create_u8: null pointer");
    return create_from_host(voxels, 1, VT_PAYLOAD_U8, VT_ORDER_X_FASTEST, palette, nx, ny, nz);
}

int32_t vt_grid_create_rgba8(const uint8_t* rgba, uint32_t nx, uint32_t ny, uint32_t nz) {
    if (!rgba) return fail(VT_EINVAL, "vt_grid_create_rgba8: null pointer");
    return create_from_host(rgba, 4, VT_PAYLOAD_RGBA8, VT_ORDER_X_FASTEST, nullptr, nx, ny, nz);
}

int32_t vt_grid_destroy(int32_t grid) {
    State& s = state();
    std::lock_guard<std::mutex> lk(s.mu);
    if (grid < 0 || (size_t)grid >= s.grids.size() || !s.grids[grid])
        return fail(VT_ENOTFOUND, "vt_grid_destroy: unknown grid");
    if (s.grids[grid]->refs.load() > 0) return fail(VT_EBUSY, "vt_grid_destroy: grid in use");
    cudaStreamSynchronize(s.stream);
    s.grids[grid]->release();
    s.grids[grid].reset();
    s.grid_epoch.fetch_add(1);
    return VT_OK;
}

int32_t vt_grid_get_info(int32_t grid, vt_grid_info* info) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_get_info: unknown grid");
    if (!info) return fail(VT_EINVAL, "vt_grid_get_info: null info");
    info->nx = g->nx;
    info->ny = g->ny;
    info->nz = g->nz;
    info->bricks_x = g->bx;
    info->bricks_y = g->by;
    info->bricks_z = g->bz;
    info->bricks_total = g->bricks;
    info->bricks_nonempty = g->nonempty;
    info->voxels_occupied = g->occupied;
    info->device_bytes = g->bytes;
    info->payload_format = g->format;
    info->slots = (uint32_t)g->slots_used;
    return VT_OK;
}

int32_t vt_grid_download_bricks(int32_t grid, uint32_t* directory, uint64_t* masks) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_download_bricks: unknown grid");
    cudaStream_t st = state().stream;
    cudaError_t e = cudaSuccess;
    if (directory) e = cudaMemcpyAsync(directory, g->dir, g->bricks * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && masks && g->slots_used)
        e = cudaMemcpyAsync(masks, g->masks, g->slots_used * 64, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_grid_download_bricks");
    return VT_OK;
}

int32_t vt_grid_download_payload(int32_t grid, void* payload, uint64_t capacity_bytes) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_download_payload: unknown grid");
    const uint64_t bytes = g->slots_used * 512 * (g->format == VT_PAYLOAD_RGBA8 ? 4 : 1);
    if (!payload || capacity_bytes < bytes)
        return fail(VT_EINVAL, "vt_grid_download_payload: null output or capacity below slots * 512 voxels");
    if (!bytes) return VT_OK;
    cudaStream_t st = state().stream;
    cudaError_t e = cudaMemcpyAsync(payload, g->payload, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_grid_download_payload");
    return VT_OK;
}

int32_t vt_grid_download_long(int32_t grid, uint32_t* words) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_download_long: unknown grid");
    if (!words) return fail(VT_EINVAL, "vt_grid_download_long: null output");
    cudaStream_t st = state().stream;
    cudaError_t e = cudaMemcpyAsync(words, g->lng, g->bricks * 12, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_grid_download_long");
    return VT_OK;
}

int32_t vt_grid_download_octants(int32_t grid, uint32_t* octants) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_download_octants: unknown grid");
    if (!octants) return fail(VT_EINVAL, "vt_grid_download_octants: null output");
    cudaStream_t st = state().stream;
    cudaError_t e = cudaMemcpyAsync(octants, g->oct, g->bricks * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_grid_download_octants");
    return VT_OK;
}

int32_t vt_trace_rays(int32_t grid, const vt_ray* d_rays, uint64_t n, vt_hit* d_hits,
                      void* stream) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_trace_rays: unknown grid");
    if (n && (!d_rays || !d_hits)) return fail(VT_EINVAL, "vt_trace_rays: null buffer");
    if (((uintptr_t)d_rays & 7u) || ((uintptr_t)d_hits & 15u))
        return fail(VT_EINVAL, "vt_trace_rays: rays must be 8-byte and hits 16-byte aligned");
    cudaError_t e = launch_rays(g->view(), d_rays, n, (uint4*)d_hits, pick_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "vt_trace_rays launch");
    return VT_OK;
}

int32_t vt_trace_rays_stats(int32_t grid, const vt_ray* d_rays, uint64_t n, vt_hit* d_hits,
                            vt_trace_stats* stats) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_trace_rays_stats: unknown grid");
    if (!stats || (n && (!d_rays || !d_hits))) return fail(VT_EINVAL, "vt_trace_rays_stats: null pointer");
    if (((uintptr_t)d_rays & 7u) || ((uintptr_t)d_hits & 15u))
        return fail(VT_EINVAL, "vt_trace_rays_stats: misaligned buffer");
    Counters* dc = nullptr;
    cudaStream_t st = state().stream;
    if (cudaMalloc(&dc, sizeof(Counters)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMalloc(counters)");
    }
    Counters hc;
    cudaError_t e = cudaMemsetAsync(dc, 0, sizeof(Counters), st);
    if (e == cudaSuccess) e = launch_trace_rays(g->view(), d_rays, n, (uint4*)d_hits, dc, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dc);
    if (e != cudaSuccess) return cuda_fail(e, "vt_trace_rays_stats");
    stats_from(hc, stats);
    return VT_OK;
}

// Host-buffer forms: the work is split into pieces (ray chunks, row bands) issued round-robin on
// the helper streams, each piece's upload, traversal and download in order on its stream, so that
// the copies of one piece overlap the traversal of the next.  Both helper streams first wait for
// the library stream's earlier work.
static cudaError_t aux_begin(State& s) {
    cudaError_t e = cudaEventRecord(s.aux_start, s.stream);
    for (int k = 0; e == cudaSuccess && k < State::kAux; ++k)
        e = cudaStreamWaitEvent(s.aux[k], s.aux_start, 0);
    return e;
}

static cudaError_t aux_end(State& s, cudaError_t e) {
    for (int k = 0; k < State::kAux; ++k) {
        const cudaError_t f = cudaStreamSynchronize(s.aux[k]);
        if (e == cudaSuccess) e = f;
    }
    return e;
}

constexpr uint64_t kHostRayChunk = 1u << 21;  // rays per piece of vt_trace_rays_host (2 Mi: as fast as 1 Mi, 5% faster than 4 Mi)

int32_t vt_trace_rays_host(int32_t grid, const vt_ray* rays, uint64_t n, vt_hit* hits) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_trace_rays_host: unknown grid");
    if (n == 0) return VT_OK;
    if (!rays || !hits) return fail(VT_EINVAL, "vt_trace_rays_host: null buffer");
    State& s = state();
    std::lock_guard<std::mutex> lk(s.host_mu);
    // records go through device memory and copies even to page-locked memory: the persistent
    // kernel's scattered 16-byte stores over the host link measured 1.4x slower end to end
    const size_t rb = (size_t)n * sizeof(vt_ray), hb = (size_t)n * sizeof(vt_hit);
    const size_t roff = (hb + 255) / 256 * 256;
    void* buf;
    int32_t rc = staging(roff + rb, &buf);
    if (rc) return rc;
    vt_hit* dh = (vt_hit*)buf;
    vt_ray* dr = (vt_ray*)((char*)buf + roff);
    const GridView v = g->view();
    // three-stage pipeline over pieces of kHostRayChunk rays: the copies in run back to back on one
    // stream, each piece's traversal (two streams, alternating) waits for its rays, and the copies
    // out (one stream) wait for the traversal; each stage runs at its own pace
    const uint64_t pieces = (n + kHostRayChunk - 1) / kHostRayChunk;
    cudaError_t e = cudaSuccess;
    while (e == cudaSuccess && s.chunk_events.size() < 2 * pieces) {
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) s.chunk_events.push_back(ev);
    }
    if (e == cudaSuccess) e = aux_begin(s);
    cudaStream_t in = s.aux[0], out = s.aux[1];
    for (uint64_t i = 0, k = 0; e == cudaSuccess && i < n; i += kHostRayChunk, ++k) {
        const uint64_t m = std::min<uint64_t>(kHostRayChunk, n - i);
        cudaStream_t st = s.aux[2 + (k & 1)];
        cudaEvent_t loaded = s.chunk_events[2 * k], traced = s.chunk_events[2 * k + 1];
        e = cudaMemcpyAsync(dr + i, rays + i, m * sizeof(vt_ray), cudaMemcpyHostToDevice, in);
        if (e == cudaSuccess) e = cudaEventRecord(loaded, in);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, loaded, 0);
        if (e == cudaSuccess) e = launch_rays(v, dr + i, m, (uint4*)(dh + i), st);
        if (e == cudaSuccess) e = cudaEventRecord(traced, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(out, traced, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hits + i, dh + i, m * sizeof(vt_hit), cudaMemcpyDeviceToHost, out);
    }
    e = aux_end(s, e);
    if (e != cudaSuccess) return cuda_fail(e, "vt_trace_rays_host");
    return VT_OK;
}

int32_t vt_render(int32_t grid, const vt_camera* camera, const vt_light* light, vt_hit* d_hits,
                  void* stream) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_render: unknown grid");
    int32_t rc = check_camera(camera);
    if (rc) return rc;
    if (!d_hits || ((uintptr_t)d_hits & 15u)) return fail(VT_EINVAL, "vt_render: hits must be 16-byte aligned");
    cudaError_t e = launch_frame(g->view(), *camera, light_view(light), (uint4*)d_hits,
                                 pick_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "vt_render launch");
    return VT_OK;
}

int32_t vt_render_stats(int32_t grid, const vt_camera* camera, const vt_light* light,
                        vt_hit* d_hits, vt_trace_stats* stats) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_render_stats: unknown grid");
    int32_t rc = check_camera(camera);
    if (rc) return rc;
    if (!stats || !d_hits || ((uintptr_t)d_hits & 15u)) return fail(VT_EINVAL, "vt_render_stats: bad buffer");
    Counters* dc = nullptr;
    cudaStream_t st = state().stream;
    if (cudaMalloc(&dc, sizeof(Counters)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMalloc(counters)");
    }
    Counters hc;
    cudaError_t e = cudaMemsetAsync(dc, 0, sizeof(Counters), st);
    if (e == cudaSuccess) e = launch_render(g->view(), *camera, light_view(light), (uint4*)d_hits, dc, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dc);
    if (e != cudaSuccess) return cuda_fail(e, "vt_render_stats");
    stats_from(hc, stats);
    return VT_OK;
}

int32_t vt_render_footprint(int32_t grid, const vt_camera* camera, const vt_light* light,
                            vt_hit* d_hits, vt_footprint* out) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_render_footprint: unknown grid");
    int32_t rc = check_camera(camera);
    if (rc) return rc;
    if (!out || !d_hits || ((uintptr_t)d_hits & 15u)) return fail(VT_EINVAL, "vt_render_footprint: bad buffer");
    const size_t words = (g->bricks + 31) / 32;
    const size_t bytes = 256 + 3 * words * 4;
    char* buf = nullptr;
    cudaStream_t st = state().stream;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMalloc(footprint)");
    }
    Counters hc;
    memset(&hc, 0, sizeof(hc));
    hc.touched = (unsigned int*)(buf + 256);
    std::vector<uint32_t> maps(3 * words);
    cudaError_t e = cudaMemsetAsync(buf, 0, bytes, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf, &hc, sizeof(hc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = launch_render(g->view(), *camera, light_view(light), (uint4*)d_hits, (Counters*)buf, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(maps.data(), buf + 256, 3 * words * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "vt_render_footprint");
    uint64_t n[3] = {0, 0, 0};
    for (int m = 0; m < 3; ++m)
        for (size_t i = 0; i < words; ++i) n[m] += (uint64_t)__builtin_popcount(maps[m * words + i]);
    out->bricks = n[0];
    out->nonempty_bricks = n[1];
    out->hit_bricks = n[2];
    out->reserved = 0;
    return VT_OK;
}

int32_t vt_render_phases(int32_t grid, const vt_camera* camera, const vt_light* light,
                         vt_hit* d_hits, vt_phase_profile* out) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_render_phases: unknown grid");
    int32_t rc = check_camera(camera);
    if (rc) return rc;
    if (!out || !d_hits || ((uintptr_t)d_hits & 15u)) return fail(VT_EINVAL, "vt_render_phases: bad buffer");
    const unsigned words = phase_profile_words();
    unsigned long long* dt = nullptr;
    cudaStream_t st = state().stream;
    if (cudaMalloc(&dt, words * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VT_ENOMEM, "cudaMalloc(phase totals)");
    }
    std::vector<unsigned long long> h(words);
    cudaError_t e = cudaMemsetAsync(dt, 0, words * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = launch_render_phases(g->view(), *camera, light_view(light), (uint4*)d_hits, dt, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), dt, words * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dt);
    if (e != cudaSuccess) return cuda_fail(e, "vt_render_phases");
    for (int k = 0; k < 2; ++k) {
        for (int p = 0; p < VT_PHASES; ++p) out->warp_cycles[k][p] = h[k * VT_PHASES + p];
        for (int j = 0; j < 2; ++j) out->passes[k][j] = h[2 * VT_PHASES + 2 * k + j];
    }
    out->warps = h[2 * VT_PHASES + 4];
    return VT_OK;
}

int32_t vt_render_host(int32_t grid, const vt_camera* camera, const vt_light* light,
                       vt_hit* hits) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_render_host: unknown grid");
    int32_t rc = check_camera(camera);
    if (rc) return rc;
    if (!hits) return fail(VT_EINVAL, "vt_render_host: null output");
    State& s = state();
    std::lock_guard<std::mutex> lk(s.host_mu);
    const uint32_t W = camera->width, H = camera->height;
    const size_t hb = (size_t)W * H * sizeof(vt_hit);
    const GridView v = g->view();
    const LightView L = light_view(light);
    cudaError_t e;
    if (void* mapped = host_mapped(hits)) {  // pinned output: the kernel writes the records there
        e = launch_frame(v, *camera, L, (uint4*)mapped, s.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
        if (e != cudaSuccess) return cuda_fail(e, "vt_render_host");
        return VT_OK;
    }
    void* buf;
    if ((rc = staging(hb, &buf))) return rc;
    // bands only pay when the copy of one is long enough to hide behind the next one's traversal
    if (s.tune_render.persistent || s.tune_render.wavefront || (uint64_t)W * H < (1u << 20)) {
        cudaStream_t st = s.stream;
        e = launch_frame(v, *camera, L, (uint4*)buf, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hits, buf, hb, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } else {
        // four row bands of whole 16-row tiles
        const uint32_t band = (H / 4 + 15) / 16 * 16;
        e = aux_begin(s);
        for (uint32_t r0 = 0, k = 0; e == cudaSuccess && r0 < H; r0 += band, ++k) {
            const uint32_t r1 = std::min(H, r0 + band);
            cudaStream_t st = s.aux[k % State::kAux];
            e = launch_render(v, *camera, L, (uint4*)buf, nullptr, st, r0, r1);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hits + (size_t)r0 * W, (vt_hit*)buf + (size_t)r0 * W,
                                    (size_t)(r1 - r0) * W * sizeof(vt_hit), cudaMemcpyDeviceToHost, st);
        }
        e = aux_end(s, e);
    }
    if (e != cudaSuccess) return cuda_fail(e, "vt_render_host");
    return VT_OK;
}

}  // extern "C"
