// vt_serve.cu — continuous-batching render service.
//
// Requests (scene, camera, resolution, spp, light) arrive from any thread through
// vt_serve_submit, which splits each image into pieces of whole 8 x 4 tile rows of at most
// `max_samples_per_piece` samples (a small request is one piece).  A dispatcher thread keeps up to
// `max_inflight` launches on the device at once, each on its own stream: whenever a launch slot is
// free it packs the oldest pending pieces, in arrival order, up to `max_views_per_launch` pieces
// and `max_samples_per_launch` samples, into one persistent work-stealing launch of the batched
// kernel (vt_batch.cu), followed by one resolve kernel that averages every piece's samples
// straight into its rows of the caller's image (page-locked host memory is written by the kernel
// itself, other memory through a device staging area and a copy).  Big requests thus run as a
// sequence of bounded launches that small requests arriving meanwhile interleave with, every
// launch is bounded in duration, and requests complete in arrival order as their last piece
// retires.  Sample records live in buffers each slot allocates once, at start.
//
// Brick grids of the scenes stay resident in a cache bounded by an HBM budget that also counts
// the slots' buffers and any temporary buffer of a piece larger than a slot's: a scene is built
// on first use, and least-recently-used scenes that no in-flight piece references are evicted to
// make room.  Every request's image depends only on its own parameters (per-sample Philox jitter
// keyed by seed and view id, pixels resolved in sample order), so it is the same alone, split
// into pieces, and in any mix of requests.
//
// With max_inflight = 1, max_views_per_launch = 1 and max_samples_per_piece = 0 (no splitting)
// the same machinery is the plain baseline: one launch per request, one launch at a time, in
// arrival order.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "vt_api_internal.h"
#include "vt_batch.h"
#include "vt_internal.h"

namespace vt {

struct ResolveView {
    const uint4* samples;
    uchar4* image;
    unsigned long long pixel_begin;
    uint32_t pixels;
    uint32_t spp;
};

// Average of each pixel's samples: per channel (sum + spp/2) / spp, alpha included.
__global__ void __launch_bounds__(256) resolve_kernel(const ResolveView* __restrict__ table,
                                                      uint32_t n, uint64_t total) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (table[mid].pixel_begin <= p)
                lo = mid;
            else
                hi = mid - 1;
        }
        const ResolveView& V = table[lo];
        const uint64_t q = p - V.pixel_begin;
        uint32_t r = 0, g = 0, b = 0, a = 0;
        for (uint32_t s = 0; s < V.spp; ++s) {
            const uint32_t c = __ldg(&V.samples[q * V.spp + s].w);
            r += c & 0xFFu;
            g += (c >> 8) & 0xFFu;
            b += (c >> 16) & 0xFFu;
            a += c >> 24;
        }
        const uint32_t h = V.spp / 2;
        V.image[q] = make_uchar4((unsigned char)((r + h) / V.spp), (unsigned char)((g + h) / V.spp),
                                 (unsigned char)((b + h) / V.spp), (unsigned char)((a + h) / V.spp));
    }
}

static int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct ServeScene {
    const uint8_t* voxels = nullptr;
    uint32_t palette[256];
    uint32_t nx = 0, ny = 0, nz = 0;
    int32_t grid = -1;
    int32_t refs = 0;  // in-flight and packed pieces
    bool loading = false;
    bool updating = false;  // a vt_serve_update_scene is writing its grid: no piece is admitted
    uint64_t last_use = 0;
    uint64_t bytes = 0;
};

struct ServeReq {
    vt_serve_request r;
    int32_t status = VT_ENOTREADY;
    int32_t error = VT_OK;  // first failure of one of its pieces
    bool cancelled = false;
    int64_t t_submit = 0, t_launch = 0, t_done = 0;
    uint64_t samples = 0;
    uint32_t pieces_pending = 0, pieces_inflight = 0;
    bool mapped_known = false;
    void* h_image = nullptr;  // device address of a page-locked host_rgba, written directly
};

// Rows row0 .. row1 - 1 of a request's image; row0 is a multiple of 4 (the tile height) and so is
// row1 unless it is the image's last row.
struct Piece {
    uint64_t req;
    uint32_t row0, row1;
    uint64_t samples;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t t_begin = nullptr, t_end = nullptr;  // device time of the slot's launch
    BatchView* d_table = nullptr;
    BatchView* h_table = nullptr;  // pinned staging
    ResolveView* d_resolve = nullptr;
    ResolveView* h_resolve = nullptr;
    unsigned long long* d_counter = nullptr;
    // sample records (16 B each) of up to `cap` samples, then an RGBA8 staging image of `cap`
    // pixels for outputs the resolve cannot write directly
    void* buf = nullptr;
    uint64_t cap = 0;
    uint64_t extra_bytes = 0;  // budget reserved for a temporary of an oversized piece
    std::vector<Piece> pieces;
    bool busy = false;
};

struct Service {
    vt_serve_config cfg;
    std::mutex mu;
    std::condition_variable cv;       // wakes the dispatcher
    std::condition_variable cv_done;  // wakes pollers
    std::thread worker;
    bool stop = false;
    std::vector<std::unique_ptr<ServeScene>> scenes;
    std::deque<Piece> pending;
    std::unordered_map<uint64_t, ServeReq> reqs;
    uint64_t next_id = 1;
    std::vector<Slot> slots;
    // device bytes counted against the budget: resident grids, the slots' buffers, and the
    // temporaries of oversized pieces in flight
    uint64_t resident_bytes = 0, slot_bytes = 0, extra_bytes = 0, tick = 0;
    vt_serve_stats stats;
    TraceTuning tune;

    ~Service();
    void run();
    int32_t admit_scene(std::unique_lock<std::mutex>& lk, int32_t scene);
    bool evict_for(uint64_t need);
    uint64_t used() const { return resident_bytes + slot_bytes + extra_bytes; }
    bool pack(Slot& slot, std::unique_lock<std::mutex>& lk);
    void launch(Slot& slot);
    void retire(Slot& slot, int32_t error);
    void fail_request(ServeReq& q, int32_t error);
    void finalize(ServeReq& q);
};

// Services are held by shared pointers: an entry point copies the pointer under g_serve_mu and
// keeps the service alive while it works on it, even if vt_serve_stop removes it meanwhile.
static std::mutex g_serve_mu;
static std::vector<std::shared_ptr<Service>> g_services;

static std::shared_ptr<Service> lookup_service(int32_t id) {
    std::lock_guard<std::mutex> lk(g_serve_mu);
    if (id < 0 || (size_t)id >= g_services.size()) return nullptr;
    return g_services[id];
}

Service::~Service() {
    if (worker.joinable()) {  // never stopped (library shutdown): stop the dispatcher first
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
            cv.notify_all();
        }
        worker.join();
    }
    for (Slot& sl : slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.t_begin) cudaEventDestroy(sl.t_begin);
        if (sl.t_end) cudaEventDestroy(sl.t_end);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        cudaFree(sl.d_table);
        cudaFree(sl.d_resolve);
        cudaFree(sl.d_counter);
        cudaFree(sl.buf);
        cudaFreeHost(sl.h_table);
        cudaFreeHost(sl.h_resolve);
    }
    for (auto& sc : scenes)
        if (sc->grid >= 0) vt_grid_destroy(sc->grid);
}

// Upper bound of a scene's resident bytes: its grid's allocation with every brick occupied.
static uint64_t scene_bound(const ServeScene& s) {
    const uint64_t bricks = (uint64_t)((s.nx + 7) / 8) * ((s.ny + 7) / 8) * ((s.nz + 7) / 8);
    return grid_bytes_bound(bricks, VT_PAYLOAD_U8);
}

// Evicts least-recently-used unreferenced scenes until `need` more bytes fit the budget; false
// if they do not.
bool Service::evict_for(uint64_t need) {
    while (used() + need > cfg.hbm_budget_bytes) {
        ServeScene* victim = nullptr;
        for (auto& s : scenes)
            if (s->grid >= 0 && s->refs == 0 && !s->loading && !s->updating &&
                (!victim || s->last_use < victim->last_use))
                victim = s.get();
        if (!victim) return false;
        vt_grid_destroy(victim->grid);
        victim->grid = -1;
        resident_bytes -= victim->bytes;
        victim->bytes = 0;
        stats.evictions++;
    }
    return true;
}

// Makes `scene` resident.  VT_OK, VT_EBUSY (no room until in-flight work ends), or an error.
int32_t Service::admit_scene(std::unique_lock<std::mutex>& lk, int32_t scene) {
    ServeScene& s = *scenes[scene];
    s.last_use = ++tick;
    if (s.grid >= 0) return VT_OK;
    const uint64_t need = scene_bound(s);
    if (need + slot_bytes > cfg.hbm_budget_bytes) return VT_ENOMEM;
    if (!evict_for(need)) return VT_EBUSY;
    s.loading = true;
    resident_bytes += need;  // reserved while the grid is built outside the lock
    lk.unlock();
    const int32_t g = vt_grid_create_u8(s.voxels, s.palette, s.nx, s.ny, s.nz);
    vt_grid_info info;
    const bool ok = g >= 0 && vt_grid_get_info(g, &info) == VT_OK;
    lk.lock();
    s.loading = false;
    cv_done.notify_all();  // a scene update may be waiting for the build to end
    resident_bytes -= need;
    if (!ok) return g < 0 ? g : VT_ECUDA;
    s.grid = g;
    s.bytes = info.device_bytes;
    resident_bytes += s.bytes;
    stats.scene_loads++;
    return VT_OK;
}

// A request whose pieces are all finished or dropped gets its final status.
void Service::finalize(ServeReq& q) {
    if (q.status != VT_ENOTREADY || q.pieces_inflight || q.pieces_pending) return;
    q.status = q.error != VT_OK ? q.error : (q.cancelled ? VT_ECANCELED : VT_OK);
    q.t_done = now_ns();
    if (q.status == VT_OK) {
        stats.completed++;
        stats.samples += q.samples;
    }
    cv_done.notify_all();
}

// Marks a request failed; its pending pieces are dropped as the dispatcher meets them.
void Service::fail_request(ServeReq& q, int32_t error) {
    if (q.error == VT_OK) q.error = error;
    finalize(q);
}

// Moves the oldest pending pieces into the free `slot`; false when nothing could be packed.
bool Service::pack(Slot& slot, std::unique_lock<std::mutex>& lk) {
    uint64_t samples = 0;
    slot.pieces.clear();
    while (!pending.empty() && slot.pieces.size() < cfg.max_views_per_launch) {
        const Piece pc = pending.front();
        ServeReq& q = reqs[pc.req];
        if (q.error != VT_OK || q.cancelled) {  // a failed request: drop its remaining pieces
            pending.pop_front();
            q.pieces_pending--;
            finalize(q);
            continue;
        }
        if (!slot.pieces.empty() && samples + pc.samples > slot.cap) break;
        uint64_t extra = 0;
        if (pc.samples > slot.cap) {  // alone, and larger than the slot's buffers
            extra = pc.samples * 20;
            if (extra + slot_bytes > cfg.hbm_budget_bytes) {
                pending.pop_front();
                q.pieces_pending--;
                fail_request(q, VT_ENOMEM);
                continue;
            }
        }
        // a scene being updated admits no piece until the update is written: the head of the
        // line keeps its place
        if (scenes[q.r.scene]->updating) break;
        // (admit_scene may release the lock while it builds a grid; only this thread pops
        // `pending`, so its front is still `pc` afterwards)
        const int32_t rc = admit_scene(lk, q.r.scene);
        if (rc == VT_EBUSY) break;  // wait for memory (the head of the line keeps its place)
        pending.pop_front();
        q.pieces_pending--;
        if (rc != VT_OK) {
            fail_request(q, rc);
            continue;
        }
        scenes[q.r.scene]->refs++;  // held until the piece retires (and never evicted below)
        if (extra) {
            if (used() + extra > cfg.hbm_budget_bytes && !evict_for(extra)) {
                scenes[q.r.scene]->refs--;
                const bool idle = std::none_of(slots.begin(), slots.end(),
                                               [](const Slot& s) { return s.busy; });
                if (idle) {  // its scene and its temporary never fit together
                    fail_request(q, VT_ENOMEM);
                    continue;
                }
                pending.push_front(pc);  // in-flight work holds the room: try again later
                q.pieces_pending++;
                break;
            }
            slot.extra_bytes = extra;
            extra_bytes += extra;
        }
        q.pieces_inflight++;
        slot.pieces.push_back(pc);
        samples += pc.samples;
        if (extra) break;
    }
    return !slot.pieces.empty();
}

void Service::launch(Slot& slot) {
    uint64_t samples = 0, pixels = 0;
    for (const Piece& pc : slot.pieces) {
        samples += pc.samples;
        pixels += (uint64_t)(pc.row1 - pc.row0) * reqs[pc.req].r.camera.width;
    }
    cudaEventRecord(slot.t_begin, slot.stream);
    char* base = (char*)slot.buf;
    char* staging = base + slot.cap * 16;
    void* temp = nullptr;
    cudaError_t e = cudaSuccess;
    if (slot.extra_bytes) {
        e = cudaMallocAsync(&temp, samples * 16 + pixels * 4, slot.stream);
        base = (char*)temp;
        staging = base + samples * 16;
    }
    uint64_t item = 0, pix = 0, off = 0;
    uint32_t n = 0;
    for (const Piece& pc : slot.pieces) {
        if (e != cudaSuccess) break;
        ServeReq& q = reqs[pc.req];
        const vt_serve_request& r = q.r;
        const uint32_t W = r.camera.width;
        Grid* g = lookup_grid(scenes[r.scene]->grid);
        if (!g) {
            e = cudaErrorInvalidValue;
            break;
        }
        if (!q.mapped_known) {
            q.h_image = host_mapped(r.host_rgba);
            q.mapped_known = true;
        }
        if (!q.t_launch) q.t_launch = now_ns();
        const uint64_t px = (uint64_t)(pc.row1 - pc.row0) * W;
        void* out = base + off * 16;
        slot.h_table[n] = make_batch_view(*g, r.camera, (r.flags & VT_VIEW_LIGHT) ? &r.light : nullptr,
                                          r.spp, r.seed, r.view_id, out, item, pc.row0);
        slot.h_resolve[n].samples = (const uint4*)out;
        slot.h_resolve[n].image = q.h_image ? (uchar4*)q.h_image + (uint64_t)pc.row0 * W
                                            : (uchar4*)(staging + pix * 4);
        slot.h_resolve[n].pixel_begin = pix;
        slot.h_resolve[n].pixels = (uint32_t)px;
        slot.h_resolve[n].spp = r.spp;
        item += batch_rows_items(r.camera, r.spp, pc.row0, pc.row1);
        pix += px;
        off += pc.samples;
        ++n;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_table, slot.h_table, n * sizeof(BatchView), cudaMemcpyHostToDevice,
                            slot.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_resolve, slot.h_resolve, n * sizeof(ResolveView),
                            cudaMemcpyHostToDevice, slot.stream);
    if (e == cudaSuccess)
        e = launch_batch(slot.d_table, n, item, slot.d_counter, tune, batch_blocks(n, item, tune),
                         slot.stream);
    if (e == cudaSuccess) {
        const unsigned rblocks =
            (unsigned)std::min<uint64_t>((pix + 255) / 256, (uint64_t)state().sm_count * 16);
        resolve_kernel<<<rblocks, 256, 0, slot.stream>>>(slot.d_resolve, n, pix);
        e = cudaGetLastError();
    }
    pix = 0;
    for (const Piece& pc : slot.pieces) {
        if (e != cudaSuccess) break;
        const ServeReq& q = reqs[pc.req];
        const uint64_t px = (uint64_t)(pc.row1 - pc.row0) * q.r.camera.width;
        if (!q.h_image)
            e = cudaMemcpyAsync(q.r.host_rgba + (uint64_t)pc.row0 * q.r.camera.width * 4,
                                staging + pix * 4, px * 4, cudaMemcpyDeviceToHost, slot.stream);
        pix += px;
    }
    if (temp) cudaFreeAsync(temp, slot.stream);
    cudaEventRecord(slot.t_end, slot.stream);
    cudaEventRecord(slot.done, slot.stream);
    slot.busy = true;
    stats.launches++;
    stats.views_launched += n;
    if (e != cudaSuccess) {  // nothing waits on a failed launch: retire it now
        cudaGetLastError();
        cudaStreamSynchronize(slot.stream);
        retire(slot, VT_ECUDA);
    }
}

void Service::retire(Slot& slot, int32_t error) {
    if (error == VT_OK) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, slot.t_begin, slot.t_end) == cudaSuccess)
            stats.device_ns += (uint64_t)((double)ms * 1e6);
        else
            cudaGetLastError();
    }
    for (const Piece& pc : slot.pieces) {
        ServeReq& q = reqs[pc.req];
        scenes[q.r.scene]->refs--;
        q.pieces_inflight--;
        if (error != VT_OK && q.error == VT_OK) q.error = error;
        finalize(q);
    }
    extra_bytes -= slot.extra_bytes;
    slot.extra_bytes = 0;
    slot.pieces.clear();
    slot.busy = false;
    cv_done.notify_all();  // scene updates wait for their scene's pieces to retire
}

void Service::run() {
    cudaSetDevice(state().device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool busy = false;
        for (Slot& sl : slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess) {
                retire(sl, VT_OK);
            } else if (q == cudaErrorNotReady) {
                busy = true;
            } else {  // a failed launch: report it on its requests
                cudaGetLastError();
                retire(sl, VT_ECUDA);
            }
        }
        if (stop) {
            for (const Piece& pc : pending) {
                ServeReq& q = reqs[pc.req];
                q.cancelled = true;
                q.pieces_pending--;
            }
            for (const Piece& pc : pending) finalize(reqs[pc.req]);
            pending.clear();
            if (!busy) break;
        }
        // admit the oldest pending pieces into free slots
        for (Slot& sl : slots) {
            if (sl.busy || pending.empty() || stop) continue;
            if (pack(sl, lk)) launch(sl);
            if (sl.busy) busy = true;
        }
        stats.pending = pending.size();
        if (busy)
            cv.wait_for(lk, std::chrono::microseconds(cfg.poll_interval_us));
        else if (!stop && pending.empty())
            cv.wait(lk);
        else if (!stop)
            cv.wait_for(lk, std::chrono::microseconds(cfg.poll_interval_us));
    }
}

}  // namespace vt

using namespace vt;

// Stops every service (vt_shutdown): their dispatchers finish in-flight launches and cancel the
// rest before the grids they reference are freed.
void vt_serve_release_all() {
    std::vector<std::shared_ptr<Service>> all;
    {
        std::lock_guard<std::mutex> lk(g_serve_mu);
        all.swap(g_services);
    }
    for (auto& s : all) {
        if (!s) continue;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            s->cv.notify_all();
        }
        if (s->worker.joinable()) s->worker.join();
        std::lock_guard<std::mutex> lk(s->mu);
        s->cv_done.notify_all();
    }
}

extern "C" {

int32_t vt_serve_default_config(vt_serve_config* cfg) {
    if (!cfg) return fail(VT_EINVAL, "vt_serve_default_config: null config");
    cfg->hbm_budget_bytes = 120ull << 30;
    cfg->max_inflight = 4;
    cfg->max_views_per_launch = 64;
    cfg->max_samples_per_launch = 8ull << 20;
    cfg->poll_interval_us = 20;
    cfg->refill_min = 32;
    cfg->max_samples_per_piece = 4ull << 20;
    return VT_OK;
}

int32_t vt_serve_start(const vt_serve_config* cfg, int32_t* service_out) {
    if (!cfg || !service_out) return fail(VT_EINVAL, "vt_serve_start: null argument");
    if (cfg->max_inflight < 1 || cfg->max_inflight > 32 || cfg->max_views_per_launch < 1 ||
        cfg->max_views_per_launch > kMaxBatchViews || cfg->refill_min < 1 || cfg->refill_min > 32 ||
        cfg->max_samples_per_launch == 0 || cfg->max_samples_per_launch > (1ull << 32))
        return fail(VT_EINVAL, "vt_serve_start: max_inflight 1..32, max_views_per_launch 1..256, "
                               "refill_min 1..32, max_samples_per_launch 1..2^32");
    int32_t rc = ensure_init();
    if (rc) return rc;
    std::shared_ptr<Service> s(new Service());
    s->cfg = *cfg;
    if (s->cfg.poll_interval_us == 0) s->cfg.poll_interval_us = 20;
    memset(&s->stats, 0, sizeof(s->stats));
    s->tune.refill_min = cfg->refill_min;
    s->tune.blocks_per_sm = 0;
    s->tune.persistent = 1;
    s->slot_bytes = cfg->max_inflight * cfg->max_samples_per_launch * 20;
    if (s->slot_bytes > cfg->hbm_budget_bytes)
        return fail(VT_ENOMEM, "vt_serve_start: the launch slots' sample buffers (max_inflight x "
                               "max_samples_per_launch x 20 B) exceed the HBM budget");
    s->slots.resize(cfg->max_inflight);
    for (Slot& sl : s->slots) {
        sl.cap = cfg->max_samples_per_launch;
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.t_begin);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.t_end);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_table, kMaxBatchViews * sizeof(BatchView));
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_resolve, kMaxBatchViews * sizeof(ResolveView));
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_counter, sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&sl.buf, sl.cap * 20);
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_table, kMaxBatchViews * sizeof(BatchView));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_resolve, kMaxBatchViews * sizeof(ResolveView));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation
                       ? fail(VT_ENOMEM, "vt_serve_start: slot buffers")
                       : cuda_fail(e, "vt_serve_start: slot resources");
        }
    }
    Service* raw = s.get();
    int32_t id;
    {
        std::lock_guard<std::mutex> lk(g_serve_mu);
        g_services.push_back(s);
        id = (int32_t)g_services.size() - 1;
    }
    raw->worker = std::thread([raw] { raw->run(); });
    *service_out = id;
    return VT_OK;
}

int32_t vt_serve_add_scene(int32_t service, const uint8_t* voxels, const uint32_t* palette,
                           uint32_t nx, uint32_t ny, uint32_t nz, int32_t* scene_out) {
    std::shared_ptr<Service> s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_add_scene: unknown service");
    if (!voxels || !palette || !scene_out) return fail(VT_EINVAL, "vt_serve_add_scene: null argument");
    int32_t rc = check_dims(nx, ny, nz);
    if (rc) return rc;
    std::unique_ptr<ServeScene> sc(new ServeScene());
    sc->voxels = voxels;
    memcpy(sc->palette, palette, sizeof(sc->palette));
    sc->nx = nx;
    sc->ny = ny;
    sc->nz = nz;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(VT_ECANCELED, "vt_serve_add_scene: service stopping");
    s->scenes.push_back(std::move(sc));
    *scene_out = (int32_t)s->scenes.size() - 1;
    return VT_OK;
}

int32_t vt_serve_update_scene(int32_t service, int32_t scene, uint32_t x0, uint32_t y0,
                              uint32_t z0, uint32_t w, uint32_t h, uint32_t d) {
    std::shared_ptr<Service> s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_update_scene: unknown service");
    std::unique_lock<std::mutex> lk(s->mu);
    if (scene < 0 || (size_t)scene >= s->scenes.size())
        return fail(VT_ENOTFOUND, "vt_serve_update_scene: unknown scene");
    ServeScene& sc = *s->scenes[scene];
    if (w == 0 || h == 0 || d == 0 || (uint64_t)x0 + w > sc.nx || (uint64_t)y0 + h > sc.ny ||
        (uint64_t)z0 + d > sc.nz)
        return fail(VT_EINVAL, "vt_serve_update_scene: empty box or box outside the scene");
    // one update of a scene at a time; then no new piece of it is admitted, and the update waits
    // for the pieces in flight (and a build in progress) to end
    while (sc.updating) s->cv_done.wait(lk);
    sc.updating = true;
    while (sc.refs > 0 || sc.loading) s->cv_done.wait(lk);
    int32_t rc = VT_OK;
    const int32_t g = sc.grid;
    if (g >= 0) {  // resident: write the box into the grid (an evicted scene is rebuilt from the
                   // caller's array, which already holds the change)
        lk.unlock();
        std::vector<uint8_t> box((size_t)w * h * d);
        for (uint32_t z = 0; z < d; ++z)
            for (uint32_t y = 0; y < h; ++y)
                memcpy(box.data() + ((size_t)z * h + y) * w,
                       sc.voxels + (((size_t)(z0 + z) * sc.ny + (y0 + y)) * sc.nx + x0), w);
        rc = vt_grid_update(g, box.data(), VT_ORDER_X_FASTEST, x0, y0, z0, w, h, d);
        vt_grid_info info;
        const bool known = vt_grid_get_info(g, &info) == VT_OK;
        lk.lock();
        if (known) {  // the slot arrays may have grown
            s->resident_bytes += info.device_bytes - sc.bytes;
            sc.bytes = info.device_bytes;
        }
    }
    sc.updating = false;
    s->cv_done.notify_all();
    s->cv.notify_one();
    return rc;
}

int32_t vt_serve_submit(int32_t service, const vt_serve_request* req, uint64_t* request_id) {
    const int64_t t = now_ns();
    std::shared_ptr<Service> s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_submit: unknown service");
    if (!req || !request_id || !req->host_rgba) return fail(VT_EINVAL, "vt_serve_submit: null argument");
    int32_t rc = check_camera(&req->camera);
    if (rc) return rc;
    if (req->spp == 0 || req->spp > 64) return fail(VT_EINVAL, "vt_serve_submit: spp must be 1..64");
    const uint64_t row_samples = (uint64_t)req->camera.width * req->spp;
    if (row_samples * req->camera.height >= (1ull << 32))
        return fail(VT_ELIMIT, "vt_serve_submit: 2^32 or more samples in one request");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(VT_ECANCELED, "vt_serve_submit: service stopping");
    if (req->scene < 0 || (size_t)req->scene >= s->scenes.size())
        return fail(VT_ENOTFOUND, "vt_serve_submit: unknown scene");
    const uint64_t id = s->next_id++;
    ServeReq& q = s->reqs[id];
    q.r = *req;
    q.t_submit = t;
    q.samples = row_samples * req->camera.height;
    // pieces of whole tile rows (4 image rows) of at most max_samples_per_piece samples
    const uint32_t H = req->camera.height;
    uint32_t rows = H;
    if (s->cfg.max_samples_per_piece)
        rows = (uint32_t)std::max<uint64_t>(4, s->cfg.max_samples_per_piece / row_samples / 4 * 4);
    for (uint32_t r0 = 0; r0 < H; r0 += rows) {
        const uint32_t r1 = std::min(H, r0 + rows);
        s->pending.push_back(Piece{id, r0, r1, (uint64_t)(r1 - r0) * row_samples});
        q.pieces_pending++;
    }
    s->stats.submitted++;
    *request_id = id;
    s->cv.notify_one();
    return VT_OK;
}

int32_t vt_serve_poll(int32_t service, uint64_t request_id, uint32_t timeout_us,
                      vt_serve_timing* timing) {
    std::shared_ptr<Service> s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_poll: unknown service");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return fail(VT_ENOTFOUND, "vt_serve_poll: unknown request");
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds(timeout_us);
    while (it->second.status == VT_ENOTREADY) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) break;
        it = s->reqs.find(request_id);
        if (it == s->reqs.end()) return fail(VT_ENOTFOUND, "vt_serve_poll: request released");
    }
    const ServeReq& q = it->second;
    if (q.status == VT_ENOTREADY) return VT_ENOTREADY;
    if (timing) {
        timing->submit_ns = q.t_submit;
        timing->launch_ns = q.t_launch;
        timing->done_ns = q.t_done;
        timing->samples = q.samples;
    }
    const int32_t st = q.status;
    s->reqs.erase(it);
    if (st != VT_OK)
        return fail(st, st == VT_ECANCELED ? "vt_serve_poll: service stopped before the request ran"
                                           : "vt_serve_poll: request failed");
    return VT_OK;
}

int32_t vt_serve_get_stats(int32_t service, vt_serve_stats* out) {
    std::shared_ptr<Service> s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_get_stats: unknown service");
    if (!out) return fail(VT_EINVAL, "vt_serve_get_stats: null output");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->resident_bytes = s->resident_bytes;
    out->pending = s->pending.size();
    return VT_OK;
}

int32_t vt_serve_stop(int32_t service) {
    std::shared_ptr<Service> s;
    {
        std::lock_guard<std::mutex> lk(g_serve_mu);
        if (service < 0 || (size_t)service >= g_services.size() || !g_services[service])
            return fail(VT_ENOTFOUND, "vt_serve_stop: unknown service");
        s = std::move(g_services[service]);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    {
        // every request is now done or cancelled: wake pollers (they hold the service alive
        // until they return; its streams and grids go with the last reference)
        std::lock_guard<std::mutex> lk(s->mu);
        s->cv_done.notify_all();
    }
    return VT_OK;
}

}  // extern "C"
