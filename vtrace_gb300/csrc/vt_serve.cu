// vt_serve.cu — continuous-batching render service.
//
// Requests (scene, camera, resolution, spp, light) arrive from any thread through
// vt_serve_submit.  A dispatcher thread keeps up to `max_inflight` launches on the device at once,
// each on its own stream: whenever a launch slot is free it packs the oldest pending requests
// (up to `max_views_per_launch` views and `max_samples_per_launch` samples) into one persistent
// work-stealing launch of the batched kernel (vt_batch.cu), resolves every request's samples to an
// RGBA8 image, copies the images to the callers' host buffers and records an event.  Requests
// that arrive while launches are running are admitted into the next free slot, so work of
// different requests overlaps on the GPU.  Brick grids of the scenes stay resident in a cache
// bounded by an HBM budget: a scene is built on first use, and least-recently-used scenes that no
// in-flight request references are evicted to make room.  Every request's image depends only on
// its own parameters (per-sample Philox jitter keyed by seed and view id), so it is the same alone
// and in any mix of requests.
//
// With max_inflight = 1 and max_views_per_launch = 1 the same machinery is the plain baseline:
// one launch per request, one launch at a time, in arrival order.
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
    int32_t refs = 0;
    bool loading = false;
    uint64_t last_use = 0;
    uint64_t bytes = 0;
};

struct ServeReq {
    vt_serve_request r;
    int32_t status = VT_ENOTREADY;
    int64_t t_submit = 0, t_launch = 0, t_done = 0;
    uint64_t samples = 0;
    void* d_samples = nullptr;
    void* d_image = nullptr;
    void* h_image = nullptr;  // device address of a page-locked host_rgba, written directly
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
    std::vector<uint64_t> reqs;
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
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, ServeReq> reqs;
    uint64_t next_id = 1;
    std::vector<Slot> slots;
    uint64_t resident_bytes = 0, tick = 0;
    vt_serve_stats stats;
    TraceTuning tune;
    std::atomic<int> pollers{0};  // threads inside vt_serve_poll (stop waits for them to leave)

    void run();
    int32_t admit_scene(std::unique_lock<std::mutex>& lk, int32_t scene);
    void evict_for(uint64_t need);
    void launch(Slot& slot, const std::vector<uint64_t>& ids);
    void retire(Slot& slot);
};

static std::mutex g_serve_mu;
static std::vector<std::unique_ptr<Service>> g_services;

static Service* lookup_service(int32_t id) {
    std::lock_guard<std::mutex> lk(g_serve_mu);
    if (id < 0 || (size_t)id >= g_services.size() || !g_services[id]) return nullptr;
    return g_services[id].get();
}

// Upper bound of a scene's resident bytes: directory + masks + payloads of every brick.
static uint64_t scene_bound(const ServeScene& s) {
    const uint64_t bricks = (uint64_t)((s.nx + 7) / 8) * ((s.ny + 7) / 8) * ((s.nz + 7) / 8);
    return bricks * (4 + 64 + 512) + 1024;
}

void Service::evict_for(uint64_t need) {
    while (resident_bytes + need > cfg.hbm_budget_bytes) {
        ServeScene* victim = nullptr;
        for (auto& s : scenes)
            if (s->grid >= 0 && s->refs == 0 && !s->loading &&
                (!victim || s->last_use < victim->last_use))
                victim = s.get();
        if (!victim) return;
        vt_grid_destroy(victim->grid);
        victim->grid = -1;
        resident_bytes -= victim->bytes;
        victim->bytes = 0;
        stats.evictions++;
    }
}

// Makes `scene` resident.  VT_OK, VT_EBUSY (no room until in-flight work ends), or an error.
int32_t Service::admit_scene(std::unique_lock<std::mutex>& lk, int32_t scene) {
    ServeScene& s = *scenes[scene];
    s.last_use = ++tick;
    if (s.grid >= 0) return VT_OK;
    const uint64_t need = scene_bound(s);
    if (need > cfg.hbm_budget_bytes) return VT_ENOMEM;
    evict_for(need);
    if (resident_bytes + need > cfg.hbm_budget_bytes) return VT_EBUSY;
    s.loading = true;
    resident_bytes += need;  // reserved while the grid is built outside the lock
    lk.unlock();
    const int32_t g = vt_grid_create_u8(s.voxels, s.palette, s.nx, s.ny, s.nz);
    vt_grid_info info;
    const bool ok = g >= 0 && vt_grid_get_info(g, &info) == VT_OK;
    lk.lock();
    s.loading = false;
    resident_bytes -= need;
    if (!ok) return g < 0 ? g : VT_ECUDA;
    s.grid = g;
    s.bytes = info.device_bytes;
    resident_bytes += s.bytes;
    stats.scene_loads++;
    return VT_OK;
}

void Service::launch(Slot& slot, const std::vector<uint64_t>& ids) {
    uint64_t item = 0, pixel = 0;
    uint32_t n = 0;
    std::vector<uint64_t> live;
    for (uint64_t id : ids) {
        ServeReq& q = reqs[id];
        const vt_serve_request& r = q.r;
        const uint64_t px = (uint64_t)r.camera.width * r.camera.height;
        Grid* g = lookup_grid(scenes[r.scene]->grid);
        // a page-locked output is written by the resolve kernel itself; else a device image and
        // a copy
        q.h_image = host_mapped(r.host_rgba);
        cudaError_t e = cudaMallocAsync(&q.d_samples, px * r.spp * 16, slot.stream);
        if (e == cudaSuccess && !q.h_image) e = cudaMallocAsync(&q.d_image, px * 4, slot.stream);
        if (e != cudaSuccess || !g) {
            cudaGetLastError();
            if (q.d_samples) cudaFreeAsync(q.d_samples, slot.stream);
            q.d_samples = nullptr;
            q.status = VT_ENOMEM;
            q.t_done = now_ns();
            continue;
        }
        slot.h_table[n] = make_batch_view(*g, r.camera, (r.flags & VT_VIEW_LIGHT) ? &r.light : nullptr,
                                          r.spp, r.seed, r.view_id, q.d_samples, item);
        slot.h_resolve[n].samples = (const uint4*)q.d_samples;
        slot.h_resolve[n].image = (uchar4*)(q.h_image ? q.h_image : q.d_image);
        slot.h_resolve[n].pixel_begin = pixel;
        slot.h_resolve[n].pixels = (uint32_t)px;
        slot.h_resolve[n].spp = r.spp;
        item += batch_view_items(r.camera, r.spp);
        pixel += px;
        ++n;
        scenes[r.scene]->refs++;
        q.t_launch = now_ns();
        live.push_back(id);
    }
    slot.reqs = live;
    if (n == 0) {
        cv_done.notify_all();
        return;
    }
    cudaEventRecord(slot.t_begin, slot.stream);
    cudaMemcpyAsync(slot.d_table, slot.h_table, n * sizeof(BatchView), cudaMemcpyHostToDevice,
                    slot.stream);
    cudaMemcpyAsync(slot.d_resolve, slot.h_resolve, n * sizeof(ResolveView),
                    cudaMemcpyHostToDevice, slot.stream);
    launch_batch(slot.d_table, n, item, slot.d_counter, tune, batch_blocks(n, item, tune),
                 slot.stream);
    const unsigned rblocks =
        (unsigned)std::min<uint64_t>((pixel + 255) / 256, (uint64_t)state().sm_count * 16);
    resolve_kernel<<<rblocks, 256, 0, slot.stream>>>(slot.d_resolve, n, pixel);
    for (uint64_t id : live) {
        ServeReq& q = reqs[id];
        const uint64_t px = (uint64_t)q.r.camera.width * q.r.camera.height;
        if (!q.h_image) {
            cudaMemcpyAsync(q.r.host_rgba, q.d_image, px * 4, cudaMemcpyDeviceToHost, slot.stream);
            cudaFreeAsync(q.d_image, slot.stream);
        }
        cudaFreeAsync(q.d_samples, slot.stream);
        q.d_samples = q.d_image = nullptr;
        q.h_image = nullptr;
    }
    cudaEventRecord(slot.t_end, slot.stream);
    cudaEventRecord(slot.done, slot.stream);
    slot.busy = true;
    stats.launches++;
    stats.views_launched += n;
}

void Service::retire(Slot& slot) {
    const int64_t t = now_ns();
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, slot.t_begin, slot.t_end) == cudaSuccess)
        stats.device_ns += (uint64_t)((double)ms * 1e6);
    else
        cudaGetLastError();
    for (uint64_t id : slot.reqs) {
        ServeReq& q = reqs[id];
        q.status = VT_OK;
        q.t_done = t;
        scenes[q.r.scene]->refs--;
        stats.completed++;
        stats.samples += q.samples;
    }
    slot.reqs.clear();
    slot.busy = false;
    cv_done.notify_all();
}

void Service::run() {
    cudaSetDevice(state().device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool busy = false;
        for (Slot& sl : slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess)
                retire(sl);
            else if (q == cudaErrorNotReady)
                busy = true;
            else {  // a failed launch: report it on its requests
                for (uint64_t id : sl.reqs) {
                    reqs[id].status = VT_ECUDA;
                    reqs[id].t_done = now_ns();
                    scenes[reqs[id].r.scene]->refs--;
                }
                sl.reqs.clear();
                sl.busy = false;
                cv_done.notify_all();
            }
        }
        if (stop) {
            for (uint64_t id : pending) {
                reqs[id].status = VT_ECANCELED;
                reqs[id].t_done = now_ns();
            }
            if (!pending.empty()) cv_done.notify_all();
            pending.clear();
            if (!busy) break;
        }
        // admit the oldest pending requests into free slots
        for (Slot& sl : slots) {
            if (sl.busy || pending.empty() || stop) continue;
            std::vector<uint64_t> pack;
            uint64_t samples = 0;
            while (!pending.empty() && pack.size() < cfg.max_views_per_launch) {
                const uint64_t id = pending.front();
                ServeReq& q = reqs[id];
                if (!pack.empty() && samples + q.samples > cfg.max_samples_per_launch) break;
                const int32_t rc = admit_scene(lk, q.r.scene);
                if (rc == VT_EBUSY) break;  // wait for memory (head of line keeps its place)
                pending.pop_front();
                if (rc != VT_OK) {
                    q.status = rc;
                    q.t_done = now_ns();
                    cv_done.notify_all();
                    continue;
                }
                scenes[q.r.scene]->refs++;  // held while packed; launch() takes its own
                pack.push_back(id);
                samples += q.samples;
            }
            for (uint64_t id : pack) scenes[reqs[id].r.scene]->refs--;
            if (!pack.empty()) launch(sl, pack);
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

extern "C" {

int32_t vt_serve_default_config(vt_serve_config* cfg) {
    if (!cfg) return fail(VT_EINVAL, "vt_serve_default_config: null config");
    cfg->hbm_budget_bytes = 120ull << 30;
    cfg->max_inflight = 4;
    cfg->max_views_per_launch = 64;
    cfg->max_samples_per_launch = 64ull << 20;
    cfg->poll_interval_us = 20;
    cfg->refill_min = 32;
    return VT_OK;
}

int32_t vt_serve_start(const vt_serve_config* cfg, int32_t* service_out) {
    if (!cfg || !service_out) return fail(VT_EINVAL, "vt_serve_start: null argument");
    if (cfg->max_inflight < 1 || cfg->max_inflight > 32 || cfg->max_views_per_launch < 1 ||
        cfg->max_views_per_launch > kMaxBatchViews || cfg->refill_min < 1 || cfg->refill_min > 32 ||
        cfg->max_samples_per_launch == 0)
        return fail(VT_EINVAL, "vt_serve_start: max_inflight 1..32, max_views_per_launch 1..256, "
                               "refill_min 1..32, max_samples_per_launch > 0");
    int32_t rc = ensure_init();
    if (rc) return rc;
    std::unique_ptr<Service> s(new Service());
    s->cfg = *cfg;
    if (s->cfg.poll_interval_us == 0) s->cfg.poll_interval_us = 20;
    memset(&s->stats, 0, sizeof(s->stats));
    s->tune.refill_min = cfg->refill_min;
    s->tune.blocks_per_sm = 0;
    s->tune.persistent = 1;
    s->slots.resize(cfg->max_inflight);
    for (Slot& sl : s->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.t_begin);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.t_end);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_table, kMaxBatchViews * sizeof(BatchView));
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_resolve, kMaxBatchViews * sizeof(ResolveView));
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_counter, sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_table, kMaxBatchViews * sizeof(BatchView));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_resolve, kMaxBatchViews * sizeof(ResolveView));
        if (e != cudaSuccess) return cuda_fail(e, "vt_serve_start: slot resources");
    }
    Service* raw = s.get();
    int32_t id;
    {
        std::lock_guard<std::mutex> lk(g_serve_mu);
        g_services.push_back(std::move(s));
        id = (int32_t)g_services.size() - 1;
    }
    raw->worker = std::thread([raw] { raw->run(); });
    *service_out = id;
    return VT_OK;
}

int32_t vt_serve_add_scene(int32_t service, const uint8_t* voxels, const uint32_t* palette,
                           uint32_t nx, uint32_t ny, uint32_t nz, int32_t* scene_out) {
    Service* s = lookup_service(service);
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
    s->scenes.push_back(std::move(sc));
    *scene_out = (int32_t)s->scenes.size() - 1;
    return VT_OK;
}

int32_t vt_serve_submit(int32_t service, const vt_serve_request* req, uint64_t* request_id) {
    const int64_t t = now_ns();
    Service* s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_submit: unknown service");
    if (!req || !request_id || !req->host_rgba) return fail(VT_EINVAL, "vt_serve_submit: null argument");
    int32_t rc = check_camera(&req->camera);
    if (rc) return rc;
    if (req->spp == 0 || req->spp > 64) return fail(VT_EINVAL, "vt_serve_submit: spp must be 1..64");
    if ((uint64_t)req->camera.width * req->camera.height * req->spp >= (1ull << 32))
        return fail(VT_ELIMIT, "vt_serve_submit: 2^32 or more samples in one request");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(VT_ECANCELED, "vt_serve_submit: service stopping");
    if (req->scene < 0 || (size_t)req->scene >= s->scenes.size())
        return fail(VT_ENOTFOUND, "vt_serve_submit: unknown scene");
    const uint64_t id = s->next_id++;
    ServeReq& q = s->reqs[id];
    q.r = *req;
    q.t_submit = t;
    q.samples = (uint64_t)req->camera.width * req->camera.height * req->spp;
    s->pending.push_back(id);
    s->stats.submitted++;
    *request_id = id;
    s->cv.notify_one();
    return VT_OK;
}

int32_t vt_serve_poll(int32_t service, uint64_t request_id, uint32_t timeout_us,
                      vt_serve_timing* timing) {
    Service* s = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_serve_mu);
        if (service >= 0 && (size_t)service < g_services.size() && g_services[service]) {
            s = g_services[service].get();
            s->pollers.fetch_add(1);
        }
    }
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_poll: unknown service");
    struct Leave {
        Service* s;
        ~Leave() { s->pollers.fetch_sub(1); }
    } leave{s};
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
    Service* s = lookup_service(service);
    if (!s) return fail(VT_ENOTFOUND, "vt_serve_get_stats: unknown service");
    if (!out) return fail(VT_EINVAL, "vt_serve_get_stats: null output");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->resident_bytes = s->resident_bytes;
    out->pending = s->pending.size();
    return VT_OK;
}

int32_t vt_serve_stop(int32_t service) {
    std::unique_ptr<Service> s;
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
    // every request is now done or cancelled: wake pollers and wait for them to leave
    while (s->pollers.load() > 0) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->cv_done.notify_all();
        }
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.t_begin) cudaEventDestroy(sl.t_begin);
        if (sl.t_end) cudaEventDestroy(sl.t_end);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        cudaFree(sl.d_table);
        cudaFree(sl.d_resolve);
        cudaFree(sl.d_counter);
        cudaFreeHost(sl.h_table);
        cudaFreeHost(sl.h_resolve);
    }
    for (auto& sc : s->scenes)
        if (sc->grid >= 0) vt_grid_destroy(sc->grid);
    return VT_OK;
}

}  // extern "C"
