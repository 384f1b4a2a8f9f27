// vt_api_internal.h — library state shared by the C ABI translation units (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "vt_kernels.h"
#include "vtrace.h"

namespace vt {

struct GridView;
struct LightView;
struct Counters;

constexpr uint32_t kMaxDim = 65535;
constexpr size_t kMaxGrids = 1u << 20;

// A brick grid resident in device memory.
struct Grid {
    uint32_t nx = 0, ny = 0, nz = 0, bx = 0, by = 0, bz = 0;
    uint64_t bricks = 0, nonempty = 0, occupied = 0;
    uint32_t format = VT_PAYLOAD_U8;
    uint32_t* dir = nullptr;
    uint32_t* oct = nullptr;  // forward distances per ray octant
    uint32_t* lng = nullptr;  // long forward boxes, 3 words per brick
    uint64_t* masks = nullptr;
    void* payload = nullptr;
    uint32_t* palette = nullptr;
    // one allocation holding dir, oct, lng and palette, and masks and payload until an update
    // grows the slots into separate allocations
    void* block = nullptr;
    size_t block_bytes = 0;
    bool pooled = false;  // `block` comes from the stream-ordered pool
    size_t bytes = 0;
    // slots of masks/payload: allocated, handed out (high-water mark), and freed by updates
    uint64_t slot_capacity = 0, slots_used = 0;
    std::vector<uint32_t> free_slots;
    std::atomic<int32_t> refs{0};  // in-flight batches / serving requests using the grid
    GridView view() const;
    bool in_block(const void* p) const;
    void free_slot_arrays();  // masks and payload (when not inside `block`)
    void release();
};

struct State {
    std::mutex mu;       // grid table and initialisation
    std::mutex host_mu;  // staging buffer of the *_host calls
    bool inited = false;
    int32_t device = 0;
    int32_t sm_count = 0;
    cudaStream_t stream = nullptr;
    // helper streams of the host-buffer calls: copies of one band overlap the next band's work
    static constexpr int kAux = 4;
    cudaStream_t aux[kAux] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t aux_start = nullptr;
    std::vector<cudaEvent_t> chunk_events;  // ordering of the pipelined host-buffer pieces
    std::vector<std::unique_ptr<Grid>> grids;
    // bumped whenever a grid is created, destroyed or changed in place (its device views change)
    std::atomic<uint64_t> grid_epoch{0};
    void* staging = nullptr;
    size_t staging_bytes = 0;
    // work counters of the persistent launches: each launch takes the next slot of the ring
    unsigned long long* counters = nullptr;
    std::atomic<uint32_t> counter_next{0};
    // defaults from sweeps on GB300: coherent camera rays keep their 8 x 4 tiles (refills would
    // mix tiles), incoherent ray buffers and path tracing refill a warp once 8 lanes are idle
    TraceTuning tune_render{16, 0, 0, 0, VT_TILE_8X4, 4}, tune_rays{8, 0, 1, 0, VT_TILE_8X4, 4},
        tune_batch{32, 0, 1, 0, VT_TILE_8X4, 4}, tune_path{8, 0, 1, 1, VT_TILE_8X4, 4};
};

constexpr uint32_t kCounterRing = 4096;
// Work counter for one persistent launch (zeroed by the launcher on its stream).
unsigned long long* next_counter();

// The timed launches of vt_render / vt_trace_rays, in the shape the current tuning selects.
cudaError_t launch_frame(const GridView& g, const vt_camera& cam, const LightView& light,
                         uint4* out, cudaStream_t stream);
cudaError_t launch_rays(const GridView& g, const vt_ray* rays, uint64_t n, uint4* out,
                        cudaStream_t stream);

State& state();
int32_t ensure_init();
int32_t cuda_fail(cudaError_t e, const char* what);
cudaStream_t pick_stream(void* stream);
Grid* lookup_grid(int32_t id);
int32_t register_grid(std::unique_ptr<Grid> g);
int32_t check_dims(uint32_t nx, uint32_t ny, uint32_t nz);
// Device bytes of a grid of `bricks` bricks when every brick is occupied: the most its one
// allocation can hold (directory, octant and long-box words, palette, masks, payloads).
uint64_t grid_bytes_bound(uint64_t bricks, uint32_t format);
int32_t check_camera(const vt_camera* cam);
// Device address of page-locked, 16-byte aligned host memory (kernels write outputs there
// directly), or nullptr for any other pointer.
void* host_mapped(void* p);
// Address a kernel can use for `p`: device or managed memory as is, page-locked host memory
// through its device mapping; nullptr for memory the device cannot reach (pageable host memory,
// unknown pointers).
void* device_address(void* p);
LightView light_view(const vt_light* light);
// Traversal counters of a counting launch as the ABI reports them.
void stats_from(const Counters& c, vt_trace_stats* st);
int32_t build_grid(const void* d_src, uint32_t format, const uint32_t* palette_host,
                   uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t stream,
                   std::unique_ptr<Grid>& out);

}  // namespace vt

// Release hooks of the other subsystems, called by vt_shutdown.
void vt_compat_release();
void vt_batch_release_all();
void vt_serve_release_all();
namespace vt {
// Forget the cached device addresses of vt_grid_build_u8_noalloc's scratch (vt_shutdown).
void noalloc_forget_addresses();
}  // namespace vt
