// vt_kernels.h — host-callable launchers of libvtrace's CUDA kernels (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vtrace.h"

namespace vt {

struct GridView;
struct LightView;
struct Counters;

// Launch shape of the persistent tracers (picked by the autotuner).
struct TraceTuning {
    uint32_t refill_min = 16;  // refill a warp when at least this many lanes are idle (1..32)
    int blocks_per_sm = 0;     // 0: as many 256-thread blocks as fit on an SM
    uint32_t persistent = 1;   // 0: one thread per ray in 8 x 4 pixel tiles, no refill
    uint32_t wavefront = 0;    // render only: shadow rays in a second pass over a compacted queue
    uint32_t tile_shape = 0;   // render tile launch: VT_TILE_* pixels per warp
    uint32_t block_warps = 4;  // render tile launch: warps per block (1, 2, 4, 8)
};

// Render in two passes (primary rays, then the queued shadow rays); stream-ordered scratch.
cudaError_t launch_render_wavefront(const GridView& g, const vt_camera& cam,
                                    const LightView& light, uint4* out, cudaStream_t stream);

// Persistent whole-tile render whose shadow rays are queued per warp and traced in full warps.
cudaError_t launch_render_queued(const GridView& g, const vt_camera& cam, const LightView& light,
                                 uint4* out, unsigned long long* counter, const TraceTuning& tune,
                                 int sm_count, cudaStream_t stream);
cudaError_t launch_render_persistent(const GridView& g, const vt_camera& cam,
                                     const LightView& light, uint4* out,
                                     unsigned long long* counter, const TraceTuning& tune,
                                     int sm_count, cudaStream_t stream);
cudaError_t launch_trace_rays_persistent(const GridView& g, const vt_ray* rays, uint64_t n,
                                         uint4* out, unsigned long long* counter,
                                         const TraceTuning& tune, int sm_count,
                                         cudaStream_t stream,
                                         const unsigned int* n_dev = nullptr);

// `tune` selects the warp tile and block shape (nullptr: 8 x 4 pixels per warp, 4 warps).
cudaError_t launch_render(const GridView& g, const vt_camera& cam, const LightView& light,
                          uint4* out, Counters* counters, cudaStream_t stream, uint32_t row0 = 0,
                          uint32_t row1 = 0, const TraceTuning* tune = nullptr);
// Warp-time phase profile of one frame (vt_phase.cu): `totals` holds phase_profile_words() words,
// zeroed, and receives per kind and phase the warp cycles, then the passes, then the warp count.
unsigned phase_profile_words();
cudaError_t launch_render_phases(const GridView& g, const vt_camera& cam, const LightView& light,
                                 uint4* out, unsigned long long* totals, cudaStream_t stream);
// n_dev as for launch_trace_rays_persistent: the device-side ray count (at most n), or nullptr.
cudaError_t launch_trace_rays(const GridView& g, const vt_ray* rays, uint64_t n, uint4* out,
                              Counters* counters, cudaStream_t stream,
                              const unsigned int* n_dev = nullptr);

// Scratch of one brick build, sized for `bricks` bricks.
struct BuildScratch {
    uint64_t* words = nullptr;      // bricks * 8 occupancy words
    uint32_t* flags = nullptr;      // bricks: 1 if the brick holds an occupied voxel
    uint32_t* offsets = nullptr;    // bricks: exclusive prefix sum of flags (the slot)
    uint32_t* block_sums = nullptr; // scan partials
    unsigned long long* occupied = nullptr;
    uint8_t* dist_a = nullptr;      // bricks: distance transform, first pass
    uint8_t* dist_b = nullptr;      // bricks: distance transform, second pass
    // nullptr, or build_staging_bytes(): the voxels of each occupied brick as a 512-voxel block
    // at brick * 512, written by the words pass and copied by the compaction
    void* staged = nullptr;
};
size_t build_scratch_bytes(uint64_t bricks);
size_t build_staging_bytes(uint64_t bricks, uint32_t format);
// Carves BuildScratch out of one buffer of build_scratch_bytes(bricks) bytes.
BuildScratch carve_build_scratch(void* base, uint64_t bricks);

// Phase 1: occupancy words, brick flags and the occupied-voxel count; phase 2: slots.
cudaError_t launch_brick_words(const void* src, uint32_t format, const uint32_t* d_palette,
                               int32_t nx, int32_t ny, int32_t nz, const BuildScratch& s,
                               cudaStream_t stream, bool nonzero_occupancy = false);
cudaError_t launch_brick_scan(const BuildScratch& s, uint64_t bricks, cudaStream_t stream);
// Dense z-fastest input (element size 1 or 4) to x-fastest; y-planes are transposed in place of
// the x and z axes.  grid.y = ceil(nx / 32) and grid.z = ny must stay within 65535.
cudaError_t launch_transpose_xz(const void* src, void* dst, size_t elem, int32_t nx, int32_t ny,
                                int32_t nz, cudaStream_t stream);
// Phase 3: directory, compacted masks and payloads.
cudaError_t launch_brick_compact(const void* src, uint32_t format, int32_t nx, int32_t ny,
                                 int32_t nz, const BuildScratch& s, uint32_t* dir,
                                 uint64_t* masks, void* payload, cudaStream_t stream);

// Phase 5: forward distances per ray octant (4 bits x 8 per brick) into `oct`; tmp_x holds one
// byte and tmp_y two bytes per brick.
// A box of bricks: origin and extent in brick coordinates.
struct BrickBox {
    int32_t x0, y0, z0, nx, ny, nz;
};
// Octant words of every brick, or (changed != nullptr) of the bricks a change of occupancy inside
// `changed` can affect.
cudaError_t launch_brick_octants(const uint32_t* dir, uint8_t* tmp_x, uint16_t* tmp_y,
                                 uint32_t* oct, int32_t bx, int32_t by, int32_t bz,
                                 cudaStream_t stream, const BrickBox* changed = nullptr,
                                 const uint32_t* occ = nullptr);
// Occupancy bitmask of the directory (brick_xmask_words() words: one bit per brick, rows along x
// padded to 32 bits), from which the passes along x read their distances when it is given
// (`occ` of the distance, octant and long-box launches) instead of scanning the directory; with
// `changed`, only the rows those passes read after a change inside it.
cudaError_t launch_brick_xmask(const uint32_t* dir, uint32_t* occ, int32_t bx, int32_t by,
                               int32_t bz, cudaStream_t stream, const BrickBox* changed = nullptr);
size_t brick_xmask_words(int32_t bx, int32_t by, int32_t bz);

// Phase 4: Chebyshev distance of every empty brick to the nearest occupied one, into dir.
// Long forward boxes (3 words per brick, axis-major) from the directory and the octant words, for
// every brick or (changed != nullptr) for the bricks a change inside `changed` can affect; tmp
// holds brick_long_scratch_words() words (13 per brick for a full pass, the runs of every brick
// and a windowed pyramid after a change).
cudaError_t launch_brick_long(const uint32_t* dir, const uint32_t* oct, uint32_t* tmp,
                              uint32_t* lng, int32_t bx, int32_t by, int32_t bz,
                              cudaStream_t stream, const BrickBox* changed = nullptr,
                              const uint32_t* occ = nullptr);
size_t brick_long_scratch_words(const BrickBox* changed, int32_t bx, int32_t by, int32_t bz);
cudaError_t launch_brick_distance(const BuildScratch& s, uint32_t* dir, int32_t bx, int32_t by,
                                  int32_t bz, cudaStream_t stream,
                                  const BrickBox* changed = nullptr, const uint32_t* occ = nullptr);

}  // namespace vt
