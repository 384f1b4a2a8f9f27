// vt_batch.h — batched multi-view launch shared by vt_batch.cu and vt_serve.cu (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vt_api_internal.h"
#include "vt_device.cuh"

namespace vt {

constexpr uint32_t kMaxBatchViews = 256;

// One view of a batched launch, as the kernel reads it (the table is copied to shared memory).
// A view may cover only the tile rows from `first_item` on (a piece of a larger image, as the
// render service splits big requests); its records are then written at their image index minus
// `rec_offset`.
struct BatchView {
    GridView g;
    vt_camera cam;
    LightView light;
    uint4* out;                     // per-sample records, [(py * width + px) * spp + s - rec_offset]
    unsigned long long begin;       // first work item of the view in the launch
    unsigned long long first_item;  // the view's own item the launch's item `begin` stands for
    uint32_t rec_offset;
    uint32_t tiles_x;
    uint32_t spp;
    uint32_t seed;
    uint32_t view_id;
    uint32_t wx_log;  // pixel tile of a work unit: (1 << wx_log) x (32 >> wx_log) pixels
};
static_assert(sizeof(BatchView) % 16 == 0, "view table entries stay 16-byte aligned");

// Work items of a view: pixel tiles of (1 << wx_log) x (32 >> wx_log) (8 x 4 by default) x spp x
// 32 lanes.
uint64_t batch_view_items(const vt_camera& cam, uint32_t spp, uint32_t wx_log = 3);
// Work items of rows row0 .. row1 - 1 of a view (row0 a multiple of the tile height).
uint64_t batch_rows_items(const vt_camera& cam, uint32_t spp, uint32_t row0, uint32_t row1,
                          uint32_t wx_log = 3);
BatchView make_batch_view(const Grid& g, const vt_camera& cam, const vt_light* light,
                          uint32_t spp, uint32_t seed, uint32_t view_id, void* out,
                          uint64_t begin, uint32_t row0 = 0, uint32_t wx_log = 3);
// log2 of a VT_TILE_* shape's width.
uint32_t tile_wx_log(uint32_t tile_shape);
// Blocks of a persistent batched launch over `total` items with an `n`-view table.
unsigned batch_blocks(uint32_t n, uint64_t total, const TraceTuning& tune);
// Counter reset + persistent kernel over a device view table.
cudaError_t launch_batch(const BatchView* d_table, uint32_t n, uint64_t total,
                         unsigned long long* counter, const TraceTuning& tune, unsigned blocks,
                         cudaStream_t stream);

}  // namespace vt
