// vt_noalloc.cu — brick build that allocates nothing (vt_grid_build_u8_noalloc).
//
// For callers that cannot allocate device memory while they work: a chunk pager that rebuilds
// small grids every frame inside a real-time loop (cudaMalloc and cudaFree synchronise the whole
// device and would stall the frame), code recording into a stream that must not see an
// allocation, or a host that owns a fixed device memory budget.  Those callers pass every input
// and output buffer themselves; the build's scratch (occupancy words, brick flags, slots, scan
// partials, distance-transform passes) lives in the file-scope array below instead of a
// cudaMalloc'd buffer.  The kernels are the ones of the allocating build (vt_grid.cu).
#include <cuda_runtime.h>

#include <mutex>

#include "vt_device.cuh"
#include "vt_kernels.h"
#include "vtrace.h"

namespace vt {

// Largest grid the scratch covers: 32768 bricks (for example 256^3 voxels).  build_scratch_bytes
// of that many bricks is 2,425,600 bytes; the array is 2.5 MiB and is resident on every device
// that loads the library until the process exits.
constexpr uint64_t kNoAllocMaxBricks = 32768;
constexpr size_t kNoAllocScratchBytes = 2621440;

static __device__ __align__(256) unsigned char g_build_scratch[kNoAllocScratchBytes];

// Device address of g_build_scratch per device (its host-side name is only a stand-in), looked up
// by the first call on each device in the device's primary context (the runtime's), and
// forgotten by vt_shutdown.  A context the runtime did not create, or a device reset without
// vt_shutdown first, would leave a stale address here.
constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_scratch_mu;
static void* g_scratch_addr[kNoAllocMaxDevices] = {};

static cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_build_scratch);  // with `dev` current
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

void noalloc_forget_addresses() {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    for (int d = 0; d < kNoAllocMaxDevices; ++d) g_scratch_addr[d] = nullptr;
}

__global__ void noalloc_counts_kernel(const uint32_t* __restrict__ flags,
                                      const uint32_t* __restrict__ offsets, uint64_t bricks,
                                      const unsigned long long* __restrict__ occupied,
                                      uint64_t* __restrict__ counts) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        counts[0] = (uint64_t)offsets[bricks - 1] + flags[bricks - 1];
        counts[1] = *occupied;
    }
}

}  // namespace vt

using namespace vt;

extern "C" int32_t vt_grid_build_u8_noalloc(const uint8_t* d_voxels, const uint32_t* d_palette,
                                            uint32_t nx, uint32_t ny, uint32_t nz,
                                            uint32_t* d_directory, uint64_t* d_masks,
                                            uint8_t* d_payload, uint64_t* d_counts,
                                            void* stream) {
    if (!d_voxels || !d_palette || !d_directory || !d_masks || !d_payload || !d_counts)
        return VT_EINVAL;
    if (((uintptr_t)d_masks & 7u) || ((uintptr_t)d_payload & 7u) || ((uintptr_t)d_counts & 7u) ||
        ((uintptr_t)d_directory & 3u) || ((uintptr_t)d_palette & 3u))
        return VT_EINVAL;
    if (nx == 0 || ny == 0 || nz == 0 || nx > 65535 || ny > 65535 || nz > 65535) return VT_EINVAL;
    const uint64_t bricks = (uint64_t)((nx + 7) / 8) * ((ny + 7) / 8) * ((nz + 7) / 8);
    if (bricks > kNoAllocMaxBricks || build_scratch_bytes(bricks) > kNoAllocScratchBytes)
        return VT_ELIMIT;
    void* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) return VT_ECUDA;
    cudaStream_t st = (cudaStream_t)stream;
    const BuildScratch s = carve_build_scratch(scratch, bricks);
    const int32_t bx = (int32_t)((nx + 7) / 8), by = (int32_t)((ny + 7) / 8),
                  bz = (int32_t)((nz + 7) / 8);
    if (launch_brick_words(d_voxels, VT_PAYLOAD_U8, d_palette, (int32_t)nx, (int32_t)ny,
                           (int32_t)nz, s, st) != cudaSuccess ||
        launch_brick_scan(s, bricks, st) != cudaSuccess ||
        launch_brick_compact(d_voxels, VT_PAYLOAD_U8, (int32_t)nx, (int32_t)ny, (int32_t)nz, s,
                             d_directory, d_masks, d_payload, st) != cudaSuccess ||
        launch_brick_distance(s, d_directory, bx, by, bz, st) != cudaSuccess)
        return VT_ECUDA;
    noalloc_counts_kernel<<<1, 32, 0, st>>>(s.flags, s.offsets, bricks, s.occupied, d_counts);
    return cudaGetLastError() == cudaSuccess ? VT_OK : VT_ECUDA;
}
