// vt_trace.cu — traversal kernels of libvtrace: per-pixel render and ray-buffer trace.
#include <cuda_runtime.h>

#include "vt_device.cuh"
#include "vt_kernels.h"

namespace vt {

// Image tile of one warp: 8 x 4 pixels, so that a warp's rays start together and stay coherent.
// A 256-thread block covers 16 x 16 pixels (2 x 4 warps).
constexpr int kTileW = 16, kTileH = 16;

template <bool STATS>
__global__ void __launch_bounds__(256) render_kernel(GridView g, vt_camera cam, LightView light,
                                                     uint4* __restrict__ out,
                                                     Counters* __restrict__ counters) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t px = blockIdx.x * kTileW + (warp & 1u) * 8u + (lane & 7u);
    const uint32_t py = blockIdx.y * kTileH + (warp >> 1) * 4u + (lane >> 3);
    if (px >= cam.width || py >= cam.height) return;
    Tally<STATS> tl;
    float o[3], d[3];
    raygen(cam, px, py, 0.5f, 0.5f, o, d);
    const HitRec h = shade_ray<STATS>(g, light, o, d, tl);
    out[(size_t)py * cam.width + px] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    tl.flush(counters);
}

template <bool STATS>
__global__ void __launch_bounds__(256) trace_rays_kernel(GridView g,
                                                         const float2* __restrict__ rays,
                                                         uint64_t n, uint4* __restrict__ out,
                                                         Counters* __restrict__ counters) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Tally<STATS> tl;
    // 24-byte rays: three 8-byte loads
    const float2 a = __ldg(rays + 3 * i), b = __ldg(rays + 3 * i + 1), c = __ldg(rays + 3 * i + 2);
    const float o[3] = {a.x, a.y, b.x}, d[3] = {b.y, c.x, c.y};
    const HitRec h = trace_ray<STATS>(g, o, d, tl);
    out[i] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    tl.flush(counters);
}

cudaError_t launch_render(const GridView& g, const vt_camera& cam, const LightView& light,
                          uint4* out, Counters* counters, cudaStream_t stream) {
    dim3 grid((cam.width + kTileW - 1) / kTileW, (cam.height + kTileH - 1) / kTileH);
    if (counters)
        render_kernel<true><<<grid, 256, 0, stream>>>(g, cam, light, out, counters);
    else
        render_kernel<false><<<grid, 256, 0, stream>>>(g, cam, light, out, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const GridView& g, const vt_ray* rays, uint64_t n, uint4* out,
                              Counters* counters, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = (n + 255) / 256;
    const float2* r2 = reinterpret_cast<const float2*>(rays);
    if (counters)
        trace_rays_kernel<true><<<(unsigned)blocks, 256, 0, stream>>>(g, r2, n, out, counters);
    else
        trace_rays_kernel<false><<<(unsigned)blocks, 256, 0, stream>>>(g, r2, n, out, nullptr);
    return cudaGetLastError();
}

}  // namespace vt
