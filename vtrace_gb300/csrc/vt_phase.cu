// vt_phase.cu — warp-time phase profile of the render kernel (vt_render_phases).
//
// The render kernel's body (render_pixel) built with the traversal's phase hooks compiled in: at
// each hook the lanes that reach it together synchronise, and the lowest of them reads the SM clock
// and charges the cycles since the warp's previous hook to that hook's phase of the current ray kind
// (camera or shadow).  The kind's first traversal pass charges the ray set-up (a kind with no pass
// charges it to its tail).  Per-warp state
// lives in shared memory and is added to the launch's totals when the warp ends.  This measures
// where each warp spends its residency, load latency included; in an issue-bound launch other warps
// issue during that latency, so a phase's share of warp time is not its share of issue slots.
#define VT_PHASE_CLOCKS 1

#include <cuda_runtime.h>
#include <stdint.h>

#include "vtrace.h"

namespace vt {

constexpr int kPhaseWarps = 4;                           // 128-thread blocks
constexpr int kPhaseSlots = 2 * VT_PHASES + 4;           // cycles per kind, then passes
constexpr unsigned kPhaseOutWords = kPhaseSlots + 1;     // + warps

struct PhaseWarp {
    unsigned long long t;                  // clock at the warp's previous hook
    unsigned long long acc[kPhaseSlots];
    int kind;                              // 0 camera rays, 1 shadow rays
    int first;                             // no traversal pass of this kind yet
};

__shared__ PhaseWarp ph_warps[kPhaseWarps];

__device__ __forceinline__ bool phase_leader(uint32_t mask) {
    return (threadIdx.x & 31u) == (uint32_t)(__ffs(mask) - 1);
}

__device__ __forceinline__ void phase_mark(uint32_t mask, int phase) {
    __syncwarp(mask);
    const unsigned long long t = clock64();
    if (phase_leader(mask)) {
        PhaseWarp& w = ph_warps[threadIdx.x >> 5];
        if (w.first && phase == VT_PHASE_LOOP) phase = VT_PHASE_SETUP;
        w.first = 0;
        w.acc[w.kind * VT_PHASES + phase] += t - w.t;
        w.t = t;
    }
    __syncwarp(mask);
}

__device__ __forceinline__ void phase_pass(uint32_t mask, bool walk) {
    if (phase_leader(mask)) {
        PhaseWarp& w = ph_warps[threadIdx.x >> 5];
        w.acc[2 * VT_PHASES + 2 * w.kind + (walk ? 0 : 1)] += 1;
    }
}

__device__ __forceinline__ void phase_kind(uint32_t mask, int kind) {
    __syncwarp(mask);
    if (phase_leader(mask)) {
        ph_warps[threadIdx.x >> 5].kind = kind;
        ph_warps[threadIdx.x >> 5].first = 1;
    }
    __syncwarp(mask);
}

}  // namespace vt

#include "vt_device.cuh"
#include "vt_kernels.h"

namespace vt {

// render_kernel<false> with its default shape: 8 x 4-pixel warp tiles, 2 x 2 warps per block, ten
// blocks per SM as the render kernel's 48 registers allow.
__global__ void __launch_bounds__(kPhaseWarps * 32, 10) render_phase_kernel(
    GridView g, vt_camera cam, LightView light, uint4* __restrict__ out,
    unsigned long long* __restrict__ totals) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t px = blockIdx.x * 16u + (warp & 1u) * 8u + (lane & 7u);
    const uint32_t py = blockIdx.y * 8u + (warp >> 1) * 4u + (lane >> 3);
    const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, px < cam.width && py < cam.height);
    if (px >= cam.width || py >= cam.height) return;
    PhaseWarp& w = ph_warps[warp];
    if (phase_leader(vmask)) {
        for (int i = 0; i < kPhaseSlots; ++i) w.acc[i] = 0;
        w.kind = 0;
        w.first = 1;
        w.t = clock64();
    }
    __syncwarp(vmask);
    Tally<false> tl;
    const HitRec h = render_pixel<false>(g, cam, light, px, py, vmask, tl);
    out[(size_t)py * cam.width + px] = make_uint4(h.w0, h.w1, h.w2, h.w3);
    VT_PHASE_MARK(vmask, VT_PHASE_TAIL);
    if (phase_leader(vmask)) {
        for (int i = 0; i < kPhaseSlots; ++i) atomicAdd(totals + i, w.acc[i]);
        atomicAdd(totals + kPhaseSlots, 1ull);
    }
}

unsigned phase_profile_words() { return kPhaseOutWords; }

cudaError_t launch_render_phases(const GridView& g, const vt_camera& cam, const LightView& light,
                                 uint4* out, unsigned long long* totals, cudaStream_t stream) {
    const dim3 grid((cam.width + 15u) / 16u, (cam.height + 7u) / 8u);
    render_phase_kernel<<<grid, kPhaseWarps * 32, 0, stream>>>(g, cam, light, out, totals);
    return cudaGetLastError();
}

}  // namespace vt
