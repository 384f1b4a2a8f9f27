// vt_lane.cuh — per-lane ray state machine of the persistent tracers (sm_103a).
//
// A persistent warp keeps one ray per lane.  Each pass of its loop advances every live lane by
// one unit of traversal — one occupied brick walked voxel by voxel, or one empty region crossed
// per axis (cross_region) — so lanes whose rays end can be refilled with new rays between
// units instead of idling until the longest ray of the warp is done.  The units are the loop
// body of dda_skip(), split so that the loop state lives in LaneRay; results are identical.
#pragma once

#include "vt_device.cuh"

namespace vt {

enum : int { kRayRunning = 0, kRayHit = 1, kRayMiss = 2 };

struct LaneRay {
    float o[3], d[3];
    float sx, sy, sz, dlx, dly, dlz;
    int32_t vx, vy, vz, stx, sty, stz;
    uint32_t slot;
    int32_t guard;
    int32_t entry_axis;  // slab entry face axis, -1 when the origin is inside the grid
    float t_entry;
    bool mx, my, mz;     // axes stepped on the final iteration
    uint32_t flags;      // VT_HIT_FLAG_INVALID for rejected input
    uint32_t oshift;     // nibble of the ray's octant in the octant words
    int32_t dom;         // dominant axis of the direction
};

// Validity, slab entry and DDA set-up (trace.frag:68-71).  Returns kRayRunning, or the final
// status when the ray is already decided (rejected input, grid missed, or a degenerate direction
// resolved by the literal loop).
__device__ __forceinline__ int ray_begin(const GridView& g, const float o[3], const float d[3],
                                         LaneRay& R) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        R.o[a] = o[a];
        R.d[a] = d[a];
    }
    R.flags = 0;
    R.mx = R.my = R.mz = false;
    R.slot = kEmptyBit;
    if (!finite3(o) || !finite3(d)) {
        R.flags = VT_HIT_FLAG_INVALID;
        return kRayMiss;
    }
    float pos[3];
    int axis;
    const int kind = slab_entry(g, o, d, pos, R.t_entry, axis);
    if (kind == 0) return kRayMiss;
    R.entry_axis = kind == 1 ? axis : -1;
    const float len = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
    dda_setup_axis(pos[0], d[0], g.nx, len, R.vx, R.stx, R.dlx, R.sx);
    dda_setup_axis(pos[1], d[1], g.ny, len, R.vy, R.sty, R.dly, R.sy);
    dda_setup_axis(pos[2], d[2], g.nz, len, R.vz, R.stz, R.dlz, R.sz);
    if (isnan(R.sx) || isnan(R.sy) || isnan(R.sz)) {
        DDAResult r;
        Tally<false> tl;
        dda_literal<false>(g, R.vx, R.vy, R.vz, R.stx, R.sty, R.stz, R.dlx, R.dly, R.dlz, R.sx,
                           R.sy, R.sz, r, tl);
        R.vx = r.vx;
        R.vy = r.vy;
        R.vz = r.vz;
        R.slot = r.slot;
        R.mx = (r.last & 1) != 0;
        R.my = (r.last & 2) != 0;
        R.mz = (r.last & 4) != 0;
        return r.hit ? kRayHit : kRayMiss;
    }
    R.guard = g.nx + g.ny + g.nz + 2;
    R.oshift = octant_shift(R.stx, R.sty, R.stz);
    R.dom = dominant_axis(d[0], d[1], d[2]);
    return grid_inside(g, R.vx, R.vy, R.vz) ? kRayRunning : kRayMiss;
}

// Directory entry of the lane's current brick.
__device__ __forceinline__ uint32_t ray_entry(const GridView& g, const LaneRay& R) {
    const uint32_t bidx = (uint32_t)(R.vx >> 3) + (uint32_t)g.bx * ((uint32_t)(R.vy >> 3) + (uint32_t)g.by * (uint32_t)(R.vz >> 3));
    return __ldg(g.dir + bidx);
}

// One unit of traversal: the rest of the current occupied brick voxel by voxel, or the crossing
// of the empty region around the current brick (`e`: its directory entry, ray_entry()).  Same
// arithmetic as dda_skip().
__device__ __forceinline__ int ray_unit(const GridView& g, LaneRay& R, uint32_t e) {
    int32_t vx = R.vx, vy = R.vy, vz = R.vz;
    const int32_t stx = R.stx, sty = R.sty, stz = R.stz;
    float sx = R.sx, sy = R.sy, sz = R.sz;
    const float dlx = R.dlx, dly = R.dly, dlz = R.dlz;
    bool mx = R.mx, my = R.my, mz = R.mz;
    int status = kRayRunning;
    const int32_t bxi = vx >> 3, byi = vy >> 3, bzi = vz >> 3;
    if (!brick_empty(e)) {
        const uint64_t* mk = g.masks + (size_t)e * 8;
        // brick-local walk to the brick's face, as in dda_skip (left within 22 iterations)
        int32_t lx = vx & 7, ly = vy & 7, lz = vz & 7;
        for (;;) {
            const uint64_t w = __ldg(mk + lz);
            if ((w >> ((ly << 3) | lx)) & 1ull) {
                status = kRayHit;
                R.slot = e;
                break;
            }
            VT_DDA_STEP_LOCAL
            if ((lx | ly | lz) & ~7) break;
        }
        vx = (bxi << 3) + lx;
        vy = (byi << 3) + ly;
        vz = (bzi << 3) + lz;
    } else {
        const uint32_t bidx = (uint32_t)bxi + (uint32_t)g.bx * ((uint32_t)byi + (uint32_t)g.by * (uint32_t)bzi);
        const uint32_t ow = octant_word(g, bidx);
        const uint32_t* lp = long_words(g, R.dom);
        const uint32_t lw = lp ? __ldg(lp + bidx) : 0u;
        int32_t nxe, nye, nze;
        empty_moves(g, e, ow, lw, bxi, byi, bzi, vx, vy, vz, stx, sty, stz, R.oshift, R.dom, nxe,
                    nye, nze);
        cross_region(sx, sy, sz, vx, vy, vz, dlx, dly, dlz, stx, sty, stz, nxe, nye, nze, mx, my,
                     mz);
    }
    if (status == kRayRunning && (!grid_inside(g, vx, vy, vz) || --R.guard <= 0)) status = kRayMiss;
    R.vx = vx;
    R.vy = vy;
    R.vz = vz;
    R.sx = sx;
    R.sy = sy;
    R.sz = sz;
    R.mx = mx;
    R.my = my;
    R.mz = mz;
    return status;
}

__device__ __forceinline__ int ray_unit(const GridView& g, LaneRay& R) {
    return ray_unit(g, R, ray_entry(g, R));
}

// Record of a finished ray (unshaded colour; misses carry `miss_rgba`).
__device__ __forceinline__ HitRec ray_record(const GridView& g, const LaneRay& R, int status,
                                             uint32_t miss_rgba) {
    if (status != kRayHit) return miss_rec(R.flags, miss_rgba);
    const int32_t last = (R.mx ? 1 : 0) | (R.my ? 2 : 0) | (R.mz ? 4 : 0);
    return hit_record(g, R.o, R.d, R.vx, R.vy, R.vz, last, R.slot, R.entry_axis, R.t_entry);
}

// Warp-aggregated work fetch: every idle lane of the warp gets the next item index from
// `counter` (one atomic per warp).  Returns the number of items handed out to the warp; an idle
// lane's item is `first + rank`, valid when below `total`.
__device__ __forceinline__ uint64_t warp_fetch(unsigned long long* counter, uint32_t idle,
                                               uint32_t lane, uint64_t& my_item) {
    const uint32_t n = __popc(idle);
    const int leader = __ffs(idle) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)n);
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    my_item = base + __popc(idle & ((1u << lane) - 1u));
    return base;
}

}  // namespace vt
