// vt_device.cuh — device-side traversal of libvtrace (sm_103a).
//
// The arithmetic restates vtrace's fragment shader (shaders/trace.frag:68-87) operation for
// operation in IEEE binary32 round-to-nearest, written with explicit __f*_rn intrinsics so that no
// multiply-add is ever contracted.  The grid is read through the brick layout built by
// vt_grid.cu:
//   dir[brick]            occupied 8^3 brick: its slot (bit 31 clear); empty brick: kEmptyBit |
//                         Chebyshev distance in bricks to the nearest occupied brick (>= 1,
//                         capped at kMaxBrickDistance); brick = bx + BX * (by + BY * bz)
//   masks[slot * 8 + lz]  u64 occupancy of z-slice lz, bit (ly * 8 + lx)
//   payload[slot*512+li]  voxel value at li = lx + 8 * (ly + 8 * lz) (u8 index or RGBA8)
// A voxel is occupied iff its colour's alpha byte is nonzero (trace.frag:78).
#pragma once

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "vtrace.h"

// Hooks of the warp-time phase profile (vt_render_phases): they compile to nothing unless the
// translation unit defines VT_PHASE_CLOCKS together with vt::phase_mark, vt::phase_pass and
// vt::phase_kind (vt_phase.cu), so every other kernel is built without them.
#ifdef VT_PHASE_CLOCKS
#define VT_PHASE_MARK(mask, phase) phase_mark((mask), (phase))
#define VT_PHASE_PASS(mask, walk) phase_pass((mask), (walk))
#define VT_PHASE_KIND(mask, kind) phase_kind((mask), (kind))
#else
#define VT_PHASE_MARK(mask, phase) ((void)0)
#define VT_PHASE_PASS(mask, walk) ((void)0)
#define VT_PHASE_KIND(mask, kind) ((void)0)
#endif

namespace vt {

constexpr uint32_t kEmptyBit = 0x80000000u;
constexpr uint32_t kMaxBrickDistance = 31;

__device__ __forceinline__ bool brick_empty(uint32_t e) { return (e & kEmptyBit) != 0u; }

struct GridView {
    const uint32_t* dir;
    const uint32_t* oct;  // forward distances per ray octant (4 bits x 8), or nullptr
    const uint32_t* lng;  // long forward boxes: 3 words per brick, axis-major (lng[a * bricks +
                          // brick], 4 bits x 8 octants), or nullptr
    const uint64_t* masks;
    const uint8_t* payload8;    // VT_PAYLOAD_U8
    const uint32_t* payload32;  // VT_PAYLOAD_RGBA8
    const uint32_t* palette;    // 256 entries (VT_PAYLOAD_U8)
    int32_t nx, ny, nz;
    int32_t bx, by, bz;
    uint32_t max_steps;  // nx + ny + nz (trace.frag:74)
    uint32_t format;
    uint32_t bricks;     // bx * by * bz
};

struct LightView {
    float dx, dy, dz;
    float ambient;
    uint32_t enabled;
    uint32_t shadows;
};

// Traversal counters of the counting kernels (vt_trace_stats).
struct GridView;

struct Counters {
    unsigned long long rays, shadow_rays, hits, steps, bricks, nonempty, tested, ties;
    // nullptr, or three bitmaps of ceil(bricks / 32) words: bricks entered, occupied bricks
    // entered, bricks holding a hit voxel (the launch's distinct footprint)
    unsigned int* touched;
};

template <bool STATS>
struct Tally {
    __device__ __forceinline__ void rays() {}
    __device__ __forceinline__ void shadow() {}
    __device__ __forceinline__ void hit() {}
    __device__ __forceinline__ void steps(uint32_t) {}
    __device__ __forceinline__ void brick() {}
    __device__ __forceinline__ void nonempty() {}
    __device__ __forceinline__ void tested() {}
    __device__ __forceinline__ void tie() {}
    __device__ __forceinline__ void flush(Counters*) {}
    __device__ __forceinline__ void bind(const Counters*, uint32_t) {}
    __device__ __forceinline__ void mark(uint32_t, int) {}
};

template <>
struct Tally<true> {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0};
    __device__ __forceinline__ void rays() { c.rays++; }
    __device__ __forceinline__ void shadow() { c.shadow_rays++; }
    __device__ __forceinline__ void hit() { c.hits++; }
    __device__ __forceinline__ void steps(uint32_t n) { c.steps += n; }
    __device__ __forceinline__ void brick() { c.bricks++; }
    __device__ __forceinline__ void nonempty() { c.nonempty++; }
    __device__ __forceinline__ void tested() { c.tested++; }
    __device__ __forceinline__ void tie() { c.ties++; }
    unsigned int* fp = nullptr;
    uint32_t fp_words = 0;
    // footprint bitmaps of the launch, if the counters carry them (`bricks` of the grid)
    __device__ __forceinline__ void bind(const Counters* g, uint32_t bricks) {
        if (g && g->touched) {
            fp = g->touched;
            fp_words = (bricks + 31u) / 32u;
        }
    }
    // set bit `b` of footprint map `m` (read first: most bricks are already marked)
    __device__ __forceinline__ void mark(uint32_t b, int m) {
        if (!fp) return;
        unsigned int* w = fp + (size_t)m * fp_words + (b >> 5);
        const unsigned int bit = 1u << (b & 31u);
        if (!(*(volatile unsigned int*)w & bit)) atomicOr(w, bit);
    }
    __device__ __forceinline__ void flush(Counters* g) {
        atomicAdd(&g->rays, c.rays);
        atomicAdd(&g->shadow_rays, c.shadow_rays);
        atomicAdd(&g->hits, c.hits);
        atomicAdd(&g->steps, c.steps);
        atomicAdd(&g->bricks, c.bricks);
        atomicAdd(&g->nonempty, c.nonempty);
        atomicAdd(&g->tested, c.tested);
        atomicAdd(&g->ties, c.ties);
    }
};

// GLSL min(x, y) := (y < x) ? y : x (GLSL 4.60 section 8.3).
__device__ __forceinline__ float glsl_min(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float glsl_sign(float x) {
    return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f);
}

// trace.frag:68-71 for one axis.
__device__ __forceinline__ void dda_setup_axis(float p, float d, int32_t n, float len, int32_t& v,
                                               int32_t& st, float& delta, float& side) {
    const float m = glsl_min(p, __fsub_rn(__int2float_rn(n), 1.0f));
    v = (int32_t)floorf(m);
    const float sg = glsl_sign(d);
    st = (int32_t)sg;
    delta = fabsf(__fdiv_rn(len, d));
    side = __fmul_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(sg, __fsub_rn(__int2float_rn(v), p)), __fmul_rn(sg, 0.5f)),
                  0.5f),
        delta);
}

struct DDAResult {
    int32_t vx, vy, vz;
    uint32_t steps;
    uint32_t slot;  // brick slot of the final voxel when hit
    int32_t last;   // axes stepped on the final iteration (bit 0 = x)
    bool hit;
    bool tie;
};

__device__ __forceinline__ bool grid_inside(const GridView& g, int32_t x, int32_t y, int32_t z) {
    return (uint32_t)x < (uint32_t)g.nx && (uint32_t)y < (uint32_t)g.ny &&
           (uint32_t)z < (uint32_t)g.nz;
}

// The literal loop of trace.frag:73-87, used when a side distance is NaN (degenerate
// directions: zero length, or a component so small that len/d overflows while the side term is
// zero).  GLSL min semantics are kept exactly; the step counter bounds the loop.
template <bool STATS>
__device__ __forceinline__ void dda_literal(const GridView& g, int32_t vx, int32_t vy, int32_t vz,
                                         int32_t stx, int32_t sty, int32_t stz, float dlx,
                                         float dly, float dlz, float sx, float sy, float sz,
                                         DDAResult& r, Tally<STATS>& tl) {
    uint32_t steps = 0, slot = kEmptyBit;
    int32_t last = 0;
    bool tie = false, hit = false;
    long long prev = -1;
    while (steps < g.max_steps && grid_inside(g, vx, vy, vz)) {
        const long long brick =
            (long long)(vx >> 3) + (long long)g.bx * ((vy >> 3) + (long long)g.by * (vz >> 3));
        slot = __ldg(g.dir + brick);
        if (brick != prev) {
            tl.brick();
            tl.mark((uint32_t)brick, 0);
            if (!brick_empty(slot)) {
                tl.nonempty();
                tl.mark((uint32_t)brick, 1);
            }
        }
        prev = brick;
        if (!brick_empty(slot)) {
            tl.tested();
            const uint64_t w = __ldg(g.masks + (size_t)slot * 8 + (vz & 7));
            if ((w >> (((vy & 7) << 3) | (vx & 7))) & 1ull) {
                hit = true;
                break;
            }
        }
        const float mnx = glsl_min(sy, sz), mny = glsl_min(sz, sx), mnz = glsl_min(sx, sy);
        const bool mx = sx <= mnx, my = sy <= mny, mz = sz <= mnz;
        if (mx) sx = __fadd_rn(sx, dlx);
        if (my) sy = __fadd_rn(sy, dly);
        if (mz) sz = __fadd_rn(sz, dlz);
        if (mx) vx += stx;
        if (my) vy += sty;
        if (mz) vz += stz;
        last = (mx ? 1 : 0) | (my ? 2 : 0) | (mz ? 4 : 0);
        if ((int)mx + (int)my + (int)mz > 1) tie = true;
        ++steps;
    }
    tl.steps(steps);
    r.vx = vx;
    r.vy = vy;
    r.vz = vz;
    r.steps = steps;
    r.slot = slot;
    r.last = last;
    r.hit = hit;
    r.tie = tie;
}

// One iteration of trace.frag:83-86 on the loop state of dda() / dda_skip(); fminf equals GLSL
// min here because the fast paths only run when no side distance is NaN, and then
// `side_a <= min(other two)` is `side_a == min(all three)` (one min fewer per step).
#define VT_DDA_STEP                                                          \
    {                                                                        \
        const float mn = fminf(fminf(sx, sy), sz);                          \
        mx = sx == mn;                                                       \
        my = sy == mn;                                                       \
        mz = sz == mn;                                                       \
        if (mx) sx = __fadd_rn(sx, dlx);                                     \
        if (my) sy = __fadd_rn(sy, dly);                                     \
        if (mz) sz = __fadd_rn(sz, dlz);                                     \
        if (mx) vx += stx;                                                   \
        if (my) vy += sty;                                                   \
        if (mz) vz += stz;                                                   \
        ++steps;                                                             \
    }

// VT_DDA_STEP on brick-local voxel coordinates (lx, ly, lz).
#define VT_DDA_STEP_LOCAL                                                    \
    {                                                                        \
        const float mn = fminf(fminf(sx, sy), sz);                          \
        mx = sx == mn;                                                       \
        my = sy == mn;                                                       \
        mz = sz == mn;                                                       \
        if (mx) sx = __fadd_rn(sx, dlx);                                     \
        if (my) sy = __fadd_rn(sy, dly);                                     \
        if (mz) sz = __fadd_rn(sz, dlz);                                     \
        if (mx) lx += stx;                                                   \
        if (my) ly += sty;                                                   \
        if (mz) lz += stz;                                                   \
    }

// The reference DDA (trace.frag:68-87) from grid-space point (px,py,pz) along (dx,dy,dz).
//
// Same voxel sequence, step count and hit as the literal loop; the work is organised by brick:
// one directory load per brick visited, no memory access at all while crossing an empty brick,
// and one 64-bit mask-word load (L1-resident) per voxel inside an occupied brick.  When no side
// distance is NaN every iteration advances at least one axis, so each axis leaves its brick
// within 8 steps; the trace.frag:74 step bound is still checked on every iteration.
template <bool STATS>
__device__ __forceinline__ void dda(const GridView& g, float px, float py, float pz, float dx,
                                    float dy, float dz, DDAResult& r, Tally<STATS>& tl) {
    const float len = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    int32_t vx, vy, vz, stx, sty, stz;
    float dlx, dly, dlz, sx, sy, sz;
    dda_setup_axis(px, dx, g.nx, len, vx, stx, dlx, sx);
    dda_setup_axis(py, dy, g.ny, len, vy, sty, dly, sy);
    dda_setup_axis(pz, dz, g.nz, len, vz, stz, dlz, sz);
    if (isnan(sx) || isnan(sy) || isnan(sz)) {
        dda_literal<STATS>(g, vx, vy, vz, stx, sty, stz, dlx, dly, dlz, sx, sy, sz, r, tl);
        return;
    }
    const int32_t vx0 = vx, vy0 = vy, vz0 = vz;
    const uint32_t max_steps = g.max_steps;
    uint32_t steps = 0, slot = kEmptyBit;
    bool mx = false, my = false, mz = false, hit = false;


    if (grid_inside(g, vx, vy, vz)) {
        for (;;) {
            const int32_t bxi = vx >> 3, byi = vy >> 3, bzi = vz >> 3;
            const uint32_t bidx = (uint32_t)bxi + (uint32_t)g.bx * ((uint32_t)byi + (uint32_t)g.by * (uint32_t)bzi);
            slot = __ldg(g.dir + bidx);
            tl.mark(bidx, 0);
            if (!brick_empty(slot)) tl.mark(bidx, 1);
            // first coordinate outside this brick (or the grid) along each stepping direction
            const int32_t ex = stx > 0 ? min((bxi << 3) + 8, g.nx) : (stx < 0 ? (bxi << 3) - 1 : INT_MIN);
            const int32_t ey = sty > 0 ? min((byi << 3) + 8, g.ny) : (sty < 0 ? (byi << 3) - 1 : INT_MIN);
            const int32_t ez = stz > 0 ? min((bzi << 3) + 8, g.nz) : (stz < 0 ? (bzi << 3) - 1 : INT_MIN);
            tl.brick();
            if (brick_empty(slot)) {
                do VT_DDA_STEP while (vx != ex && vy != ey && vz != ez && steps < max_steps);
            } else {
                tl.nonempty();
                const uint64_t* mk = g.masks + (size_t)slot * 8;
                for (;;) {
                    tl.tested();
                    const uint64_t w = __ldg(mk + (vz & 7));
                    if ((w >> (((vy & 7) << 3) | (vx & 7))) & 1ull) {
                        hit = true;
                        break;
                    }
                    VT_DDA_STEP
                    if (vx == ex || vy == ey || vz == ez || steps >= max_steps) break;
                }
                if (hit) break;
            }
            if (steps >= max_steps || !grid_inside(g, vx, vy, vz)) break;
        }
    }
    tl.steps(steps);
    r.vx = vx;
    r.vy = vy;
    r.vz = vz;
    r.steps = steps;
    r.slot = slot;
    r.last = (mx ? 1 : 0) | (my ? 2 : 0) | (mz ? 4 : 0);
    r.hit = hit;
    // every iteration advanced at least one axis by one voxel, monotonically: some iteration
    // advanced two or more iff the voxel moves outnumber the iterations
    r.tie = (uint32_t)(abs(vx - vx0) + abs(vy - vy0) + abs(vz - vz0)) != steps;
}

// Exact value of k successive binary32 additions of d to s (the reference's side += delta
// recurrence for one axis, trace.frag:84).  Every addition is the same operation on the running
// value, so only their count matters: the low three bits of k as predicated groups of 1, 2 and 4,
// then groups of 8 (the warp runs the loop as often as its longest chain needs; 8% faster frames
// than one loop in groups of 4 with a remainder loop).  k >= 0.
__device__ __forceinline__ float add_chain(float s, float d, int32_t k) {
    if (k & 1) s = __fadd_rn(s, d);
    if (k & 2) {
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
    }
    if (k & 4) {
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
    }
#pragma unroll 1
    for (k >>= 3; k > 0; --k) {
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
        s = __fadd_rn(s, d);
    }
    return s;
}

// Number of an axis's events S(k) <= t_star among k < n_exit, with S(k) evaluated exactly; the
// axis is known not to reach its exit (S(n_exit - 1) > t_star).  Starts from the estimate
// floor((t_star - s) / delta) and settles it with exact additions and comparisons.
__device__ __forceinline__ void advance_axis(float& s, int32_t& v, float delta, int32_t st,
                                             int32_t n_exit, float t_star, bool& stepped_last) {
    if (s > t_star) {  // also every axis with no step: its side distance is +inf
        stepped_last = false;
        return;
    }
    // t_star - s >= 0, and S(n_exit - 1) > t_star >= S(0) gives n_exit >= 2: k >= 0 for add_chain
    int32_t k = min((int32_t)__fdividef(__fsub_rn(t_star, s), delta), n_exit - 2);
    float x = add_chain(s, delta, k);  // S(k)
    if (x > t_star) {                  // the estimate overshot: walk up from S(0)
        k = 0;
        x = s;
    }
    float y = __fadd_rn(x, delta);  // S(k + 1)
    while (y <= t_star && k + 1 < n_exit) {
        x = y;
        y = __fadd_rn(y, delta);
        ++k;
    }
    s = y;
    v += st * (k + 1);
    stepped_last = x == t_star;
}

// Number of additions for an axis that cannot leave the box first: the estimate
// floor((amin - s) / delta) of its events after S(0) up to `amin` (the smallest approximate exit),
// at most n_exit - 2; 0 when its first event is already past it (also the axes with no step, whose
// side distance is +inf).  Only a speed hint: finish_axis checks the prefix exactly.  A margin of
// one addition below the estimate (so that the prefix never passes T*) measured 2% slower frames
// than settling the rare overshoot from S(0).
__device__ __forceinline__ int32_t prefix_count(float s, float delta, int32_t n_exit, float amin) {
    if (s > amin) return 0;
    return max(min((int32_t)__fdividef(__fsub_rn(amin, s), delta), n_exit - 2), 0);
}

// State of one axis after the crossing, from h = S(k) (its one chain): an axis whose chain ends at
// or before t_star walks up exactly to its last event at or before t_star; a candidate that leaves
// first (h = S(N - 1) = t_star, k = N - 1) stops at once and steps out of the box.  A chain past
// t_star with k = 0 means no event in the crossing (also the axes with no step); with k > 0 it is
// a candidate that does not leave first, or a prefix past t_star (an event of this axis between
// T* and amin, or the estimate's rounding), settled from S(0) by advance_axis.  One path for the
// leaving and the staying axes, so lanes of a warp that leave along different axes do not diverge
// here (3% faster frames than a separate exit step for the candidates).
__device__ __forceinline__ void finish_axis(float& s, int32_t& v, float h, int32_t k, float delta,
                                            int32_t st, int32_t n_exit, float t_star,
                                            bool& stepped_last) {
    if (h <= t_star) {
        float x = h, y = __fadd_rn(h, delta);
        while (y <= t_star && k + 1 < n_exit) {
            x = y;
            y = __fadd_rn(y, delta);
            ++k;
        }
        s = y;
        v += st * (k + 1);
        stepped_last = x == t_star;
    } else if (k == 0) {
        stepped_last = false;
    } else {
        advance_axis(s, v, delta, st, n_exit, t_star, stepped_last);
    }
}

// Crossing of an empty box of voxels by the reference DDA, computed per axis.
//
// In trace.frag's loop each axis a advances on the iterations where its side distance is the
// minimum; its values form the sequence S_a(0) = side_a, S_a(k+1) = S_a(k) + delta_a (binary32).
// Ties merge into one iteration, so after any iteration whose minimum is T every axis b has
// taken n_b = #{k : S_b(k) <= T} steps.  The box is left on the iteration where some axis takes
// its N_a-th step (N_a = moves to the box face), i.e. at T* = min_a S_a(N_a - 1).  Nothing in
// the box is occupied, so that iteration is reached without a hit, and the state after it is:
// side_b = S_b(n_b), voxel_b += step_b * n_b, and the axes that stepped on it are those whose
// last processed value equals T*.
//
// Only the axes that can leave first need their exit value S_a(N_a - 1) exactly: the
// approximation s + (N-1) * delta (one fused multiply-add) is within (N + 2) * 2^-24 of the exact
// chain relative to its magnitude, so any axis whose approximation exceeds the smallest by more
// than the sum of both bounds (taken 4x larger here) cannot be the minimum.  Each axis runs one
// chain of additions, so a warp whose lanes leave their boxes along different axes runs three
// chains rather than one per axis and role (4% faster frames than exit chains followed by
// separate advances): the candidates to their exit value, the others to the prefix of their
// estimated count, from which finish_axis walks up once T* is known.  Every value compared
// is computed with real binary32 additions, so the result is bit-identical to iterating the
// reference loop.
__device__ __forceinline__ void cross_region(float& sx, float& sy, float& sz, int32_t& vx,
                                             int32_t& vy, int32_t& vz, float dlx, float dly,
                                             float dlz, int32_t stx, int32_t sty, int32_t stz,
                                             int32_t nxe, int32_t nye, int32_t nze, bool& mx,
                                             bool& my, bool& mz) {
    // An axis with no step (N = 0, side and delta +inf) gives NaN here, which fminf and the
    // candidate comparison below pass over.
    const float ax = __fmaf_rn(__int2float_rn(nxe - 1), dlx, sx);
    const float ay = __fmaf_rn(__int2float_rn(nye - 1), dly, sy);
    const float az = __fmaf_rn(__int2float_rn(nze - 1), dlz, sz);
    // Candidates: an axis within 2 * amin of the smallest approximation carries at most
    // (Nmax + 2) * 2 * amin * 2^-24 of error, so (Nmax + 2) * amin * 2^-20 bounds the errors of
    // both sides of its comparison with the smallest (with the 4x margin above); axes beyond it
    // cannot leave first.
    const float amin = fminf(fminf(ax, ay), az);
    const int32_t nmax = max(max(nxe, nye), nze);
    const float lim = __fmaf_rn(__int2float_rn(nmax + 2) * 0x1p-20f, amin, amin);
    const bool cx = ax <= lim;
    const bool cy = ay <= lim;
    const bool cz = az <= lim;
    const int32_t kx = cx ? nxe - 1 : prefix_count(sx, dlx, nxe, amin);
    const int32_t ky = cy ? nye - 1 : prefix_count(sy, dly, nye, amin);
    const int32_t kz = cz ? nze - 1 : prefix_count(sz, dlz, nze, amin);
    VT_PHASE_MARK(__activemask(), VT_PHASE_CROSS_BOX);
    const float hx = add_chain(sx, dlx, kx);
    const float hy = add_chain(sy, dly, ky);
    const float hz = add_chain(sz, dlz, kz);
    const float ts = fminf(fminf(cx ? hx : INFINITY, cy ? hy : INFINITY), cz ? hz : INFINITY);
    VT_PHASE_MARK(__activemask(), VT_PHASE_CROSS_CHAINS);
    finish_axis(sx, vx, hx, kx, dlx, stx, nxe, ts, mx);
    finish_axis(sy, vy, hy, ky, dly, sty, nye, ts, my);
    finish_axis(sz, vz, hz, kz, dlz, stz, nze, ts, mz);
}

// Moves along one axis from voxel v (in brick bi) to the far face of a box reaching r bricks
// forward (this brick included) in step direction st, clipped to the grid's n voxels: the face is
// the first voxel past the box for st = +1 (at most n) and the first voxel before it for st = -1
// (at least -1).  0 for st = 0 (unused).
__device__ __forceinline__ int32_t axis_moves(int32_t bi, int32_t r, int32_t v, int32_t st,
                                              int32_t n) {
    const int32_t neg = st < 0 ? 1 : 0;
    const int32_t f = min(max(((bi + st * r + neg) << 3) - neg, -1), n);
    return (f - v) * st;
}

// Voxel moves to the far face, along each stepping axis, of the empty box the ray crosses next
// from the empty brick (bxi, byi, bzi).  Three boxes are known empty: the cube of bricks within
// Chebyshev distance D - 1 (D from the directory entry `e`), which reaches D bricks forward along
// every stepping direction; the box of K bricks from this brick toward the ray's octant (K from
// the octant word `ow`); and, when K >= D, the box that is K bricks across and L >= K bricks
// long along the ray's dominant axis `dom` (L from the long-box word `lw`).  The ray only moves
// forward, so the crossing uses the forward reach of the chosen box per axis, clipped to the
// grid.  Axes with no step get 0 (unused by cross_region).
__device__ __forceinline__ void empty_moves(const GridView& g, uint32_t e, uint32_t ow,
                                            uint32_t lw, int32_t bxi, int32_t byi, int32_t bzi,
                                            int32_t vx, int32_t vy, int32_t vz, int32_t stx,
                                            int32_t sty, int32_t stz, uint32_t oct_shift,
                                            int32_t dom, int32_t& nxe, int32_t& nye,
                                            int32_t& nze) {
    const int32_t D = max((int32_t)(e & 0xFFu), 1);
    const int32_t K = (int32_t)((ow >> oct_shift) & 15u);
    const int32_t L = max(K, (int32_t)((lw >> oct_shift) & 15u));
    // the box across (rk) and along the dominant axis (rl) by selects: lanes choosing the cube and
    // lanes choosing the long box run the same instructions (1% faster frames than a branch)
    const bool box = K >= D;
    const int32_t rk = box ? K : D, rl = box ? L : D;
    const int32_t rx = dom == 0 ? rl : rk;
    const int32_t ry = dom == 1 ? rl : rk;
    const int32_t rz = dom == 2 ? rl : rk;
    nxe = axis_moves(bxi, rx, vx, stx, g.nx);
    nye = axis_moves(byi, ry, vy, sty, g.ny);
    nze = axis_moves(bzi, rz, vz, stz, g.nz);
}

// Dominant axis of a direction (largest |component|; ties to the lower axis).
__device__ __forceinline__ int32_t dominant_axis(float dx, float dy, float dz) {
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    return ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
}

// The long-box words of the ray's dominant axis, or nullptr.
__device__ __forceinline__ const uint32_t* long_words(const GridView& g, int32_t dom) {
    return g.lng ? g.lng + (size_t)dom * g.bricks : nullptr;
}

// The octant word of brick `bidx`; 0 (no forward boxes) for a grid built without octant words.
// Loaded together with the directory entry, before the entry is tested, so that both loads are in
// flight at once.
__device__ __forceinline__ uint32_t octant_word(const GridView& g, uint32_t bidx) {
    return g.oct ? __ldg(g.oct + bidx) : 0u;
}

__device__ __forceinline__ uint32_t octant_shift(int32_t stx, int32_t sty, int32_t stz) {
    return 4u * ((stx < 0 ? 1u : 0u) | (sty < 0 ? 2u : 0u) | (stz < 0 ? 4u : 0u));
}

// Same result as dda() (hit, voxel, slot, final mask), organised for speed: occupied bricks are
// walked voxel by voxel against their occupancy bits; from an empty brick the ray crosses the
// empty box of empty_moves() in one cross_region().  The step count and tie flag of the literal
// loop are not tracked here (the counting kernels use dda()).
__device__ __forceinline__ void dda_skip(const GridView& g, float px, float py, float pz,
                                         float dx, float dy, float dz, DDAResult& r) {
    const float len = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    int32_t vx, vy, vz, stx, sty, stz;
    float dlx, dly, dlz, sx, sy, sz;
    dda_setup_axis(px, dx, g.nx, len, vx, stx, dlx, sx);
    dda_setup_axis(py, dy, g.ny, len, vy, sty, dly, sy);
    dda_setup_axis(pz, dz, g.nz, len, vz, stz, dlz, sz);
    if (isnan(sx) || isnan(sy) || isnan(sz)) {
        Tally<false> tl;
        dda_literal<false>(g, vx, vy, vz, stx, sty, stz, dlx, dly, dlz, sx, sy, sz, r, tl);
        return;
    }
    const uint32_t max_steps = g.max_steps;
    const uint32_t oshift = octant_shift(stx, sty, stz);
    const int32_t dom = dominant_axis(dx, dy, dz);
    const uint32_t* lp = long_words(g, dom);
    uint32_t steps = 0, slot = kEmptyBit;  // steps: counted by VT_DDA_STEP, not used here
    bool mx = false, my = false, mz = false, hit = false;
    // guard: passes that run a unit; each advances at least one axis, monotonically, inside the
    // grid.  pend_w / pend_c: lanes needing a walk / a crossing were passed over last pass.
    int32_t guard = g.nx + g.ny + g.nz + 2;
    bool pend_w = false, pend_c = false;
    while (grid_inside(g, vx, vy, vz) && guard > 0) {
        const int32_t bxi = vx >> 3, byi = vy >> 3, bzi = vz >> 3;
        // fewer than 2^31 bricks (vt_grid_create checks): the index fits 32 bits
        const uint32_t bidx = (uint32_t)bxi + (uint32_t)g.bx * ((uint32_t)byi + (uint32_t)g.by * (uint32_t)bzi);
        const uint32_t e = __ldg(g.dir + bidx);
        {
            // One kind of unit per pass among the lanes running this loop together: the kind
            // more of them need (walk or crossing) runs while the others wait, and a kind passed
            // over runs next, so a warp issues one kind's instructions per pass instead of both
            // (5% faster frames).  Every pass runs a unit on at least one of these lanes, so the
            // waits end.
            const bool walk = !brick_empty(e);
            const uint32_t act = __activemask();
            VT_PHASE_MARK(act, VT_PHASE_LOOP);
            const uint32_t wb = __ballot_sync(act, walk), cb = act & ~wb;
            bool run_walk = __popc(wb) >= __popc(cb);
            if (run_walk ? (cb && pend_c) : (wb && pend_w)) run_walk = !run_walk;
            pend_w = !run_walk && wb;
            pend_c = run_walk && cb;
            VT_PHASE_PASS(act, run_walk);
            if (walk != run_walk) continue;
        }
        --guard;
        if (!brick_empty(e)) {
            slot = e;
            const uint64_t* mk = g.masks + (size_t)slot * 8;
            // Brick-local coordinates; the walk ends when one leaves 0..7.  Where a grid face cuts
            // the brick, the voxels past the face have no occupancy bits, so walking on to the
            // brick's face only defers the loop's grid-exit test: the ray misses either way, and a
            // miss keeps none of the walk's state.  Ends: with no side distance NaN, every
            // iteration steps an axis whose step is not 0 (an axis with step 0 has side +inf, the
            // minimum only when all three are), so the brick is left within 22 iterations.
            int32_t lx = vx & 7, ly = vy & 7, lz = vz & 7;
            for (;;) {
                const uint64_t w = __ldg(mk + lz);
                if ((w >> ((ly << 3) | lx)) & 1ull) {
                    hit = true;
                    break;
                }
                VT_DDA_STEP_LOCAL
                if ((lx | ly | lz) & ~7) break;
            }
            vx = (bxi << 3) + lx;
            vy = (byi << 3) + ly;
            vz = (bzi << 3) + lz;
            VT_PHASE_MARK(__activemask(), VT_PHASE_WALK);
            if (hit) break;
        } else {
            const uint32_t ow = octant_word(g, bidx);
            const uint32_t lw = lp ? __ldg(lp + bidx) : 0u;
            int32_t nxe, nye, nze;
            empty_moves(g, e, ow, lw, bxi, byi, bzi, vx, vy, vz, stx, sty, stz, oshift, dom, nxe,
                        nye, nze);
            cross_region(sx, sy, sz, vx, vy, vz, dlx, dly, dlz, stx, sty, stz, nxe, nye, nze, mx,
                         my, mz);
            VT_PHASE_MARK(__activemask(), VT_PHASE_CROSS_FINISH);
        }
    }
    (void)max_steps;
    r.vx = vx;
    r.vy = vy;
    r.vz = vz;
    r.steps = steps;
    r.slot = slot;
    r.last = (mx ? 1 : 0) | (my ? 2 : 0) | (mz ? 4 : 0);
    r.hit = hit;
    r.tie = false;
}

// Ray/box entry against [0,nx]x[0,ny]x[0,nz]: 0 = miss, 1 = enters from outside, 2 = origin
// inside.  Same operation order as the oracle's slab test.
__device__ __forceinline__ int slab_entry(const GridView& g, const float o[3], const float d[3],
                                          float pos[3], float& t_entry, int& axis) {
    const float size[3] = {__int2float_rn(g.nx), __int2float_rn(g.ny), __int2float_rn(g.nz)};
    // an origin strictly inside the box has tn < 0 < tf on every axis: the slab test below would
    // return "inside" with the origin as the entry point, so skip its six divisions
    if (o[0] > 0.0f && o[0] < size[0] && o[1] > 0.0f && o[1] < size[1] && o[2] > 0.0f &&
        o[2] < size[2]) {
        pos[0] = o[0];
        pos[1] = o[1];
        pos[2] = o[2];
        t_entry = 0.0f;
        axis = -1;
        return 2;
    }
    float tn = -INFINITY, tf = INFINITY;
    int ax = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
            if (o[a] < 0.0f || o[a] > size[a]) return 0;
            continue;
        }
        const float ta = __fdiv_rn(__fsub_rn(0.0f, o[a]), d[a]);
        const float tb = __fdiv_rn(__fsub_rn(size[a], o[a]), d[a]);
        const float lo = ta < tb ? ta : tb;
        const float hi = ta < tb ? tb : ta;
        if (lo > tn) {
            tn = lo;
            ax = a;
        }
        if (hi < tf) tf = hi;
    }
    if (tn > tf || tf < 0.0f) return 0;
    if (tn <= 0.0f) {
        pos[0] = o[0];
        pos[1] = o[1];
        pos[2] = o[2];
        t_entry = 0.0f;
        axis = -1;
        return 2;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        float p = __fadd_rn(o[b], __fmul_rn(tn, d[b]));
        p = p < 0.0f ? 0.0f : p;
        p = p > size[b] ? size[b] : p;
        pos[b] = p;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b)
        if (b == ax) pos[b] = d[b] > 0.0f ? 0.0f : size[b];
    t_entry = tn;
    axis = ax;
    return 1;
}

__device__ __forceinline__ uint32_t face_code(int axis, bool normal_positive) {
    return (uint32_t)(1 + 2 * axis + (normal_positive ? 0 : 1));
}

// Packed vt_hit: {x | y<<16, z | index<<16 | face<<24, t bits, rgba}.
struct HitRec {
    uint32_t w0, w1, w2, w3;
};

__device__ __forceinline__ HitRec miss_rec(uint32_t flags, uint32_t rgba) {
    HitRec h;
    h.w0 = 0xFFFFFFFFu;
    h.w1 = 0xFFFFu | (flags << 24);
    h.w2 = __float_as_uint(INFINITY);
    h.w3 = rgba;
    return h;
}

__device__ __forceinline__ bool finite3(const float a[3]) {
    return isfinite(a[0]) && isfinite(a[1]) && isfinite(a[2]);
}

__device__ __forceinline__ uint32_t voxel_value(const GridView& g, uint32_t slot, int32_t x,
                                                int32_t y, int32_t z, uint32_t& index) {
    const uint32_t li = (uint32_t)(x & 7) | ((uint32_t)(y & 7) << 3) | ((uint32_t)(z & 7) << 6);
    if (g.format == VT_PAYLOAD_U8) {
        index = __ldg(g.payload8 + (size_t)slot * 512 + li);
        return __ldg(g.palette + index);
    }
    index = 0;
    return __ldg(g.payload32 + (size_t)slot * 512 + li);
}

// Hit record of a finished ray: face of the final iteration's step (the entry face when the ray
// hit its first voxel after entering from outside, none when it started inside the hit voxel),
// t of that face plane, and the voxel's unshaded colour.  Mirrors vto_trace_ray_f32.
__device__ __forceinline__ HitRec hit_record(const GridView& g, const float o[3], const float d[3],
                                             int32_t vx, int32_t vy, int32_t vz, int32_t last,
                                             uint32_t slot, int entry_axis, float t_entry) {
    uint32_t face = 0;
    float t = 0.0f;
    if (last != 0) {  // the ray moved: the face of the final iteration's step
        const int a = (last & 1) ? 0 : ((last & 2) ? 1 : 2);
        const int32_t va = a == 0 ? vx : (a == 1 ? vy : vz);
        const float da = a == 0 ? d[0] : (a == 1 ? d[1] : d[2]);
        const float oa = a == 0 ? o[0] : (a == 1 ? o[1] : o[2]);
        const float plane = __int2float_rn(da > 0.0f ? va : va + 1);
        t = __fdiv_rn(__fsub_rn(plane, oa), da);
        face = face_code(a, da < 0.0f);
    } else if (entry_axis >= 0) {
        const int a = entry_axis;
        const float da = a == 0 ? d[0] : (a == 1 ? d[1] : d[2]);
        t = t_entry;
        face = face_code(a, da < 0.0f);
    }
    uint32_t index;
    const uint32_t rgba = voxel_value(g, slot, vx, vy, vz, index);
    HitRec h;
    h.w0 = (uint32_t)vx | ((uint32_t)vy << 16);
    h.w1 = (uint32_t)vz | (index << 16) | ((face | VT_HIT_FLAG_HIT) << 24);
    h.w2 = __float_as_uint(t);
    h.w3 = rgba;
    return h;
}

// One ray: validity, slab entry, DDA, record.  Mirrors vto_trace_ray_f32.  The counting build
// walks every iteration (dda); the plain build crosses empty space per axis (dda_skip).
template <bool STATS>
__device__ __forceinline__ HitRec trace_ray(const GridView& g, const float o[3], const float d[3],
                                            Tally<STATS>& tl) {
    tl.rays();
    if (!finite3(o) || !finite3(d)) return miss_rec(VT_HIT_FLAG_INVALID, 0u);
    float pos[3], t_entry;
    int entry_axis;
    const int kind = slab_entry(g, o, d, pos, t_entry, entry_axis);
    if (kind == 0) return miss_rec(0u, 0u);
    DDAResult r;
    if (STATS)
        dda<STATS>(g, pos[0], pos[1], pos[2], d[0], d[1], d[2], r, tl);
    else
        dda_skip(g, pos[0], pos[1], pos[2], d[0], d[1], d[2], r);
    if (r.tie) tl.tie();
    if (!r.hit) return miss_rec(0u, 0u);
    tl.mark((uint32_t)(r.vx >> 3) + (uint32_t)g.bx * ((uint32_t)(r.vy >> 3) + (uint32_t)g.by * (uint32_t)(r.vz >> 3)), 2);
    return hit_record(g, o, d, r.vx, r.vy, r.vz, r.last, r.slot, kind == 1 ? entry_axis : -1,
                      t_entry);
}

// Primary ray for pixel (px, py) + sub-pixel offset (jx, jy).  Mirrors vto_raygen.
__device__ __forceinline__ void raygen(const vt_camera& c, uint32_t px, uint32_t py, float jx,
                                       float jy, float o[3], float d[3]) {
    const float inv_w2 = __fdiv_rn(2.0f, __uint2float_rn(c.width));
    const float inv_h2 = __fdiv_rn(2.0f, __uint2float_rn(c.height));
    const float fx = __fadd_rn(__uint2float_rn(px), jx);
    const float fy = __fadd_rn(__uint2float_rn(py), jy);
    const float sx = __fsub_rn(__fmul_rn(fx, inv_w2), 1.0f);
    const float sy = __fsub_rn(1.0f, __fmul_rn(fy, inv_h2));
    float r[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        r[a] = __fadd_rn(__fadd_rn(c.forward[a], __fmul_rn(sx, c.right[a])), __fmul_rn(sy, c.up[a]));
    const float len = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(r[0], r[0]), __fmul_rn(r[1], r[1])), __fmul_rn(r[2], r[2])));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        d[a] = __fdiv_rn(r[a], len);
        o[a] = c.origin[a];
    }
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), the published counter-based generator.
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

__device__ __forceinline__ void jitter(uint32_t seed, uint32_t view, uint32_t px, uint32_t py,
                                       uint32_t s, float& jx, float& jy) {
    uint32_t r[4];
    philox4x32_10(px, py, s, view, seed, 0x56544752u, r);
    jx = __fmul_rn(__uint2float_rn(r[0] >> 8), 0x1p-24f);
    jy = __fmul_rn(__uint2float_rn(r[1] >> 8), 0x1p-24f);
}

// Lambert term of a hit record's face for light L: false when there is no face (the origin lies
// in the hit voxel); otherwise `ndl` = n.L of the face normal.
__device__ __forceinline__ bool face_lit(const HitRec& h, const LightView& L, float& ndl) {
    const uint32_t face = (h.w1 >> 24) & VT_FACE_MASK;
    if (face == 0) return false;
    const int a = (int)(face - 1) / 2;
    const float la = a == 0 ? L.dx : (a == 1 ? L.dy : L.dz);
    ndl = (face & 1u) ? la : -la;
    return true;
}

// Origin of the shadow ray of a hit: the hit point on the entered face, moved 1/64 voxel off the
// face into the voxel the ray came from.  Mirrors the oracle's shade_from_ray.
__device__ __forceinline__ void shadow_origin(const HitRec& h, const float o[3], const float d[3],
                                              float so[3]) {
    const uint32_t face = (h.w1 >> 24) & VT_FACE_MASK;
    const int a = (int)(face - 1) / 2;
    const bool npos = (face & 1u) != 0u;
    const int32_t hv[3] = {(int32_t)(h.w0 & 0xFFFFu), (int32_t)(h.w0 >> 16),
                           (int32_t)(h.w1 & 0xFFFFu)};
    const float t = __uint_as_float(h.w2);
#pragma unroll
    for (int b = 0; b < 3; ++b) so[b] = __fadd_rn(o[b], __fmul_rn(t, d[b]));
    const int32_t ha = a == 0 ? hv[0] : (a == 1 ? hv[1] : hv[2]);
    const float plane = __int2float_rn(npos ? ha + 1 : ha);
    const float sa = npos ? __fadd_rn(plane, 0.015625f) : __fsub_rn(plane, 0.015625f);
#pragma unroll
    for (int b = 0; b < 3; ++b)
        if (b == a) so[b] = sa;
}

// k = ambient + (1 - ambient) * max(n.L, 0) * visible; colour = floor(base * k + 0.5).
__device__ __forceinline__ uint32_t shade_rgba(uint32_t base, float ndl, float vis, float ambient) {
    const float lam = ndl > 0.0f ? ndl : 0.0f;
    const float k = __fadd_rn(ambient, __fmul_rn(__fsub_rn(1.0f, ambient), __fmul_rn(lam, vis)));
    uint32_t res = base & 0xFF000000u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float v = __fadd_rn(__fmul_rn(__uint2float_rn((base >> (8 * c)) & 0xFFu), k), 0.5f);
        const uint32_t q = v >= 255.0f ? 255u : (v <= 0.0f ? 0u : (uint32_t)v);
        res |= q << (8 * c);
    }
    return res;
}

// Primary hit + Lambert shading + optional hard shadow.  Mirrors the oracle's shade_from_ray.
template <bool STATS>
__device__ __forceinline__ HitRec shade_ray(const GridView& g, const LightView& L,
                                            const float o[3], const float d[3],
                                            Tally<STATS>& tl) {
    HitRec h = trace_ray<STATS>(g, o, d, tl);
    const uint32_t flags = h.w1 >> 24;
    if (!(flags & VT_HIT_FLAG_HIT)) {
        h.w3 = VT_SKY_RGBA;
        return h;
    }
    tl.hit();
    float ndl;
    if (!L.enabled || !face_lit(h, L, ndl)) return h;
    float vis = 1.0f;
    uint32_t extra = 0;
    if (ndl > 0.0f && L.shadows) {
        float so[3];
        shadow_origin(h, o, d, so);
        const float ld[3] = {L.dx, L.dy, L.dz};
        const HitRec s = trace_ray<STATS>(g, so, ld, tl);
        tl.shadow();
        extra |= VT_HIT_FLAG_SHADOW_RAY;
        if ((s.w1 >> 24) & VT_HIT_FLAG_HIT) {
            vis = 0.0f;
            extra |= VT_HIT_FLAG_SHADOWED;
        }
    }
    h.w3 = shade_rgba(h.w3, ndl, vis, L.ambient);
    h.w1 |= extra << 24;
    return h;
}

// One pixel of vt_render (the body of render_kernel): camera ray, shading and shadow ray, with the
// warp (lanes `vmask`) re-converged between the camera rays and the shadow rays.  Same record as
// shade_ray.
template <bool STATS>
__device__ __forceinline__ HitRec render_pixel(const GridView& g, const vt_camera& cam,
                                               const LightView& light, uint32_t px, uint32_t py,
                                               uint32_t vmask, Tally<STATS>& tl) {
    float o[3], d[3];
    raygen(cam, px, py, 0.5f, 0.5f, o, d);
    HitRec h = trace_ray<STATS>(g, o, d, tl);
    // The warp's shadow rays start together: lanes reaching theirs at different times would run
    // them as separate groups (a third of the lanes per traversal pass).
    __syncwarp(vmask);
    VT_PHASE_MARK(vmask, VT_PHASE_TAIL);
    VT_PHASE_KIND(vmask, 1);
    const uint32_t flags = h.w1 >> 24;
    float ndl = 0.0f;
    if (!(flags & VT_HIT_FLAG_HIT)) {
        h.w3 = VT_SKY_RGBA;
    } else {
        tl.hit();
        if (light.enabled && face_lit(h, light, ndl)) {
            float vis = 1.0f;
            uint32_t extra = 0;
            if (ndl > 0.0f && light.shadows) {
                float so[3];
                shadow_origin(h, o, d, so);
                const float ld[3] = {light.dx, light.dy, light.dz};
                const HitRec s = trace_ray<STATS>(g, so, ld, tl);
                tl.shadow();
                extra |= VT_HIT_FLAG_SHADOW_RAY;
                if ((s.w1 >> 24) & VT_HIT_FLAG_HIT) {
                    vis = 0.0f;
                    extra |= VT_HIT_FLAG_SHADOWED;
                }
            }
            h.w3 = shade_rgba(h.w3, ndl, vis, light.ambient);
            h.w1 |= extra << 24;
        }
    }
    return h;
}

}  // namespace vt

