// vt_update.cu — writing a box of voxels into a resident brick grid (chunk paging).
//
// vtrace streams its world in 16^3 chunks around the camera (src/gen/pager.rs:52-78), uploading
// one new texture per frame (src/render.rs:246-261).  Here a chunk (any box, any alignment) is
// written into an existing grid instead, in place:
//
//   1. the box is uploaded (and reordered if it is z-fastest);
//   2. one thread per (affected brick, z-slice) merges the box's voxels with the brick's current
//      payload into a new occupancy word and payload slice (scratch), and flags the brick;
//   3. the host reads the flags and old directory entries of the affected bricks, keeps the slot
//      of bricks that stay occupied, frees the slots of bricks that became empty and hands out
//      slots (free list, then the high-water mark, growing the slot arrays by doubling) to bricks
//      that became occupied;
//   4. the new words and payloads are scattered into their slots and the directory entries
//      rewritten;
//   5. the Chebyshev distance field, the octant forward distances and the long forward boxes are
//      recomputed for the bricks within their caps (31, 15 and 15 bricks) of the affected ones:
//      a change cannot reach farther, and each pass reads the previous one only that far.
//
// The grid afterwards traverses exactly as a grid built from the updated dense array (same
// occupancy, payload, distances and octant words; only slot numbers may differ).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "vt_api_internal.h"
#include "vt_device.cuh"
#include "vt_internal.h"

namespace vt {

struct UpdateBox {
    int32_t x0, y0, z0, w, h, d;      // voxel box
    int32_t bx0, by0, bz0, kx, ky, kz;  // affected bricks
};

// One thread per (affected brick k, z-slice lz): merge and flag.  `src` is the x-fastest box.
template <typename T>
__global__ void __launch_bounds__(256) update_merge_kernel(GridView g, UpdateBox u,
                                                           const T* __restrict__ src,
                                                           uint64_t* __restrict__ words,
                                                           T* __restrict__ payload,
                                                           uint32_t* __restrict__ flags,
                                                           uint32_t* __restrict__ old_dir,
                                                           long long* __restrict__ occ_delta) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t K = (uint64_t)u.kx * u.ky * u.kz;
    if (t >= K * 8) return;
    const uint64_t k = t >> 3;
    const int32_t lz = (int32_t)(t & 7);
    const int32_t bxi = u.bx0 + (int32_t)(k % u.kx);
    const int32_t byi = u.by0 + (int32_t)((k / u.kx) % u.ky);
    const int32_t bzi = u.bz0 + (int32_t)(k / ((uint64_t)u.kx * u.ky));
    const size_t b = (size_t)bxi + (size_t)g.bx * ((size_t)byi + (size_t)g.by * bzi);
    const uint32_t e = g.dir[b];
    const bool was = !brick_empty(e);
    const int32_t z = bzi * 8 + lz;
    uint64_t word = 0;
    T* out = payload + k * 512 + lz * 64;
    for (int32_t ly = 0; ly < 8; ++ly) {
        const int32_t y = byi * 8 + ly;
        for (int32_t lx = 0; lx < 8; ++lx) {
            const int32_t x = bxi * 8 + lx;
            T v = 0;
            if (x < g.nx && y < g.ny && z < g.nz) {
                if (x >= u.x0 && x < u.x0 + u.w && y >= u.y0 && y < u.y0 + u.h && z >= u.z0 &&
                    z < u.z0 + u.d) {
                    v = src[(size_t)(x - u.x0) + (size_t)u.w * ((size_t)(y - u.y0) + (size_t)u.h * (z - u.z0))];
                } else if (was) {
                    const size_t li = (size_t)lx + 8 * (ly + 8 * lz);
                    if (sizeof(T) == 1)
                        v = (T)g.payload8[(size_t)e * 512 + li];
                    else
                        v = (T)g.payload32[(size_t)e * 512 + li];
                }
            }
            const uint32_t rgba = sizeof(T) == 1 ? g.palette[(uint32_t)v] : (uint32_t)v;
            if (rgba >> 24) word |= 1ull << (ly * 8 + lx);
            out[ly * 8 + lx] = v;
        }
    }
    words[k * 8 + lz] = word;
    const uint64_t old_word = was ? g.masks[(size_t)e * 8 + lz] : 0ull;
    const long long delta = (long long)__popcll(word) - (long long)__popcll(old_word);
    if (delta) atomicAdd((unsigned long long*)occ_delta, (unsigned long long)delta);
    // the brick's flag: OR of its 8 slices (lanes 8j..8j+7 of a warp hold one brick, and are
    // active together because the thread count is a multiple of 8)
    const unsigned active = __activemask();
    uint32_t f = word != 0ull;
#pragma unroll
    for (int s = 1; s < 8; s <<= 1) f |= __shfl_xor_sync(active, f, s);
    if (lz == 0) {
        flags[k] = f;
        old_dir[k] = e;
    }
}

// One thread per (affected brick, z-slice): scatter into the assigned slot, rewrite the entry.
template <typename T>
__global__ void __launch_bounds__(256) update_scatter_kernel(GridView g, UpdateBox u,
                                                             const uint64_t* __restrict__ words,
                                                             const T* __restrict__ payload,
                                                             const uint32_t* __restrict__ slots,
                                                             uint32_t* __restrict__ dir,
                                                             uint64_t* __restrict__ masks,
                                                             T* __restrict__ dst) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t K = (uint64_t)u.kx * u.ky * u.kz;
    if (t >= K * 8) return;
    const uint64_t k = t >> 3;
    const int32_t lz = (int32_t)(t & 7);
    const int32_t bxi = u.bx0 + (int32_t)(k % u.kx);
    const int32_t byi = u.by0 + (int32_t)((k / u.kx) % u.ky);
    const int32_t bzi = u.bz0 + (int32_t)(k / ((uint64_t)u.kx * u.ky));
    const size_t b = (size_t)bxi + (size_t)g.bx * ((size_t)byi + (size_t)g.by * bzi);
    const uint32_t slot = slots[k];
    if (lz == 0) dir[b] = slot;  // kEmptyBit | 1 for a brick left empty: distances follow
    if (brick_empty(slot)) return;
    masks[(size_t)slot * 8 + lz] = words[k * 8 + lz];
    const T* in = payload + k * 512 + lz * 64;
    T* out = dst + (size_t)slot * 512 + lz * 64;
    for (int i = 0; i < 64; ++i) out[i] = in[i];
}

// Grows the slot arrays of `g` to at least `need` slots (doubling), copying the live ones.
static int32_t grow_slots(Grid& g, uint64_t need, cudaStream_t st) {
    if (need <= g.slot_capacity) return VT_OK;
    const uint64_t cap = std::max<uint64_t>(need, g.slot_capacity * 2);
    const size_t psize = g.format == VT_PAYLOAD_U8 ? 512 : 2048;
    uint64_t* m = nullptr;
    void* p = nullptr;
    if (cudaMalloc(&m, cap * 64) != cudaSuccess || cudaMalloc(&p, cap * psize) != cudaSuccess) {
        cudaFree(m);
        cudaGetLastError();
        return fail(VT_ENOMEM, "vt_grid_update: cannot grow the brick slots");
    }
    cudaError_t e = cudaMemcpyAsync(m, g.masks, g.slot_capacity * 64, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p, g.payload, g.slot_capacity * psize, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(m);
        cudaFree(p);
        return cuda_fail(e, "vt_grid_update: slot copy");
    }
    // slot arrays of the build's single allocation stay allocated with it: only later ones go
    g.bytes += (g.in_block(g.masks) ? cap : cap - g.slot_capacity) * (64 + psize);
    g.free_slot_arrays();
    g.masks = m;
    g.payload = p;
    state().grid_epoch.fetch_add(1);  // the grid's device view changed
    g.slot_capacity = cap;
    return VT_OK;
}

}  // namespace vt

using namespace vt;

extern "C" int32_t vt_grid_update(int32_t grid, const void* voxels, uint32_t order, uint32_t x0,
                                  uint32_t y0, uint32_t z0, uint32_t w, uint32_t h, uint32_t d) {
    Grid* g = lookup_grid(grid);
    if (!g) return fail(VT_ENOTFOUND, "vt_grid_update: unknown grid");
    if (!voxels) return fail(VT_EINVAL, "vt_grid_update: null voxels");
    if (order != VT_ORDER_X_FASTEST && order != VT_ORDER_Z_FASTEST)
        return fail(VT_EINVAL, "vt_grid_update: bad order");
    if (w == 0 || h == 0 || d == 0 || (uint64_t)x0 + w > g->nx || (uint64_t)y0 + h > g->ny ||
        (uint64_t)z0 + d > g->nz)
        return fail(VT_EINVAL, "vt_grid_update: box empty or outside the grid");
    if (g->refs.load() > 0)
        return fail(VT_EBUSY, "vt_grid_update: grid is referenced by a batch or a service");
    State& s = state();
    cudaStream_t st = s.stream;
    const size_t elem = g->format == VT_PAYLOAD_U8 ? 1 : 4;
    UpdateBox u;
    u.x0 = (int32_t)x0;
    u.y0 = (int32_t)y0;
    u.z0 = (int32_t)z0;
    u.w = (int32_t)w;
    u.h = (int32_t)h;
    u.d = (int32_t)d;
    u.bx0 = u.x0 >> 3;
    u.by0 = u.y0 >> 3;
    u.bz0 = u.z0 >> 3;
    u.kx = ((u.x0 + u.w - 1) >> 3) - u.bx0 + 1;
    u.ky = ((u.y0 + u.h - 1) >> 3) - u.by0 + 1;
    u.kz = ((u.z0 + u.d - 1) >> 3) - u.bz0 + 1;
    const uint64_t K = (uint64_t)u.kx * u.ky * u.kz;
    const size_t box = (size_t)w * h * d * elem;
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    // scratch: box (x2 for reordering), words, payloads, flags, old entries, slots, delta,
    // distance and octant temporaries
    const size_t o_box = 0, o_box2 = al(box), o_words = o_box2 + (order == VT_ORDER_Z_FASTEST ? al(box) : 0);
    const size_t o_pay = o_words + al(K * 64), o_flags = o_pay + al(K * 512 * elem);
    const size_t o_old = o_flags + al(K * 4), o_slots = o_old + al(K * 4), o_delta = o_slots + al(K * 4);
    const size_t o_da = o_delta + 256, o_db = o_da + al(g->bricks), o_ty = o_db + al(g->bricks);
    const size_t o_run = o_ty + al(g->bricks * 2);
    const BrickBox changed = {u.bx0, u.by0, u.bz0, u.kx, u.ky, u.kz};
    const size_t o_occ = o_run + al(4 * brick_long_scratch_words(&changed, (int32_t)g->bx,
                                                                  (int32_t)g->by, (int32_t)g->bz));
    const size_t total = o_occ + al(4 * brick_xmask_words((int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz));
    char* scr = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&scr, total, st);
    if (e != cudaSuccess) return cuda_fail(e, "vt_grid_update: scratch");
    int32_t rc = VT_OK;
    std::vector<uint32_t> flags(K), old(K), slots(K);
    long long delta = 0;
    do {
        // 1. upload, reorder
        e = cudaMemcpyAsync(scr + o_box, voxels, box, cudaMemcpyHostToDevice, st);
        const void* src = scr + o_box;
        if (e == cudaSuccess && order == VT_ORDER_Z_FASTEST) {
            e = launch_transpose_xz(scr + o_box, scr + o_box2, elem, u.w, u.h, u.d, st);
            src = scr + o_box2;
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(scr + o_delta, 0, 8, st);
        if (e != cudaSuccess) { rc = cuda_fail(e, "vt_grid_update: upload"); break; }
        // 2. merge
        const GridView v = g->view();
        const unsigned blocks = (unsigned)((K * 8 + 255) / 256);
        if (elem == 1)
            update_merge_kernel<uint8_t><<<blocks, 256, 0, st>>>(
                v, u, (const uint8_t*)src, (uint64_t*)(scr + o_words), (uint8_t*)(scr + o_pay),
                (uint32_t*)(scr + o_flags), (uint32_t*)(scr + o_old), (long long*)(scr + o_delta));
        else
            update_merge_kernel<uint32_t><<<blocks, 256, 0, st>>>(
                v, u, (const uint32_t*)src, (uint64_t*)(scr + o_words), (uint32_t*)(scr + o_pay),
                (uint32_t*)(scr + o_flags), (uint32_t*)(scr + o_old), (long long*)(scr + o_delta));
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(flags.data(), scr + o_flags, K * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(old.data(), scr + o_old, K * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&delta, scr + o_delta, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { rc = cuda_fail(e, "vt_grid_update: merge"); break; }
        // 3. slots: free first, so that freed slots are reused by this update's new bricks
        uint64_t fresh = 0;
        for (uint64_t k = 0; k < K; ++k) {
            const bool was = !(old[k] & kEmptyBit), now = flags[k] != 0;
            if (was && !now) g->free_slots.push_back(old[k]);
            if (!was && now) ++fresh;
        }
        const uint64_t reuse = std::min<uint64_t>(fresh, g->free_slots.size());
        if ((rc = grow_slots(*g, g->slots_used + (fresh - reuse), st))) break;
        for (uint64_t k = 0; k < K; ++k) {
            const bool was = !(old[k] & kEmptyBit), now = flags[k] != 0;
            if (!now) {
                slots[k] = kEmptyBit | 1u;
            } else if (was) {
                slots[k] = old[k];
            } else if (!g->free_slots.empty()) {
                slots[k] = g->free_slots.back();
                g->free_slots.pop_back();
            } else {
                slots[k] = (uint32_t)g->slots_used++;
            }
        }
        // 4. scatter
        e = cudaMemcpyAsync(scr + o_slots, slots.data(), K * 4, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { rc = cuda_fail(e, "vt_grid_update: slots"); break; }
        const GridView v2 = g->view();
        if (elem == 1)
            update_scatter_kernel<uint8_t><<<blocks, 256, 0, st>>>(
                v2, u, (const uint64_t*)(scr + o_words), (const uint8_t*)(scr + o_pay),
                (const uint32_t*)(scr + o_slots), g->dir, g->masks, (uint8_t*)g->payload);
        else
            update_scatter_kernel<uint32_t><<<blocks, 256, 0, st>>>(
                v2, u, (const uint64_t*)(scr + o_words), (const uint32_t*)(scr + o_pay),
                (const uint32_t*)(scr + o_slots), g->dir, g->masks, (uint32_t*)g->payload);
        e = cudaGetLastError();
        // 5. distances and octant words over the whole directory
        BuildScratch bs;
        bs.dist_a = (uint8_t*)(scr + o_da);
        bs.dist_b = (uint8_t*)(scr + o_db);
        uint32_t* occ = (uint32_t*)(scr + o_occ);
        if (e == cudaSuccess)
            e = launch_brick_xmask(g->dir, occ, (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz, st,
                                   &changed);
        if (e == cudaSuccess)
            e = launch_brick_distance(bs, g->dir, (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz, st,
                                      &changed, occ);
        if (e == cudaSuccess)
            e = launch_brick_octants(g->dir, (uint8_t*)(scr + o_da), (uint16_t*)(scr + o_ty), g->oct,
                                     (int32_t)g->bx, (int32_t)g->by, (int32_t)g->bz, st, &changed, occ);
        if (e == cudaSuccess)
            e = launch_brick_long(g->dir, g->oct, (uint32_t*)(scr + o_run), g->lng, (int32_t)g->bx,
                                  (int32_t)g->by, (int32_t)g->bz, st, &changed, occ);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { rc = cuda_fail(e, "vt_grid_update: scatter"); break; }
        uint64_t nonempty = 0;
        for (uint64_t k = 0; k < K; ++k) {
            const bool was = !(old[k] & kEmptyBit), now = flags[k] != 0;
            nonempty += (uint64_t)now - (uint64_t)was;
        }
        g->nonempty += nonempty;  // modular: a net decrease wraps back
        g->occupied = (uint64_t)((long long)g->occupied + delta);
    } while (0);
    cudaFreeAsync(scr, st);
    cudaStreamSynchronize(st);
    return rc;
}
