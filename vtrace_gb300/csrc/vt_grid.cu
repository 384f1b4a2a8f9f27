// vt_grid.cu — brick re-layout of a dense voxel grid (the ingest side of vtrace's add_texture,
// lib/memory.c:286-385): x-fastest u8 palette indices or RGBA8 texels in device memory become
// an 8^3-brick directory, 512-bit occupancy masks and dense payloads of occupied bricks only.
//
// Three passes, all coalesced along x:
//   words   one thread per (brick, z-slice): reads 8 rows of 8 voxels, builds the 64-bit
//           occupancy word; the 8 lanes of a brick OR their words into the brick's flag
//   scan    exclusive prefix sum of the flags = each occupied brick's slot
//   compact one thread per (brick, z-slice) of occupied bricks: copies the word and the slice's
//           64 voxels into the slot; writes the directory
// Lanes are assigned slice-fastest, so a warp covers 4 consecutive bricks along x: its reads are
// 8 z-planes x 32 contiguous bytes per row and its word writes are 256 contiguous bytes.
// With a staging buffer (one 512-voxel block per brick, indexed by brick), the words pass also
// writes the voxels of each occupied brick there, brick-major, while it holds them, and the
// compaction copies whole staged blocks: without it the compaction re-reads the dense grid's rows,
// whose 32-byte sectors each span four bricks along x, so a grid with few occupied bricks is read
// several times over (4.8x the payload on a 1024^3 grid with 9.5% of its bricks occupied).
#include <cuda_runtime.h>

#include "vt_device.cuh"
#include "vt_kernels.h"

namespace vt {

constexpr int kScanThreads = 1024, kScanItems = 4;
constexpr uint64_t kScanBlock = (uint64_t)kScanThreads * kScanItems;

static inline uint64_t align_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

static uint64_t scan_partials(uint64_t n) {
    // partial sums of every recursion level of the scan
    uint64_t total = 0;
    while (n > kScanBlock) {
        n = (n + kScanBlock - 1) / kScanBlock;
        total += align_up(n, 64);
    }
    return total + 64;
}

size_t build_scratch_bytes(uint64_t bricks) {
    return (size_t)(align_up(bricks * 64, 256) + align_up(bricks * 4, 256) * 2 +
                    align_up(scan_partials(bricks) * 4, 256) + 256 + align_up(bricks, 256) * 2);
}

size_t build_staging_bytes(uint64_t bricks, uint32_t format) {
    return (size_t)align_up(bricks * 512 * (format == VT_PAYLOAD_RGBA8 ? 4 : 1), 256);
}

BuildScratch carve_build_scratch(void* base, uint64_t bricks) {
    char* p = (char*)base;
    BuildScratch s;
    s.words = (uint64_t*)p;
    p += align_up(bricks * 64, 256);
    s.flags = (uint32_t*)p;
    p += align_up(bricks * 4, 256);
    s.offsets = (uint32_t*)p;
    p += align_up(bricks * 4, 256);
    s.block_sums = (uint32_t*)p;
    p += align_up(scan_partials(bricks) * 4, 256);
    s.occupied = (unsigned long long*)p;
    p += 256;
    s.dist_a = (uint8_t*)p;
    p += align_up(bricks, 256);
    s.dist_b = (uint8_t*)p;
    return s;
}

struct BrickCoord {
    int32_t bxi, byi, bzi;
};

__device__ __forceinline__ BrickCoord brick_coord(uint64_t brick, int32_t bx, int32_t by) {
    BrickCoord c;
    c.bxi = (int32_t)(brick % (uint64_t)bx);
    const uint64_t r = brick / (uint64_t)bx;
    c.byi = (int32_t)(r % (uint64_t)by);
    c.bzi = (int32_t)(r / (uint64_t)by);
    return c;
}

// Brick of thread (blockIdx.x * blockDim.x + threadIdx.x) in `box`; false past its end.
__device__ __forceinline__ bool box_brick(const BrickBox& box, int32_t bx, int32_t by,
                                          BrickCoord& c, uint64_t& b) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)box.nx * box.ny * box.nz) return false;
    c.bxi = box.x0 + (int32_t)(t % (uint64_t)box.nx);
    const uint64_t r = t / (uint64_t)box.nx;
    c.byi = box.y0 + (int32_t)(r % (uint64_t)box.ny);
    c.bzi = box.z0 + (int32_t)(r / (uint64_t)box.ny);
    b = (uint64_t)c.bxi + (uint64_t)bx * ((uint64_t)c.byi + (uint64_t)by * (uint64_t)c.bzi);
    return true;
}

// Occupancy bits of 8 u8 voxels packed in a u64 when "occupied" means "nonzero index": the high
// bit of each byte of ((v & 0x7F..) + 0x7F..) | v is set iff the byte is nonzero; the multiply
// gathers the eight high bits into the top byte (bit k from byte k).
__device__ __forceinline__ uint32_t nonzero_bytes(uint64_t v) {
    const uint64_t hi = (((v & 0x7F7F7F7F7F7F7F7Full) + 0x7F7F7F7F7F7F7F7Full) | v) & 0x8080808080808080ull;
    return (uint32_t)(((hi >> 7) * 0x0102040810204080ull) >> 56);
}

// Occupancy bits of one 8-voxel row: bit lx set iff voxel x0+lx is inside the grid and occupied.
template <uint32_t FMT>
__device__ __forceinline__ uint32_t row_bits(const void* src, const uint8_t* lut, size_t row_base,
                                             int32_t x0, int32_t nx, bool nz = false) {
    uint32_t bits = 0;
    if (FMT == VT_PAYLOAD_U8) {
        const uint8_t* row = (const uint8_t*)src + row_base + x0;
        if (x0 + 8 <= nx && (((uintptr_t)row) & 7u) == 0) {
            const uint2 v = __ldg((const uint2*)row);
            if (nz) return nonzero_bytes(((uint64_t)v.y << 32) | v.x);
#pragma unroll
            for (int k = 0; k < 4; ++k) bits |= (uint32_t)lut[(v.x >> (8 * k)) & 0xFFu] << k;
#pragma unroll
            for (int k = 0; k < 4; ++k) bits |= (uint32_t)lut[(v.y >> (8 * k)) & 0xFFu] << (k + 4);
        } else {
            for (int k = 0; k < 8 && x0 + k < nx; ++k) {
                const uint8_t b = __ldg(row + k);
                bits |= (uint32_t)(nz ? b != 0 : lut[b]) << k;
            }
        }
    } else {
        const uint32_t* row = (const uint32_t*)src + row_base + x0;
        if (x0 + 8 <= nx && (((uintptr_t)row) & 15u) == 0) {
            const uint4 a = __ldg((const uint4*)row), b = __ldg((const uint4*)row + 1);
            const uint32_t t[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) bits |= (uint32_t)((t[k] >> 24) != 0u) << k;
        } else {
            for (int k = 0; k < 8 && x0 + k < nx; ++k)
                bits |= (uint32_t)((__ldg(row + k) >> 24) != 0u) << k;
        }
    }
    return bits;
}

// Z-slice lz of brick c: 8 rows of 8 voxels, zero past the grid's edge, stored as 64 elements
// (x fastest, then y) at dst (8-byte aligned for u8, 16-byte for RGBA8).
template <uint32_t FMT>
__device__ __forceinline__ void copy_slice(const void* __restrict__ src, int32_t nx, int32_t ny,
                                           int32_t nz, const BrickCoord& c, uint32_t lz,
                                           void* __restrict__ dst) {
    const int32_t z = c.bzi * 8 + (int32_t)lz, x0 = c.bxi * 8;
    for (int ly = 0; ly < 8; ++ly) {
        const int32_t y = c.byi * 8 + ly;
        const bool row_in = z < nz && y < ny;
        const size_t row_base = (size_t)nx * ((size_t)y + (size_t)ny * (size_t)z);
        if (FMT == VT_PAYLOAD_U8) {
            const uint8_t* row = (const uint8_t*)src + row_base + x0;
            uint2 v = make_uint2(0u, 0u);
            if (row_in) {
                if (x0 + 8 <= nx && (((uintptr_t)row) & 7u) == 0) {
                    v = __ldg((const uint2*)row);
                } else {
                    uint32_t b[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    for (int k = 0; k < 8 && x0 + k < nx; ++k) b[k] = __ldg(row + k);
                    v.x = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24);
                    v.y = b[4] | (b[5] << 8) | (b[6] << 16) | (b[7] << 24);
                }
            }
            ((uint2*)dst)[ly] = v;
        } else {
            const uint32_t* row = (const uint32_t*)src + row_base + x0;
            uint4 a = make_uint4(0u, 0u, 0u, 0u), b = a;
            if (row_in) {
                if (x0 + 8 <= nx && (((uintptr_t)row) & 15u) == 0) {
                    a = __ldg((const uint4*)row);
                    b = __ldg((const uint4*)row + 1);
                } else {
                    uint32_t q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    for (int k = 0; k < 8 && x0 + k < nx; ++k) q[k] = __ldg(row + k);
                    a = make_uint4(q[0], q[1], q[2], q[3]);
                    b = make_uint4(q[4], q[5], q[6], q[7]);
                }
            }
            uint4* p = (uint4*)dst + 2 * ly;
            p[0] = a;
            p[1] = b;
        }
    }
}

// NZ: u8 grid whose palette has alpha 0 at index 0 only, so that occupancy is "index != 0" and the
// row bits come from byte arithmetic instead of palette lookups.
template <uint32_t FMT, bool NZ>
__global__ void __launch_bounds__(256) brick_words_kernel(const void* __restrict__ src,
                                                          const uint32_t* __restrict__ palette,
                                                          int32_t nx, int32_t ny, int32_t nz,
                                                          int32_t bx, int32_t by, uint64_t bricks,
                                                          uint64_t* __restrict__ words,
                                                          uint32_t* __restrict__ flags,
                                                          unsigned long long* occupied,
                                                          void* __restrict__ staged) {
    __shared__ uint8_t lut[256];
    if (FMT == VT_PAYLOAD_U8 && !NZ) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            lut[i] = (uint8_t)((__ldg(palette + i) >> 24) != 0u);
        __syncthreads();
    }
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lz = (uint32_t)(t & 7u);
    const uint64_t brick = t >> 3;
    const bool valid = brick < bricks;
    uint64_t w = 0;
    BrickCoord c = {0, 0, 0};
    bool whole = false;  // the slice's rows are in r[], 8-byte aligned and inside the grid
    uint64_t r[8];
    if (valid) {
        c = brick_coord(brick, bx, by);
        const int32_t z = c.bzi * 8 + (int32_t)lz, x0 = c.bxi * 8;
        if (z < nz) {
            const size_t plane = (size_t)nx * (size_t)ny * (size_t)z;
            if (NZ && x0 + 8 <= nx && (nx & 7) == 0 && c.byi * 8 + 8 <= ny) {
                // whole rows, 8-byte aligned: issue the eight loads before using any
                const uint8_t* base = (const uint8_t*)src + plane + (size_t)nx * (size_t)(c.byi * 8) + x0;
                whole = true;
#pragma unroll
                for (int ly = 0; ly < 8; ++ly) r[ly] = __ldg((const unsigned long long*)(base + (size_t)nx * ly));
#pragma unroll
                for (int ly = 0; ly < 8; ++ly) w |= (uint64_t)nonzero_bytes(r[ly]) << (8 * ly);
            } else {
                for (int ly = 0; ly < 8; ++ly) {
                    const int32_t y = c.byi * 8 + ly;
                    if (y >= ny) break;
                    const size_t row_base = plane + (size_t)nx * (size_t)y;
                    w |= (uint64_t)row_bits<FMT>(src, NZ ? nullptr : lut, row_base, x0, nx, NZ) << (8 * ly);
                }
            }
        }
    }
    uint64_t any = w;
    any |= __shfl_xor_sync(0xFFFFFFFFu, any, 1);
    any |= __shfl_xor_sync(0xFFFFFFFFu, any, 2);
    any |= __shfl_xor_sync(0xFFFFFFFFu, any, 4);
    if (valid) {
        words[brick * 8 + lz] = w;
        if (lz == 0) flags[brick] = any != 0 ? 1u : 0u;
        if (staged && any) {  // the brick's block in the staging buffer, slice lz
            constexpr size_t E = FMT == VT_PAYLOAD_RGBA8 ? 4 : 1;
            uint8_t* dst = (uint8_t*)staged + (brick * 512 + lz * 64) * E;
            if (whole) {
                uint4* p = (uint4*)dst;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    p[k] = make_uint4((uint32_t)r[2 * k], (uint32_t)(r[2 * k] >> 32),
                                      (uint32_t)r[2 * k + 1], (uint32_t)(r[2 * k + 1] >> 32));
            } else {
                copy_slice<FMT>(src, nx, ny, nz, c, lz, dst);  // rows just read: cache hits
            }
        }
    }
    unsigned long long pc = (unsigned long long)__popcll(w);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pc += __shfl_xor_sync(0xFFFFFFFFu, pc, off);
    if ((threadIdx.x & 31) == 0 && pc) atomicAdd(occupied, pc);
}

// Exclusive scan of up to kScanBlock items per block; block totals go to `sums`.
__global__ void __launch_bounds__(kScanThreads) scan_block_kernel(const uint32_t* __restrict__ in,
                                                                  uint32_t* __restrict__ out,
                                                                  uint64_t n,
                                                                  uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanBlock + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        local += v[k];
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t wt = warp_tot[lane], wi = wt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, off);
            if (lane >= (uint32_t)off) wi += y;
        }
        warp_tot[lane] = wi - wt;  // exclusive prefix of warp totals
        if (lane == 31) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, uint64_t n,
                                const uint32_t* __restrict__ block_offsets) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += block_offsets[i / kScanBlock];
}

static cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* partial,
                                  cudaStream_t stream) {
    const uint64_t blocks = (n + kScanBlock - 1) / kScanBlock;
    scan_block_kernel<<<(unsigned)blocks, kScanThreads, 0, stream>>>(in, out, n, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || blocks == 1) return e;
    // scan the block totals in place one level up, then add them back
    uint32_t* next = partial + align_up(blocks, 64);
    e = scan_exclusive(partial, partial, blocks, next, stream);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(out, n, partial);
    return cudaGetLastError();
}

cudaError_t launch_brick_scan(const BuildScratch& s, uint64_t bricks, cudaStream_t stream) {
    return scan_exclusive(s.flags, s.offsets, bricks, s.block_sums, stream);
}

cudaError_t launch_brick_words(const void* src, uint32_t format, const uint32_t* d_palette,
                               int32_t nx, int32_t ny, int32_t nz, const BuildScratch& s,
                               cudaStream_t stream, bool nonzero_occupancy) {
    const int32_t bx = (nx + 7) / 8, by = (ny + 7) / 8, bz = (nz + 7) / 8;
    const uint64_t bricks = (uint64_t)bx * by * bz;
    const uint64_t threads = bricks * 8;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    cudaError_t e = cudaMemsetAsync(s.occupied, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    if (format == VT_PAYLOAD_U8 && nonzero_occupancy)
        brick_words_kernel<VT_PAYLOAD_U8, true><<<blocks, 256, 0, stream>>>(
            src, d_palette, nx, ny, nz, bx, by, bricks, s.words, s.flags, s.occupied, s.staged);
    else if (format == VT_PAYLOAD_U8)
        brick_words_kernel<VT_PAYLOAD_U8, false><<<blocks, 256, 0, stream>>>(
            src, d_palette, nx, ny, nz, bx, by, bricks, s.words, s.flags, s.occupied, s.staged);
    else
        brick_words_kernel<VT_PAYLOAD_RGBA8, false><<<blocks, 256, 0, stream>>>(
            src, nullptr, nx, ny, nz, bx, by, bricks, s.words, s.flags, s.occupied, s.staged);
    return cudaGetLastError();
}

template <uint32_t FMT>
__global__ void __launch_bounds__(256) brick_compact_kernel(
    const void* __restrict__ src, int32_t nx, int32_t ny, int32_t nz, int32_t bx, int32_t by,
    uint64_t bricks, const uint64_t* __restrict__ words, const uint32_t* __restrict__ flags,
    const uint32_t* __restrict__ offsets, uint32_t* __restrict__ dir, uint64_t* __restrict__ masks,
    void* __restrict__ payload, const void* __restrict__ staged) {
    constexpr size_t E = FMT == VT_PAYLOAD_RGBA8 ? 4 : 1;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lz = (uint32_t)(t & 7u);
    const uint64_t brick = t >> 3;
    if (brick >= bricks) return;
    const uint32_t f = __ldg(flags + brick);
    const uint32_t slot = __ldg(offsets + brick);
    if (lz == 0) dir[brick] = f ? slot : kEmptyBit;  // distance filled in by the distance passes
    if (!f) return;
    masks[(size_t)slot * 8 + lz] = __ldg(words + brick * 8 + lz);
    if (staged) {
        // the brick's staged block, 16 bytes per lane and load: the 8 lanes of a brick read 128
        // contiguous bytes per instruction
        const uint4* from = (const uint4*)((const uint8_t*)staged + brick * 512 * E);
        uint4* to = (uint4*)((uint8_t*)payload + (size_t)slot * 512 * E);
#pragma unroll
        for (uint32_t k = 0; k < 4 * E; ++k) to[lz + 8 * k] = __ldg(from + lz + 8 * k);
        return;
    }
    copy_slice<FMT>(src, nx, ny, nz, brick_coord(brick, bx, by), lz,
                    (uint8_t*)payload + ((size_t)slot * 512 + lz * 64) * E);
}

cudaError_t launch_brick_compact(const void* src, uint32_t format, int32_t nx, int32_t ny,
                                 int32_t nz, const BuildScratch& s, uint32_t* dir,
                                 uint64_t* masks, void* payload, cudaStream_t stream) {
    const int32_t bx = (nx + 7) / 8, by = (ny + 7) / 8, bz = (nz + 7) / 8;
    const uint64_t bricks = (uint64_t)bx * by * bz;
    const unsigned blocks = (unsigned)((bricks * 8 + 255) / 256);
    if (format == VT_PAYLOAD_U8)
        brick_compact_kernel<VT_PAYLOAD_U8><<<blocks, 256, 0, stream>>>(
            src, nx, ny, nz, bx, by, bricks, s.words, s.flags, s.offsets, dir, masks, payload,
            s.staged);
    else
        brick_compact_kernel<VT_PAYLOAD_RGBA8><<<blocks, 256, 0, stream>>>(
            src, nx, ny, nz, bx, by, bricks, s.words, s.flags, s.offsets, dir, masks, payload,
            s.staged);
    return cudaGetLastError();
}

// Occupancy bitmask of the brick lattice for the passes along x: row (y, z) is occ_words(bx) words,
// bit x of the row set iff brick (x, y, z) is occupied.  One thread per word.
__host__ __device__ __forceinline__ int32_t occ_words(int32_t bx) { return (bx + 31) >> 5; }

__global__ void __launch_bounds__(256) brick_xmask_kernel(const uint32_t* __restrict__ dir,
                                                          uint32_t* __restrict__ occ, int32_t bx,
                                                          int32_t by, int32_t y0, int32_t ny,
                                                          int32_t z0, uint64_t words) {
    // words of the rows y0 .. y0 + ny - 1 of the planes z0 ..
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= words) return;
    const int32_t rw = occ_words(bx);
    const uint64_t r = t / (uint64_t)rw;
    const uint64_t row = (uint64_t)(z0 + (int32_t)(r / (uint64_t)ny)) * by + y0 + (int32_t)(r % (uint64_t)ny);
    const int32_t x0 = (int32_t)(t - r * (uint64_t)rw) * 32;
    const uint64_t w = row * rw + (uint64_t)(x0 >> 5);
    const uint32_t* d = dir + row * (uint64_t)bx + x0;
    const int32_t n = min(32, bx - x0);
    uint32_t m = 0;
    for (int32_t k = 0; k < n; ++k) m |= (uint32_t)!brick_empty(__ldg(d + k)) << k;
    occ[w] = m;
}

// Steps from brick x of an occupancy row to the nearest occupied brick in direction s (+1 / -1),
// the brick itself included (0 when occupied), or `cap` (<= 31) when none lies within cap - 1
// steps; beyond the row counts as empty.  Reads at most two words.
__device__ __forceinline__ int32_t occ_fwd(const uint32_t* __restrict__ row, int32_t rw, int32_t x,
                                           int32_t s, int32_t cap) {
    const int32_t w = x >> 5, b = x & 31;
    if (s > 0) {
        uint64_t v = __ldg(row + w);
        if (w + 1 < rw) v |= (uint64_t)__ldg(row + w + 1) << 32;
        const uint32_t m = (uint32_t)(v >> b) & ((1u << cap) - 1u);  // bit k: brick x + k
        return m ? __ffs(m) - 1 : cap;
    }
    uint64_t v = (uint64_t)__ldg(row + w) << 32;
    if (w > 0) v |= __ldg(row + w - 1);
    const uint32_t m = (uint32_t)((v << (31 - b)) >> 32) & ~((1u << (32 - cap)) - 1u);  // bit 31 - k: brick x - k
    return m ? __clz(m) : cap;
}

cudaError_t launch_brick_xmask(const uint32_t* dir, uint32_t* occ, int32_t bx, int32_t by,
                               int32_t bz, cudaStream_t stream, const BrickBox* changed) {
    // after a change, the rows the passes along x read: those of the distance pass's window (its
    // y and z reach, kMaxBrickDistance twice over, covers the octant and long-box windows)
    int32_t y0 = 0, ny = by, z0 = 0, nz = bz;
    if (changed) {
        const int32_t R = 2 * (int32_t)kMaxBrickDistance;
        y0 = max(changed->y0 - R, 0);
        z0 = max(changed->z0 - R, 0);
        ny = min(changed->y0 + changed->ny + R, by) - y0;
        nz = min(changed->z0 + changed->nz + R, bz) - z0;
    }
    const uint64_t words = (uint64_t)occ_words(bx) * ny * nz;
    brick_xmask_kernel<<<(unsigned)((words + 255) / 256), 256, 0, stream>>>(dir, occ, bx, by, y0,
                                                                             ny, z0, words);
    return cudaGetLastError();
}

size_t brick_xmask_words(int32_t bx, int32_t by, int32_t bz) {
    return (size_t)occ_words(bx) * by * bz;
}

// Chebyshev (L-infinity) distance, in bricks, from each empty brick to the nearest occupied one,
// capped at kMaxBrickDistance.  The transform is separable: pass x computes the 1D distance
// along x; passes y and z take min over the line of max(|offset|, previous pass), which composes
// max over axes.  Each thread handles one brick and scans a window of +-kMaxBrickDistance.
template <int AXIS>
__global__ void __launch_bounds__(256) brick_distance_kernel(uint32_t* __restrict__ dir,
                                                             const uint8_t* __restrict__ in,
                                                             uint8_t* __restrict__ out,
                                                             int32_t bx, int32_t by, int32_t bz,
                                                             BrickBox box,
                                                             const uint32_t* __restrict__ occ) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    if (AXIS == 0 && occ) {  // pass x from the occupancy rows
        const int32_t rw = occ_words(bx);
        const uint32_t* row = occ + ((uint64_t)c.bzi * by + c.byi) * rw;
        const int32_t cap = (int32_t)kMaxBrickDistance;
        out[b] = (uint8_t)min(occ_fwd(row, rw, c.bxi, 1, cap), occ_fwd(row, rw, c.bxi, -1, cap));
        return;
    }
    const int32_t pos = AXIS == 0 ? c.bxi : (AXIS == 1 ? c.byi : c.bzi);
    const int32_t n = AXIS == 0 ? bx : (AXIS == 1 ? by : bz);
    const int64_t stride = AXIS == 0 ? 1 : (AXIS == 1 ? (int64_t)bx : (int64_t)bx * by);
    const int32_t cap = (int32_t)kMaxBrickDistance;
    // min over offsets j of max(|j|, val(pos + j)), visiting |j| = 0, 1, 2, ... and stopping once
    // |j| reaches the best value found (no farther offset can improve it)
    int32_t best = cap;
    for (int32_t r = 0; r < best; ++r) {
#pragma unroll
        for (int sgn = 0; sgn < 2; ++sgn) {
            if (r == 0 && sgn) continue;
            const int32_t p = sgn ? pos - r : pos + r;
            if (p < 0 || p >= n) continue;
            const int64_t idx = (int64_t)b + (int64_t)(p - pos) * stride;
            const int32_t val = AXIS == 0 ? (brick_empty(__ldg(dir + idx)) ? cap : 0) : (int32_t)__ldg(in + idx);
            best = min(best, max(r, val));
        }
    }
    if (AXIS < 2) {
        out[b] = (uint8_t)best;
    } else if (brick_empty(dir[b])) {
        dir[b] = kEmptyBit | (uint32_t)max(best, 1);
    }
}

// Forward (octant) distances: for every brick and each of the 8 sign combinations (sx, sy, sz) of
// a ray direction, the largest K <= kMaxOctantDistance such that the box of K x K x K bricks
// starting at the brick and extending in the directions (sx, sy, sz) holds no occupied brick
// (0 for an occupied brick).  Separable: pass x gives the 1D forward distance for sx = +/-1,
// pass y takes min_j max(j, pass_x(b + j*sy)) for the four (sx, sy), pass z likewise for all
// eight.  Packed 4 bits per octant, octant index (sx<0) | (sy<0)<<1 | (sz<0)<<2.
constexpr int kMaxOctantDistance = 15;

__global__ void __launch_bounds__(256) brick_octant_x_kernel(const uint32_t* __restrict__ dir,
                                                             uint8_t* __restrict__ out,
                                                             int32_t bx, int32_t by,
                                                             BrickBox box,
                                                             const uint32_t* __restrict__ occ) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    if (occ) {
        const int32_t rw = occ_words(bx);
        const uint32_t* row = occ + ((uint64_t)c.bzi * by + c.byi) * rw;
        const int32_t cap = (int32_t)kMaxOctantDistance;
        out[b] = (uint8_t)(occ_fwd(row, rw, c.bxi, 1, cap) | (occ_fwd(row, rw, c.bxi, -1, cap) << 4));
        return;
    }
    uint32_t packed = 0;
#pragma unroll
    for (int neg = 0; neg < 2; ++neg) {
        const int32_t sx = neg ? -1 : 1;
        int32_t best = kMaxOctantDistance;
        for (int32_t k = 0; k < kMaxOctantDistance; ++k) {
            const int32_t x = c.bxi + k * sx;
            if (x < 0 || x >= bx) break;
            if (!brick_empty(__ldg(dir + (int64_t)b + (int64_t)k * sx))) {
                best = k;
                break;
            }
        }
        packed |= (uint32_t)best << (4 * neg);
    }
    out[b] = (uint8_t)packed;
}

__global__ void __launch_bounds__(256) brick_octant_y_kernel(const uint8_t* __restrict__ in,
                                                             uint16_t* __restrict__ out,
                                                             int32_t bx, int32_t by,
                                                             BrickBox box) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    uint32_t packed = 0;
#pragma unroll
    for (int ny = 0; ny < 2; ++ny) {  // one walk per sy serves both sx
        const int32_t sy = ny ? -1 : 1;
        int32_t best[2] = {(int32_t)kMaxOctantDistance, (int32_t)kMaxOctantDistance};
        for (int32_t j = 0; j < max(best[0], best[1]); ++j) {
            const int32_t y = c.byi + j * sy;
            if (y < 0 || y >= by) break;
            const uint32_t f = __ldg(in + (int64_t)b + (int64_t)j * sy * bx);
#pragma unroll
            for (int nx = 0; nx < 2; ++nx) best[nx] = min(best[nx], max(j, (int32_t)((f >> (4 * nx)) & 15u)));
        }
#pragma unroll
        for (int nx = 0; nx < 2; ++nx) packed |= (uint32_t)best[nx] << (4 * (nx | (ny << 1)));
    }
    out[b] = (uint16_t)packed;
}

__global__ void __launch_bounds__(256) brick_octant_z_kernel(const uint16_t* __restrict__ in,
                                                             uint32_t* __restrict__ out,
                                                             int32_t bx, int32_t by, int32_t bz,
                                                             BrickBox box) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    const int64_t plane = (int64_t)bx * by;
    uint32_t packed = 0;
#pragma unroll
    for (int nz = 0; nz < 2; ++nz) {  // one walk per sz serves the four (sx, sy)
        const int32_t sz = nz ? -1 : 1;
        int32_t best[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) best[q] = (int32_t)kMaxOctantDistance;
        int32_t lim = (int32_t)kMaxOctantDistance;
        for (int32_t l = 0; l < lim; ++l) {
            const int32_t z = c.bzi + l * sz;
            if (z < 0 || z >= bz) break;
            const uint32_t f = __ldg(in + (int64_t)b + (int64_t)l * sz * plane);
            lim = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                best[q] = min(best[q], max(l, (int32_t)((f >> (4 * q)) & 15u)));
                lim = max(lim, best[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) packed |= (uint32_t)best[q] << (4 * (q | (nz << 2)));
    }
    out[b] = packed;
}

// Forward empty runs: for axis a and direction s = +1 / -1, the number of consecutive empty
// bricks from this one (itself included) toward s along a, capped at kMaxOctantDistance; beyond the
// grid counts as empty.  Nibble 2a + (s < 0).
__global__ void __launch_bounds__(256) brick_run_kernel(const uint32_t* __restrict__ dir,
                                                        uint32_t* __restrict__ run, int32_t bx,
                                                        int32_t by, int32_t bz, BrickBox box,
                                                        const uint32_t* __restrict__ occ) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    const int32_t pos[3] = {c.bxi, c.byi, c.bzi}, n[3] = {bx, by, bz};
    const int64_t stride[3] = {1, (int64_t)bx, (int64_t)bx * by};
    uint32_t packed = 0;
    int a0 = 0;
    if (occ) {  // axis x from the occupancy rows
        const int32_t rw = occ_words(bx);
        const uint32_t* row = occ + ((uint64_t)c.bzi * by + c.byi) * rw;
        const int32_t cap = (int32_t)kMaxOctantDistance;
        packed = (uint32_t)occ_fwd(row, rw, c.bxi, 1, cap) | ((uint32_t)occ_fwd(row, rw, c.bxi, -1, cap) << 4);
        a0 = 1;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a < a0) continue;
#pragma unroll
        for (int neg = 0; neg < 2; ++neg) {
            const int32_t sg = neg ? -1 : 1;
            int32_t best = kMaxOctantDistance;
            for (int32_t k = 0; k < (int32_t)kMaxOctantDistance; ++k) {
                const int32_t p = pos[a] + k * sg;
                if (p < 0 || p >= n[a]) break;
                if (!brick_empty(__ldg(dir + (int64_t)b + (int64_t)k * sg * stride[a]))) {
                    best = k;
                    break;
                }
            }
            packed |= (uint32_t)best << (4 * (2 * a + neg));
        }
    }
    run[b] = packed;
}

// Window minima of the runs: level p of axis a holds, for octant o (nibble o), the smallest run
// along a toward o over the 2^p x 2^p bricks across from the brick toward o (cells beyond the
// grid count as the cap).  Level 0 repacks the runs per octant; level p + 1 is the minimum of four
// level-p blocks.  The levels are stored for the bricks of the index window `pw` (the whole
// lattice for a full build): pyr[(p * 3 + a) * |pw| + local index in pw].
__device__ __forceinline__ int64_t pyr_index(const BrickBox& pw, int32_t x, int32_t y, int32_t z) {
    if (x < pw.x0 || y < pw.y0 || z < pw.z0 || x >= pw.x0 + pw.nx || y >= pw.y0 + pw.ny ||
        z >= pw.z0 + pw.nz)
        return -1;  // not stored: the windows of a partial pass are nested so that this is not read
    return (int64_t)(x - pw.x0) + (int64_t)pw.nx * ((int64_t)(y - pw.y0) + (int64_t)pw.ny * (z - pw.z0));
}

// WIN: `pw` is a window of the lattice (a partial pass, whose windows are nested so that every
// neighbour read lies in it; checked all the same); otherwise it is the whole lattice and the local
// index is the brick index.  Neighbours are addressed by local strides.
template <bool WIN>
__device__ __forceinline__ bool pyr_in(const BrickBox& pw, int a, int32_t v) {
    if (!WIN) return true;
    const int32_t lo = a == 0 ? pw.x0 : (a == 1 ? pw.y0 : pw.z0);
    const int32_t n = a == 0 ? pw.nx : (a == 1 ? pw.ny : pw.nz);
    return v >= lo && v < lo + n;
}

template <bool WIN>
__global__ void __launch_bounds__(256) brick_pyramid_kernel(const uint32_t* __restrict__ run,
                                                            uint32_t* __restrict__ pyr, int32_t p,
                                                            int32_t bx, int32_t by, int32_t bz,
                                                            BrickBox box, BrickBox pw) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    const uint64_t pn = (uint64_t)pw.nx * pw.ny * pw.nz;
    const int32_t pos[3] = {c.bxi, c.byi, c.bzi}, n[3] = {bx, by, bz};
    const int64_t ls[3] = {1, (int64_t)pw.nx, (int64_t)pw.nx * pw.ny};
    const int64_t self_i = WIN ? pyr_index(pw, c.bxi, c.byi, c.bzi) : (int64_t)b;
    if (self_i < 0) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        uint32_t packed = 0;
        if (p == 0) {
            const uint32_t r = __ldg(run + b);
#pragma unroll
            for (int o = 0; o < 8; ++o) packed |= ((r >> (4 * (2 * a + ((o >> a) & 1)))) & 15u) << (4 * o);
        } else {
            const int e1 = (a + 1) % 3, e2 = (a + 2) % 3;
            const int32_t h = 1 << (p - 1);
            const uint32_t* prev = pyr + (uint64_t)((p - 1) * 3 + a) * pn;
            const uint32_t self = __ldg(prev + self_i);
#pragma unroll
            for (int q = 0; q < 4; ++q) {  // lateral signs (bit 0: e1 negative, bit 1: e2 negative)
                const int32_t s1 = (q & 1) ? -1 : 1, s2 = (q & 2) ? -1 : 1;
                const int32_t c1 = pos[e1] + h * s1, c2 = pos[e2] + h * s2;
                const bool in1 = c1 >= 0 && c1 < n[e1] && pyr_in<WIN>(pw, e1, c1);
                const bool in2 = c2 >= 0 && c2 < n[e2] && pyr_in<WIN>(pw, e2, c2);
                const int64_t d1 = (int64_t)h * s1 * ls[e1], d2 = (int64_t)h * s2 * ls[e2];
                const uint32_t w1 = in1 ? __ldg(prev + self_i + d1) : 0xFFFFFFFFu;
                const uint32_t w2 = in2 ? __ldg(prev + self_i + d2) : 0xFFFFFFFFu;
                const uint32_t w3 = in1 && in2 ? __ldg(prev + self_i + d1 + d2) : 0xFFFFFFFFu;
#pragma unroll
                for (int o = 0; o < 8; ++o) {
                    if (((o >> e1) & 1) != (q & 1) || ((o >> e2) & 1) != ((q >> 1) & 1)) continue;
                    const uint32_t sh = 4 * o;
                    const uint32_t m = min(min((self >> sh) & 15u, (w1 >> sh) & 15u),
                                           min((w2 >> sh) & 15u, (w3 >> sh) & 15u));
                    packed |= m << sh;
                }
            }
        }
        pyr[(uint64_t)(p * 3 + a) * pn + self_i] = packed;
    }
}

// Long forward boxes: for axis a and octant o with forward cube K (octant word), the largest
// L <= kMaxOctantDistance such that the box L bricks long along a and K x K across, all toward o,
// is empty: the smallest run along a over the box's K x K cross-section, read as the minimum of
// four overlapping 2^p blocks of the pyramid (2^p <= K < 2^(p+1)).  L >= K since the cube is
// empty; K = 0 (occupied brick) gives 0 and K at the cap gives the cap.
template <bool WIN>
__global__ void __launch_bounds__(256) brick_long_kernel(const uint32_t* __restrict__ oct,
                                                         const uint32_t* __restrict__ pyr,
                                                         uint32_t* __restrict__ lng, int32_t bx,
                                                         int32_t by, int32_t bz, BrickBox box,
                                                         BrickBox pw) {
    BrickCoord c;
    uint64_t b;
    if (!box_brick(box, bx, by, c, b)) return;
    const uint64_t bricks = (uint64_t)bx * by * bz;
    const uint64_t pn = (uint64_t)pw.nx * pw.ny * pw.nz;
    const int32_t pos[3] = {c.bxi, c.byi, c.bzi}, n[3] = {bx, by, bz};
    const int64_t ls[3] = {1, (int64_t)pw.nx, (int64_t)pw.nx * pw.ny};
    const int64_t self_i = WIN ? pyr_index(pw, c.bxi, c.byi, c.bzi) : (int64_t)b;
    const uint32_t ow = __ldg(oct + b);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int e1 = (a + 1) % 3, e2 = (a + 2) % 3;
        uint32_t packed = 0;
        for (int o = 0; o < 8; ++o) {
            const int32_t K = (int32_t)((ow >> (4 * o)) & 15u);
            int32_t L = K;
            if (K > 0 && K < (int32_t)kMaxOctantDistance && self_i >= 0) {
                const int32_t p = 31 - __clz(K);  // 2^p <= K < 2^(p+1), p <= 3
                const int32_t off = K - (1 << p);
                const int32_t s1 = (o >> e1) & 1 ? -1 : 1, s2 = (o >> e2) & 1 ? -1 : 1;
                const uint32_t* lev = pyr + (uint64_t)(p * 3 + a) * pn;
                L = kMaxOctantDistance;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int32_t o1 = (k & 1) ? off : 0, o2 = (k & 2) ? off : 0;
                    const int32_t c1 = pos[e1] + o1 * s1, c2 = pos[e2] + o2 * s2;
                    if (c1 < 0 || c1 >= n[e1] || c2 < 0 || c2 >= n[e2]) continue;
                    if (!pyr_in<WIN>(pw, e1, c1) || !pyr_in<WIN>(pw, e2, c2)) continue;
                    const int64_t cc = self_i + (int64_t)o1 * s1 * ls[e1] + (int64_t)o2 * s2 * ls[e2];
                    L = min(L, (int32_t)((__ldg(lev + cc) >> (4 * o)) & 15u));
                }
                L = max(L, K);
            }
            packed |= (uint32_t)L << (4 * o);
        }
        lng[(uint64_t)a * bricks + b] = packed;
    }
}

static unsigned box_blocks(const BrickBox& b) {
    return (unsigned)(((uint64_t)b.nx * b.ny * b.nz + 255) / 256);
}

// The box grown by (gx, gy, gz) bricks on each side, clipped to the lattice.
static BrickBox grow(const BrickBox& b, int32_t gx, int32_t gy, int32_t gz, int32_t bx, int32_t by,
                     int32_t bz) {
    BrickBox r;
    r.x0 = max(b.x0 - gx, 0);
    r.y0 = max(b.y0 - gy, 0);
    r.z0 = max(b.z0 - gz, 0);
    r.nx = min(b.x0 + b.nx + gx, bx) - r.x0;
    r.ny = min(b.y0 + b.ny + gy, by) - r.y0;
    r.nz = min(b.z0 + b.nz + gz, bz) - r.z0;
    return r;
}

cudaError_t launch_brick_octants(const uint32_t* dir, uint8_t* tmp_x, uint16_t* tmp_y,
                                 uint32_t* oct, int32_t bx, int32_t by, int32_t bz,
                                 cudaStream_t stream, const BrickBox* changed,
                                 const uint32_t* occ) {
    // pass z at the bricks within reach of a change reads pass y up to 14 bricks away in z, which
    // reads pass x up to 14 away in y
    const int32_t R = (int32_t)kMaxOctantDistance - 1;
    const BrickBox all = {0, 0, 0, bx, by, bz};
    const BrickBox w = changed ? grow(*changed, R, R, R, bx, by, bz) : all;
    const BrickBox wy = grow(w, 0, 0, R, bx, by, bz), wx = grow(w, 0, R, R, bx, by, bz);
    brick_octant_x_kernel<<<box_blocks(wx), 256, 0, stream>>>(dir, tmp_x, bx, by, wx, occ);
    brick_octant_y_kernel<<<box_blocks(wy), 256, 0, stream>>>(tmp_x, tmp_y, bx, by, wy);
    brick_octant_z_kernel<<<box_blocks(w), 256, 0, stream>>>(tmp_y, oct, bx, by, bz, w);
    return cudaGetLastError();
}

// Index windows of the long-box passes after a change inside `changed`: long words within 15
// bricks of it; the pyramid's level 3 within 6 more (the long kernel reads level p up to
// K - 2^p <= 6 bricks across), level 2 within 4 more, level 1 within 2, level 0 and the runs
// within 1 (level p + 1 reads level p 2^p bricks across).
struct LongWindows {
    BrickBox w, wp[4];
};

static LongWindows long_windows(const BrickBox& changed, int32_t bx, int32_t by, int32_t bz);

size_t brick_long_scratch_words(const BrickBox* changed, int32_t bx, int32_t by, int32_t bz) {
    const uint64_t bricks = (uint64_t)bx * by * bz;
    if (!changed) return (size_t)(13 * bricks);
    const BrickBox& p0 = long_windows(*changed, bx, by, bz).wp[0];
    return (size_t)(bricks + 12ull * (uint64_t)p0.nx * p0.ny * p0.nz);
}

cudaError_t launch_brick_long(const uint32_t* dir, const uint32_t* oct, uint32_t* tmp,
                              uint32_t* lng, int32_t bx, int32_t by, int32_t bz,
                              cudaStream_t stream, const BrickBox* changed,
                              const uint32_t* occ) {
    // tmp: runs (1 word per brick), then the pyramid (12 words per brick of its index window)
    const uint64_t bricks = (uint64_t)bx * by * bz;
    uint32_t* run = tmp;
    uint32_t* pyr = tmp + bricks;
    const BrickBox all = {0, 0, 0, bx, by, bz};
    LongWindows L;
    if (changed) {
        L = long_windows(*changed, bx, by, bz);
    } else {
        L.w = all;
        for (int p = 0; p < 4; ++p) L.wp[p] = all;
    }
    brick_run_kernel<<<box_blocks(L.wp[0]), 256, 0, stream>>>(dir, run, bx, by, bz, L.wp[0], occ);
    for (int32_t p = 0; p < 4; ++p) {
        if (changed)
            brick_pyramid_kernel<true><<<box_blocks(L.wp[p]), 256, 0, stream>>>(
                run, pyr, p, bx, by, bz, L.wp[p], L.wp[0]);
        else
            brick_pyramid_kernel<false><<<box_blocks(L.wp[p]), 256, 0, stream>>>(
                run, pyr, p, bx, by, bz, L.wp[p], L.wp[0]);
    }
    if (changed)
        brick_long_kernel<true><<<box_blocks(L.w), 256, 0, stream>>>(oct, pyr, lng, bx, by, bz, L.w, L.wp[0]);
    else
        brick_long_kernel<false><<<box_blocks(L.w), 256, 0, stream>>>(oct, pyr, lng, bx, by, bz, L.w, L.wp[0]);
    return cudaGetLastError();
}

static LongWindows long_windows(const BrickBox& changed, int32_t bx, int32_t by, int32_t bz) {
    const int32_t R = (int32_t)kMaxOctantDistance;
    LongWindows L;
    L.w = grow(changed, R, R, R, bx, by, bz);
    L.wp[3] = grow(L.w, 6, 6, 6, bx, by, bz);
    L.wp[2] = grow(L.wp[3], 4, 4, 4, bx, by, bz);
    L.wp[1] = grow(L.wp[2], 2, 2, 2, bx, by, bz);
    L.wp[0] = grow(L.wp[1], 1, 1, 1, bx, by, bz);
    return L;
}

cudaError_t launch_brick_distance(const BuildScratch& s, uint32_t* dir, int32_t bx, int32_t by,
                                  int32_t bz, cudaStream_t stream, const BrickBox* changed,
                                  const uint32_t* occ) {
    // distances change only within kMaxBrickDistance of a change; each pass reads the previous
    // one up to that far along its axis
    const int32_t R = (int32_t)kMaxBrickDistance;
    const BrickBox all = {0, 0, 0, bx, by, bz};
    const BrickBox w = changed ? grow(*changed, R, R, R, bx, by, bz) : all;
    const BrickBox w1 = grow(w, 0, 0, R, bx, by, bz), w0 = grow(w, 0, R, R, bx, by, bz);
    brick_distance_kernel<0><<<box_blocks(w0), 256, 0, stream>>>(dir, nullptr, s.dist_a, bx, by, bz, w0, occ);
    brick_distance_kernel<1><<<box_blocks(w1), 256, 0, stream>>>(dir, s.dist_a, s.dist_b, bx, by, bz, w1, nullptr);
    brick_distance_kernel<2><<<box_blocks(w), 256, 0, stream>>>(dir, s.dist_b, nullptr, bx, by, bz, w, nullptr);
    return cudaGetLastError();
}

}  // namespace vt

// ---------------------------------------------------------------------------------------------
// Order conversion of dense input: z-fastest (src/voxel/rawchunk.rs:292, element (x, y, z) at
// z + nz * (y + ny * x)) to the x-fastest order the brick build reads.  Each y-plane is an
// nx x nz matrix stored row-major by x; 32 x 32 tiles are staged through shared memory so that
// both the reads (along z) and the writes (along x) are contiguous per warp.
// ---------------------------------------------------------------------------------------------
namespace vt {

template <typename T>
__global__ void __launch_bounds__(256) transpose_xz_kernel(const T* __restrict__ src,
                                                           T* __restrict__ dst, int32_t nx,
                                                           int32_t ny, int32_t nz) {
    __shared__ T tile[32][33];
    const int32_t z0 = blockIdx.x * 32, x0 = blockIdx.y * 32;
    const size_t y = blockIdx.z;
    const int32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
#pragma unroll
    for (int32_t r = ty; r < 32; r += 8) {
        const int32_t x = x0 + r, z = z0 + tx;
        if (x < nx && z < nz) tile[r][tx] = src[(size_t)z + (size_t)nz * (y + (size_t)ny * x)];
    }
    __syncthreads();
#pragma unroll
    for (int32_t r = ty; r < 32; r += 8) {
        const int32_t z = z0 + r, x = x0 + tx;
        if (x < nx && z < nz) dst[(size_t)x + (size_t)nx * (y + (size_t)ny * z)] = tile[tx][r];
    }
}

cudaError_t launch_transpose_xz(const void* src, void* dst, size_t elem, int32_t nx, int32_t ny,
                                int32_t nz, cudaStream_t stream) {
    const dim3 grid((nz + 31) / 32, (nx + 31) / 32, ny);
    if (elem == 1)
        transpose_xz_kernel<uint8_t><<<grid, 256, 0, stream>>>((const uint8_t*)src, (uint8_t*)dst,
                                                               nx, ny, nz);
    else
        transpose_xz_kernel<uint32_t><<<grid, 256, 0, stream>>>((const uint32_t*)src,
                                                                (uint32_t*)dst, nx, ny, nz);
    return cudaGetLastError();
}

}  // namespace vt
