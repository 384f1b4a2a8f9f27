/*
 * vtrace.h — C ABI of libvtrace, a GB300 (sm_103a) voxel ray-traversal engine.
 *
 * Two groups of entry points live here:
 *
 *  1. The seven symbols vtrace's Rust host binds over FFI (src/render.rs:110-128), with the same
 *     names, argument meaning and error convention, but headless: there is no window, no Vulkan and
 *     no swapchain; a frame is one CUDA launch into a device framebuffer.
 *
 *  2. New vt_* calls for the traversal hot path: grid creation (brick re-layout), ray-buffer
 *     tracing, per-pixel rendering with shading and hard shadows, batched multi-view rendering in
 *     one persistent kernel replayed from a CUDA graph, and a continuous-batching serving loop.
 *
 * Conventions
 *  - vt_* calls return int32 status codes (VT_OK == 0, negative on error); vt_last_error() gives a
 *    message for the calling thread's most recent failure.
 *  - Grids are identified by int32 ids >= 0 (like the texture ids add_texture returns).
 *  - Pointers documented as "device" are CUDA device pointers; "host" pointers are ordinary host
 *    memory (pinned memory makes the copies asynchronous and faster, but is not required).
 *  - `stream` parameters are cudaStream_t values passed as void*; NULL selects the library's own
 *    (non-blocking) stream, so a caller that wants the legacy default stream passes
 *    cudaStreamLegacy.  Calls that take a stream are asynchronous with respect to the host unless
 *    stated.
 *  - Voxel grids are x-fastest: index = x + nx * (y + ny * z), the layout the reference uploads
 *    with bufferRowLength = 0 (lib/memory.c:353-366).
 */
#ifndef VTRACE_H
#define VTRACE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define VT_OK 0
#define VT_EINVAL (-1)     /* bad argument (null pointer, zero or oversized dimension, bad id) */
#define VT_ENOMEM (-2)     /* device or host allocation failed, or an HBM budget is exhausted */
#define VT_ECUDA (-3)      /* a CUDA runtime call failed; vt_last_error() names it */
#define VT_ENOTFOUND (-4)  /* unknown grid / batch / request id */
#define VT_ETIMEDOUT (-5)  /* a bounded wait ran out */
#define VT_EBUSY (-6)      /* resource still referenced by in-flight work */
#define VT_ECANCELED (-7)  /* request cancelled or service stopped */
#define VT_ENOTREADY (-8)  /* request accepted but not finished yet */
#define VT_ELIMIT (-9)     /* a fixed capacity of this library was exceeded */

/* ---------------------------------------------------------------- records */

/* One traced ray's first hit, 16 bytes (one 128-bit store on the device).
 *  x, y, z        hit voxel (0xFFFF on a miss)
 *  palette_index  voxel value of the hit (u8 grids); 0 for RGBA8 grids and misses
 *  face           bits 0-2: entered face as its outward normal, VT_FACE_*; 0 when the ray starts
 *                 inside the hit voxel or misses.  Bits 3-7: VT_HIT_FLAG_* (bit 6 is reserved
 *                 and always 0; multi-axis ties are counted in vt_trace_stats.ties).
 *  t              ray parameter of the entered face plane, (plane - origin[a]) / dir[a]; 0 when the
 *                 origin lies in the hit voxel; +inf on a miss
 *  rgba           colour, little-endian R | G<<8 | B<<16 | A<<24: the voxel colour for
 *                 vt_trace_rays, the shaded colour for vt_render, VT_SKY_RGBA on a render miss */
typedef struct vt_hit {
    uint16_t x, y, z;
    uint8_t palette_index;
    uint8_t face;
    float t;
    uint32_t rgba;
} vt_hit;

#define VT_FACE_NONE 0
#define VT_FACE_POS_X 1
#define VT_FACE_NEG_X 2
#define VT_FACE_POS_Y 3
#define VT_FACE_NEG_Y 4
#define VT_FACE_POS_Z 5
#define VT_FACE_NEG_Z 6
#define VT_FACE_MASK 0x07u

#define VT_HIT_FLAG_SHADOW_RAY 0x08u /* a shadow ray was traced for this hit */
#define VT_HIT_FLAG_INVALID 0x10u    /* non-finite origin or direction: reported as a miss */
#define VT_HIT_FLAG_SHADOWED 0x20u   /* the shadow ray found an occupied voxel */
#define VT_HIT_FLAG_HIT 0x80u        /* an occupied voxel was found */

/* sRGB encoding of the reference's clear colour (0.53, 0.81, 0.92, 1) (lib/command.c:57-60). */
#define VT_SKY_RGBA 0xFFF6E8C0u

/* A ray in grid (voxel) coordinates: the grid occupies [0,nx] x [0,ny] x [0,nz]. 24 bytes. */
typedef struct vt_ray {
    float origin[3];
    float dir[3];
} vt_ray;

/* Pinhole camera in grid coordinates.  For pixel (px, py) with sub-pixel offset (jx, jy) in [0,1)
 * (0.5 without jitter) the primary ray is origin + t * normalize(forward + sx*right + sy*up) with
 * sx = (px + jx) * (2/width) - 1 and sy = 1 - (py + jy) * (2/height), evaluated in IEEE binary32
 * round-to-nearest in exactly that order.  `right` and `up` carry the tan(fov/2) and aspect
 * scaling; vt_camera_look_at fills them. */
typedef struct vt_camera {
    float origin[3];
    float forward[3];
    float right[3];
    float up[3];
    uint32_t width, height;
} vt_camera;

/* Directional light for vt_render.  `dir` points from the surface towards the light (unit length).
 * Shading: k = ambient + (1 - ambient) * max(n.L, 0) * visible, colour = floor(base * k + 0.5). */
typedef struct vt_light {
    float dir[3];
    float ambient;
    uint32_t shadows; /* nonzero: trace one hard-shadow ray per lit hit */
} vt_light;

typedef struct vt_grid_info {
    uint32_t nx, ny, nz;
    uint32_t bricks_x, bricks_y, bricks_z;
    uint64_t bricks_total;
    uint64_t bricks_nonempty;
    uint64_t voxels_occupied;
    uint64_t device_bytes; /* directory + masks + payloads + palette */
    uint32_t payload_format; /* VT_PAYLOAD_* */
    uint32_t slots;          /* brick slots in use (the masks vt_grid_download_bricks copies):
                                bricks_nonempty, plus slots vt_grid_update freed and not reused */
} vt_grid_info;

#define VT_PAYLOAD_U8 1    /* palette index per voxel + 256-entry RGBA8 palette */
#define VT_PAYLOAD_RGBA8 2 /* RGBA8 texel per voxel (the reference's add_texture format) */

/* Per-launch traversal counters gathered by the counting variant of the kernels. */
typedef struct vt_trace_stats {
    uint64_t rays;                /* primary + shadow rays traced */
    uint64_t shadow_rays;
    uint64_t hits;                /* primary rays that found an occupied voxel */
    uint64_t steps;               /* DDA loop iterations over all rays */
    uint64_t bricks_entered;      /* brick visits (directory lookups) over all rays */
    uint64_t nonempty_bricks_entered;
    uint64_t voxels_tested;       /* occupancy-bit tests inside non-empty bricks */
    uint64_t ties;                /* rays with an iteration that advanced two or three axes at
                                     once (an exact tie on a voxel edge or corner) */
} vt_trace_stats;

/* ---------------------------------------------------------------- library state */

/* Select the CUDA device and create the library's stream.  Optional: every other call initialises
 * the library on device 0 when needed.  Returns VT_OK or VT_ECUDA. */
int32_t vt_init(int32_t device);
/* Free every grid, batch and buffer and destroy the library's stream. */
void vt_shutdown(void);
/* Message for the calling thread's most recent failed call ("" if none). */
const char* vt_last_error(void);
/* ABI version: (major << 16) | minor. */
uint32_t vt_version(void);
/* Device the library runs on and its SM count; for sizing persistent launches. */
int32_t vt_device_info(int32_t* device, int32_t* sm_count, uint64_t* free_bytes, uint64_t* total_bytes);
/* The library's own stream (a cudaStream_t): the stream of calls given a NULL stream and of the
 * reference-compatible entry points.  Callers order their own work after the library's on it.
 * Initialises the library; NULL if that fails. */
void* vt_get_stream(void);

/* Launch shape of a tracing entry point.  persistent = 0: one thread per ray, rays packed in
 * 8 x 4 pixel tiles per warp.  persistent = 1: resident warps keep one ray per lane and refill
 * lanes whose rays have ended with new work once at least `refill_min` lanes are idle (1..32;
 * 32 = only when the whole warp is idle), with at most `blocks_per_sm` 256-thread blocks per SM
 * (0 = as many as fit).  VT_KERNEL_BATCH is always persistent; its refill_min 32 (the default)
 * hands warps whole 8 x 4 tile units traced to the end in each lane.  vtrace_gb300.autotune picks
 * them per workload. */
typedef struct vt_tuning {
    uint32_t refill_min;
    int32_t blocks_per_sm;
    uint32_t persistent;
    uint32_t wavefront; /* VT_KERNEL_RENDER tile launches: trace shadow rays in a second pass over
                           a compacted queue instead of in the primary ray's thread; with
                           persistent = 1: resident warps take whole 8 x 4 tiles and queue their
                           shadow rays per warp, tracing them 32 at a time.
                           VT_KERNEL_PATH: advance all paths one vertex at a time through ray
                           queues (the default; faster than either per-path form) */
    uint32_t tile_shape;  /* VT_KERNEL_RENDER fused tile launch and VT_KERNEL_BATCH work units
                             (batches created afterwards): the pixels of one warp, VT_TILE_* */
    uint32_t block_warps; /* VT_KERNEL_RENDER fused tile launch: warps per block, 1, 2, 4 or 8
                             (0 = 4); the block's warp tiles are arranged about twice as wide as
                             high */
} vt_tuning;

#define VT_TILE_8X4 0u  /* 8 pixels wide, 4 high (the default) */
#define VT_TILE_4X8 1u
#define VT_TILE_16X2 2u
#define VT_TILE_32X1 3u

#define VT_KERNEL_RENDER 1
#define VT_KERNEL_TRACE_RAYS 2
#define VT_KERNEL_BATCH 3
#define VT_KERNEL_PATH 4 /* vt_path_trace: wavefront = ray queues per path vertex; else
                            persistent = paths refilled per lane, else a thread per pixel */

int32_t vt_get_tuning(int32_t kernel, vt_tuning* out);
int32_t vt_set_tuning(int32_t kernel, const vt_tuning* in);

/* ---------------------------------------------------------------- grids */

/* Build a brick grid (8^3 bricks, 512-bit occupancy masks, dense payloads for occupied bricks)
 * from an x-fastest u8 palette-index grid and a 256-entry RGBA8 palette (both host memory).
 * A voxel is occupied iff its palette entry's alpha byte is nonzero, the reference's
 * `texture(...).w > 0.0` rule (shaders/trace.frag:78).  Returns a grid id >= 0 or an error. */
int32_t vt_grid_create_u8(const uint8_t* voxels, const uint32_t* palette,
                          uint32_t nx, uint32_t ny, uint32_t nz);
/* Same, with the voxel array already in device memory (x-fastest, nx*ny*nz bytes, left unchanged);
 * the palette is host memory.  The build runs on `stream`; the call returns after the build has
 * finished.  Device memory during any build of more than 512 bricks: besides the grid, about 75
 * bytes of scratch per brick and, when it fits, a staging buffer as large as the dense array
 * padded to whole bricks, released (to the stream-ordered pool) when the call returns; without
 * room for the staging buffer the build reads the dense array twice instead. */
int32_t vt_grid_create_u8_device(const uint8_t* d_voxels, const uint32_t* palette,
                                 uint32_t nx, uint32_t ny, uint32_t nz, void* stream);
/* Build a brick grid from an x-fastest RGBA8 texel array (host), the format of the reference's
 * add_texture (lib/memory.c:286-385).  Occupied iff alpha > 0. */
int32_t vt_grid_create_rgba8(const uint8_t* rgba, uint32_t nx, uint32_t ny, uint32_t nz);

/* Element orders of a dense input array. */
#define VT_ORDER_X_FASTEST 0u /* element (x, y, z) at x + nx*(y + ny*z): the order add_texture's
                                 buffer-to-image copy reads (lib/memory.c:353-366) */
#define VT_ORDER_Z_FASTEST 1u /* element (x, y, z) at z + nz*(y + ny*x): RawDynamicChunk::at
                                 (src/voxel/rawchunk.rs:292) and RawStaticChunk's [x][y][z]
                                 array (src/voxel/rawchunk.rs:19), the chunks the Rust host builds */
/* Build a grid from a dense host array of u8 palette indices (format VT_PAYLOAD_U8, palette of 256
 * RGBA8 required) or RGBA8 texels (VT_PAYLOAD_RGBA8, palette ignored) in either order: grid voxel
 * (x, y, z) is the input's element (x, y, z).  Z-fastest input is reordered on the device.  The
 * reference itself hands its z-fastest chunks to add_texture, whose copy reads them x-fastest
 * (the x and z axes of the rendered texture are the chunk's z and x): that behaviour is
 * add_texture's, and VT_ORDER_Z_FASTEST is the geometrically faithful reading. */
int32_t vt_grid_create(const void* voxels, uint32_t format, uint32_t order,
                       const uint32_t* palette, uint32_t nx, uint32_t ny, uint32_t nz);
int32_t vt_grid_destroy(int32_t grid);
/* Chunk paging (src/gen/pager.rs:52-78, one chunk per frame at src/render.rs:246-261): write a
 * w x h x d box of voxels (host memory, `order`; u8 palette indices for VT_PAYLOAD_U8 grids,
 * RGBA8 texels for VT_PAYLOAD_RGBA8 grids) into the grid at (x0, y0, z0), in place.  Bricks
 * that become occupied take freed or new slots (the slot arrays grow by doubling), bricks that
 * become empty give theirs back, and the empty-space distances are recomputed, so that the grid
 * traverses exactly as one built from the updated array.  Synchronous on the library stream; not
 * concurrent with launches that read the grid, nor with other calls on the same grid.
 * VT_EBUSY while a batch or a service references the grid. */
int32_t vt_grid_update(int32_t grid, const void* voxels, uint32_t order, uint32_t x0, uint32_t y0,
                       uint32_t z0, uint32_t w, uint32_t h, uint32_t d);
/* No counterpart in the reference.  Builds the brick layout of an x-fastest u8 grid into buffers
 * the caller owns, allocating nothing, for callers that cannot allocate device memory while they
 * run (a pager rebuilding chunks inside a real-time frame loop, where cudaMalloc/cudaFree would
 * synchronise the device; code recording into a captured stream; a fixed memory budget).
 * All pointers are device memory: d_voxels (nx*ny*nz bytes), d_palette (256 RGBA8),
 * d_directory (one u32 per brick), d_masks (8 u64 per brick) and d_payload (512 bytes per brick)
 * sized for every brick of the grid, and d_counts (2 u64: occupied bricks, occupied voxels).
 * Outputs have the layout of vt_grid_download_bricks; payload slot s holds voxel values at
 * lx + 8*(ly + 8*lz).  The build's scratch is a 2.5 MiB static device array: grids of at most
 * 32768 bricks (e.g. 256^3 voxels) are accepted, larger ones return VT_ELIMIT.  Every call
 * shares that array, so calls whose work overlaps on the GPU (different streams) race; serialise
 * them on one stream.  Asynchronous on `stream` (NULL = the legacy default stream); the first call
 * on each device looks up the array's device address and should come before any stream capture.
 * The address is kept per device for the runtime's primary context: call it from that context,
 * and call vt_shutdown before resetting the device (vt_shutdown forgets the address; the next
 * call looks it up again).
 * Returns VT_OK, VT_EINVAL (null or misaligned pointer, bad size), VT_ELIMIT or VT_ECUDA; it
 * does not set vt_last_error. */
int32_t vt_grid_build_u8_noalloc(const uint8_t* d_voxels, const uint32_t* d_palette,
                                 uint32_t nx, uint32_t ny, uint32_t nz, uint32_t* d_directory,
                                 uint64_t* d_masks, uint8_t* d_payload, uint64_t* d_counts,
                                 void* stream);
int32_t vt_grid_get_info(int32_t grid, vt_grid_info* info);
/* Copy the grid's brick directory and occupancy masks to host memory; either may be NULL.
 * directory: bricks_total u32, x-fastest over bricks; an occupied brick's entry is its slot
 * (bit 31 clear); an empty brick's entry is 0x80000000 | d, d = Chebyshev distance in bricks to
 * the nearest occupied brick (1..31, saturating).  masks: vt_grid_info.slots * 8 u64 by slot,
 * word lz holding bit (ly * 8 + lx) of z-slice lz. */
int32_t vt_grid_download_bricks(int32_t grid, uint32_t* directory, uint64_t* masks);
/* Copy the grid's forward-distance words (bricks_total u32): for a ray octant
 * o = (dx<0) | (dy<0)<<1 | (dz<0)<<2, nibble o holds the largest K <= 15 such that the K x K x K
 * bricks starting at the brick and extending along the octant's directions are all empty. */
int32_t vt_grid_download_octants(int32_t grid, uint32_t* octants);
/* Copy the grid's long-box words: 3 * bricks_total u32, axis-major (word a * bricks_total + brick
 * for axis a = x, y, z); nibble o (octant o = (sx<0) | (sy<0)<<1 | (sz<0)<<2) holds the largest
 * L <= 15 such that the box L bricks long along axis a and K x K across (K = the octant word's
 * nibble o), from the brick toward octant o, holds no occupied brick. */
int32_t vt_grid_download_long(int32_t grid, uint32_t* words);
/* Copy the grid's brick payloads: vt_grid_info.slots blocks of 512 voxels by slot, each x fastest,
 * then y, then z (one byte per voxel for VT_PAYLOAD_U8, four for VT_PAYLOAD_RGBA8), zero past the
 * grid's edge.  VT_EINVAL if capacity_bytes is smaller than slots * 512 * that size. */
int32_t vt_grid_download_payload(int32_t grid, void* payload, uint64_t capacity_bytes);

/* ---------------------------------------------------------------- tracing */

/* Trace n rays (device array) against a grid; writes n vt_hit records (device).  Hit colour is the
 * voxel's unshaded RGBA8, miss colour 0.  Asynchronous on `stream`. */
int32_t vt_trace_rays(int32_t grid, const vt_ray* d_rays, uint64_t n, vt_hit* d_hits, void* stream);
/* Same through host buffers: copies rays in, traces, copies hits out, and returns when done. */
int32_t vt_trace_rays_host(int32_t grid, const vt_ray* rays, uint64_t n, vt_hit* hits);

/* Render one image: one primary ray per pixel (pixel centres), first hit, face-normal Lambert
 * shading and, when light->shadows is set, one hard-shadow ray per lit hit.  light may be NULL
 * (unshaded voxel colour, no shadow rays).  Writes width*height records, row-major from the top
 * row (device).  Asynchronous on `stream`. */
int32_t vt_render(int32_t grid, const vt_camera* camera, const vt_light* light,
                  vt_hit* d_hits, void* stream);
/* Same through a host output buffer; returns when the records are in `hits`.  Page-locked
 * memory (cudaHostAlloc / cudaHostRegister, 16-byte aligned) is written by the render kernel
 * directly; other memory through a device staging buffer and copies. */
int32_t vt_render_host(int32_t grid, const vt_camera* camera, const vt_light* light, vt_hit* hits);
/* Counting variant of vt_render / vt_trace_rays: same records, plus traversal counters (a slower
 * kernel build; for roofline accounting, not for timing).  rays == NULL selects the render form. */
int32_t vt_render_stats(int32_t grid, const vt_camera* camera, const vt_light* light,
                        vt_hit* d_hits, vt_trace_stats* stats);
/* Distinct bricks a frame touches along the reference's iteration path (the counting kernel, not
 * timed): the conservative "unique footprint" of a launch, beside the per-ray byte counts of
 * vt_trace_stats. */
typedef struct vt_footprint {
    uint64_t bricks;          /* distinct bricks entered (directory entries read) */
    uint64_t nonempty_bricks; /* distinct occupied bricks entered (masks read) */
    uint64_t hit_bricks;      /* distinct bricks holding a hit voxel (payload read) */
    uint64_t reserved;
} vt_footprint;
int32_t vt_render_footprint(int32_t grid, const vt_camera* camera, const vt_light* light,
                            vt_hit* d_hits, vt_footprint* out);
/* Warp-time phase profile of one vt_render frame (a separate, slower build of the render kernel,
 * default 8x4-pixel warp tiles in 128-thread blocks; same records as vt_render).  At each
 * warp-synchronous point of the traversal the warp reads the SM clock and charges the cycles since
 * its previous point to a phase: its residency in each phase, load latency included (in an
 * issue-bound launch other warps issue meanwhile), not issue slots.  The clock reads add about a
 * third to the frame time. */
#define VT_PHASE_SETUP 0        /* ray set-up up to the first traversal pass (raygen or shadow
                                   origin, slab, DDA set-up; a warp with no pass charges its tail) */
#define VT_PHASE_LOOP 1         /* traversal loop top: inside test, directory load, kind ballot */
#define VT_PHASE_WALK 2         /* walks through occupied bricks */
#define VT_PHASE_CROSS_BOX 3    /* empty-box crossing: box, exit approximations, prefix estimates */
#define VT_PHASE_CROSS_CHAINS 4 /* empty-box crossing: chains of binary32 additions */
#define VT_PHASE_CROSS_FINISH 5 /* empty-box crossing: prefix walk-ups, exits, settles */
#define VT_PHASE_TAIL 6         /* hit record; after the shadow ray also shading and the store */
#define VT_PHASES 7
typedef struct vt_phase_profile {
    uint64_t warp_cycles[2][VT_PHASES]; /* [0 camera rays, 1 shadow rays][VT_PHASE_*] */
    uint64_t passes[2][2];              /* [camera, shadow][0 walk, 1 crossing] traversal passes */
    uint64_t warps;                     /* warps of the launch */
} vt_phase_profile;
int32_t vt_render_phases(int32_t grid, const vt_camera* camera, const vt_light* light,
                         vt_hit* d_hits, vt_phase_profile* out);
int32_t vt_trace_rays_stats(int32_t grid, const vt_ray* d_rays, uint64_t n, vt_hit* d_hits,
                            vt_trace_stats* stats);

/* Fill a vt_camera that looks from `eye` at `target` with world-up `up`, vertical field of view
 * `vfov_degrees`, and the given image size (computed in double, stored as float). */
int32_t vt_camera_look_at(const float eye[3], const float target[3], const float up[3],
                          float vfov_degrees, uint32_t width, uint32_t height, vt_camera* out);

/* ---------------------------------------------------------------- path tracing */

/* Multi-bounce diffuse path tracing on the same traversal (vtrace's stated goal, README.md:2; no
 * counterpart in the reference's code).  Per sample: a Philox-jittered camera ray; at every hit
 * the throughput takes the voxel colour (byte / 255), a next-event ray toward the sun adds
 * throughput * sun * n.l when unblocked, and the path continues along a cosine-weighted
 * direction about the face normal, for at most max_bounces bounces; rays leaving the grid add
 * throughput * sky.  Radiance is averaged over spp samples in sample order.  Deterministic for a
 * given seed and bit-identical to the library's CPU restatement. */
#define VT_PATH_OUT_F32X4 0u /* float4 (r, g, b, 1) per pixel, linear radiance */
#define VT_PATH_OUT_RGBA8 1u /* u32 per pixel: clamp(c, 0, 1) * 255 rounded half up, alpha 255 */
typedef struct vt_path_params {
    uint32_t spp;         /* samples per pixel, 1..65536 */
    uint32_t max_bounces; /* bounces after the camera ray's hit, 0..64 */
    uint32_t seed;
    uint32_t out_format;  /* VT_PATH_OUT_* */
    float sky[3];         /* radiance of rays that leave the grid */
    float sun_dir[3];     /* unit direction toward the sun */
    float sun[3];         /* sun irradiance; all zero: no next-event rays */
} vt_path_params;
/* d_out: width*height pixels of the chosen format (device, 16-byte aligned; width*height below
 * 2^32, else VT_ELIMIT).  d_rays_traced: NULL or a device u64 the launch adds the number of rays
 * it traced to. */
int32_t vt_path_trace(int32_t grid, const vt_camera* camera, const vt_path_params* params,
                      void* d_out, uint64_t* d_rays_traced, void* stream);
/* Synchronous, host output (written by the kernel directly when page-locked and 16-byte
 * aligned); rays_traced may be NULL. */
int32_t vt_path_trace_host(int32_t grid, const vt_camera* camera, const vt_path_params* params,
                           void* out, uint64_t* rays_traced);

/* ---------------------------------------------------------------- batched multi-view */

/* One view of a batch: a camera over a grid with `spp` jittered samples per pixel.  Sample s of
 * pixel (px, py) uses the sub-pixel offset Philox4x32-10(counter = {px, py, s, view_id},
 * key = {seed, 0x56544752}) words 0 and 1, each >> 8 and scaled by 2^-24, and is written to
 * d_out[(py * width + px) * spp + s] (device memory, or page-locked host memory that the kernel
 * writes over the host link; 16-byte aligned; width * height * spp below 2^32, else VT_ELIMIT;
 * other host memory is refused with VT_EINVAL).  The light is used when flags & VT_VIEW_LIGHT. */
typedef struct vt_view {
    int32_t grid;
    uint32_t spp;
    uint32_t seed;
    uint32_t view_id;
    uint32_t flags;
    vt_camera camera;
    vt_light light;
    vt_hit* d_out;
} vt_view;

#define VT_VIEW_LIGHT 1u

/* Build a batch of up to 256 views: one persistent work-stealing launch over all their samples
 * (uneven sizes are balanced by dynamic fetching), captured once into a CUDA graph.  The grids
 * stay referenced (vt_grid_destroy returns VT_EBUSY) until vt_batch_destroy.  The launch shape
 * is the VT_KERNEL_BATCH tuning at creation time. */
int32_t vt_batch_create(const vt_view* views, uint32_t n, int32_t* batch_out);
/* Replay the batch's graph on `stream` (asynchronous). */
int32_t vt_batch_run(int32_t batch, void* stream);
/* The same launch without the graph (for comparison and for streams that cannot take graphs). */
int32_t vt_batch_run_direct(int32_t batch, void* stream);
/* Primary rays (sum of width * height * spp) and work items of a batch. */
int32_t vt_batch_info(int32_t batch, uint64_t* primary_rays, uint64_t* work_items);
/* Counting run of a batch (no counterpart in the reference): the same records through a slower
 * kernel build that walks every reference iteration, plus its traversal counters (for roofline
 * accounting, not for timing).  Synchronous on the library stream. */
int32_t vt_batch_stats(int32_t batch, vt_trace_stats* stats);
int32_t vt_batch_destroy(int32_t batch);

/* ---------------------------------------------------------------- serving */

/* A continuous-batching render service: requests arrive from any thread and are split into pieces
 * of whole 4-row bands of at most max_samples_per_piece samples; a dispatcher thread keeps up to
 * max_inflight launches on the device (one stream each), packing the oldest pending pieces (up to
 * max_views_per_launch pieces / max_samples_per_launch samples) into one persistent work-stealing
 * launch as launch slots free up; each piece's samples are averaged into its rows of the request's
 * RGBA8 image in the caller's host buffer, and a request is done when its last piece is.  Scene
 * brick grids stay resident in a cache built on first use, least-recently-used unreferenced scenes
 * evicted.  hbm_budget_bytes bounds the resident grids plus the launch slots' sample buffers
 * (max_inflight x max_samples_per_launch x 20 bytes, allocated at start) plus the temporary buffer
 * of any piece larger than a slot's; a scene is admitted against the size its grid would have with
 * every brick occupied, then counted at its real size.  While a scene's grid is built the device
 * also holds its voxel array and the build's scratch for a moment; those are outside the budget.
 * max_inflight = 1, max_views_per_launch = 1 and max_samples_per_piece = 0 is the plain
 * per-request baseline. */
typedef struct vt_serve_config {
    uint64_t hbm_budget_bytes;
    uint32_t max_inflight;           /* concurrent launches, 1..32 */
    uint32_t max_views_per_launch;   /* 1..256 */
    uint64_t max_samples_per_launch; /* pack pieces up to this many samples per launch (1..2^32) */
    uint32_t poll_interval_us;       /* completion polling period of the dispatcher */
    uint32_t refill_min;             /* persistent-warp refill threshold of the launches */
    uint64_t max_samples_per_piece;  /* split requests into pieces of at most this many samples
                                        (whole 4-row bands, at least one); 0 = never split */
} vt_serve_config;

/* One render request.  The image is width*height RGBA8 (row-major from the top row): per pixel
 * and channel, (sum of the spp samples' colours + spp/2) / spp, samples jittered as in vt_view.
 * host_rgba must stay valid until the request is polled done (pinned memory avoids a staging
 * copy). */
typedef struct vt_serve_request {
    int32_t scene;
    uint32_t spp;
    uint32_t seed;
    uint32_t view_id;
    uint32_t flags; /* VT_VIEW_LIGHT */
    vt_camera camera;
    vt_light light;
    uint8_t* host_rgba;
} vt_serve_request;

typedef struct vt_serve_timing {
    int64_t submit_ns; /* steady clock at vt_serve_submit */
    int64_t launch_ns; /* when its launch was enqueued */
    int64_t done_ns;   /* when the dispatcher saw its image in host memory */
    uint64_t samples;
} vt_serve_timing;

typedef struct vt_serve_stats {
    uint64_t submitted, completed, launches, views_launched, samples;
    uint64_t scene_loads, evictions, resident_bytes, pending;
    uint64_t device_ns; /* summed device time of the finished launches (kernels, resolves and
                           copies, timed by events on their streams); with max_inflight 1 the
                           launches never overlap and this is the time the GPU was busy */
} vt_serve_stats;

int32_t vt_serve_default_config(vt_serve_config* cfg);
int32_t vt_serve_start(const vt_serve_config* cfg, int32_t* service_out);
/* Register a scene (x-fastest u8 voxels and palette in host memory, kept valid by the caller for
 * the life of the service: the cache rebuilds evicted scenes from it). */
int32_t vt_serve_add_scene(int32_t service, const uint8_t* voxels, const uint32_t* palette,
                           uint32_t nx, uint32_t ny, uint32_t nz, int32_t* scene_out);
/* Chunk paging into the scene cache (src/gen/pager.rs:52-78): the caller has changed the voxels of
 * the box (x0, y0, z0) + (w, h, d) of the scene's registered array; if the scene is resident, the
 * box is written into its grid in place (vt_grid_update), else the next build reads the array.
 * Pieces of the scene admitted after the call returns render the change (ones admitted while the
 * caller was changing the array, before the call, may render either state); the call waits until
 * the scene's pieces in flight have retired, and holds back new ones meanwhile (requests behind
 * them in arrival order wait too).  The grid's slot arrays may grow, past the budget for a
 * moment.  VT_EINVAL for an empty box or one outside the scene. */
int32_t vt_serve_update_scene(int32_t service, int32_t scene, uint32_t x0, uint32_t y0,
                              uint32_t z0, uint32_t w, uint32_t h, uint32_t d);
/* Queue a request (width * height * spp below 2^32, else VT_ELIMIT). */
int32_t vt_serve_submit(int32_t service, const vt_serve_request* req, uint64_t* request_id);
/* Wait up to timeout_us for a request: VT_OK (image written; the request is released),
 * VT_ENOTREADY, or the request's error (VT_ENOMEM when its scene exceeds the budget,
 * VT_ECANCELED when the service stopped first). */
int32_t vt_serve_poll(int32_t service, uint64_t request_id, uint32_t timeout_us,
                      vt_serve_timing* timing);
int32_t vt_serve_get_stats(int32_t service, vt_serve_stats* out);
/* Finish in-flight launches, cancel pending requests, free everything of the service (once no
 * other thread is inside a call on it).  Safe while other threads submit or poll: their calls
 * return VT_ECANCELED / VT_ENOTFOUND or the request's final status. */
int32_t vt_serve_stop(int32_t service);

/* ---------------------------------------------------------------- MagicaVoxel models (host) */

/* src/voxel/magica_voxel.rs:18-44 (dot_vox 4.1.0 for the file format).  `bytes` is a whole .vox
 * file in host memory; nothing is read from disk. */
typedef struct vt_vox_info {
    uint32_t version;     /* the file's version field (150, 200, ...) */
    uint32_t models;      /* SIZE + XYZI pairs, in file order */
    uint32_t has_palette; /* 1 if an RGBA chunk is present */
    uint32_t reserved;
} vt_vox_info;
typedef struct vt_vox_model {
    uint32_t size[3]; /* the model's SIZE chunk: x, y, z (MagicaVoxel's z points up) */
    uint32_t voxels;  /* voxels in its XYZI chunk */
} vt_vox_model;
int32_t vt_vox_inspect(const uint8_t* bytes, uint64_t size, vt_vox_info* info);
int32_t vt_vox_model_info(const uint8_t* bytes, uint64_t size, uint32_t model, vt_vox_model* out);
/* The texture load_magica_voxel builds from model `model`: a RawDynamicChunk<Color> of
 * (size.x, size.y, size.z) voxels, z-fastest (VT_ORDER_Z_FASTEST), 4 bytes per voxel, zero where
 * empty; voxel (x, y, z, c) lands at chunk coordinate (x, size.y - z - 1, y) with the RGBA chunk's
 * entry c - 1.  Pass it to add_texture(rgba, size.x, size.y, size.z) for what vtrace renders, or
 * to vt_grid_create(..., VT_ORDER_Z_FASTEST, ...) for the chunk's own geometry.  VT_EINVAL for a
 * malformed file, a file without an RGBA chunk, a voxel outside the chunk (where vtrace panics)
 * or a short buffer; VT_ENOTFOUND for a model index past the last model. */
int32_t vt_vox_model_chunk(const uint8_t* bytes, uint64_t size, uint32_t model, uint8_t* rgba,
                           uint64_t capacity_bytes);

/* ---------------------------------------------------------------- scene generators (host) */

/* Seeded synthetic content, deterministic across platforms (integer hashing and IEEE binary32
 * arithmetic without contraction).  All write x-fastest u8 palette indices (0 = empty). */
int32_t vt_gen_palette(uint32_t seed, uint32_t* palette256);
/* fBm-noise heightfield terrain, y up, `octaves` octaves, scaled to `occupancy` (0..1). */
int32_t vt_gen_terrain(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t octaves,
                       float occupancy, uint8_t* voxels);
/* `count` random axis-aligned boxes and spheres with radius in [rmin, rmax]. */
int32_t vt_gen_shapes(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t count,
                      float rmin, float rmax, uint8_t* voxels);
/* 3D gradient-noise cave: voxel solid where noise > threshold chosen for `occupancy`. */
int32_t vt_gen_cave(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, float occupancy,
                    uint8_t* voxels);
/* n rays with origins uniform inside [0,nx]x[0,ny]x[0,nz] and directions uniform on the sphere. */
int32_t vt_gen_rays_uniform(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint64_t n,
                            vt_ray* rays);

/* ---------------------------------------------------------------- reference-compatible ABI */

/* render_tick_info of lib/common.h:89-92: pointers to column-major float[16] matrices. */
typedef struct render_tick_info {
    void* perspective;
    void* camera;
} render_tick_info;

/* user_input of lib/common.h:145-151. */
typedef struct user_input {
    uint8_t keys[6];
    double mouse_x;
    double mouse_y;
    double last_mouse_x;
    double last_mouse_y;
} user_input;

/* lib/entry.c:54-57.  Initialise the headless renderer: CUDA device, stream and a 1000x1000
 * RGBA8 framebuffer (VTRACE_WIDTH / VTRACE_HEIGHT override the size).  Returns
 * ((uint64_t)cudaError << 32) | custom; 0 on success. */
uint64_t entry(void);
/* lib/entry.c:150-248.  Render every instance into the framebuffer with the given projection and
 * camera matrices and write the framebuffer size back.  Returns 0, or -1 on error. */
int32_t render_tick(int32_t* window_width, int32_t* window_height, const render_tick_info* info);
/* lib/entry.c:146-148.  There is no window: returns a zeroed, library-owned struct. */
user_input* get_input_data_pointer(void);
/* lib/memory.c:286-385.  Upload a width x height x depth RGBA8 texture (x-fastest, caller keeps
 * ownership) as a brick grid.  Returns the texture id >= 0, or -1. At most 65536 textures. */
int32_t add_texture(const uint8_t* data, uint32_t width, uint32_t height, uint32_t depth);
/* lib/memory.c:235-248.  Returns a host buffer for instance_count column-major mat4 instances
 * (64 B each, texture id stored as the bit pattern of element [3][3]); NULL on failure.
 * instance_count == 0 is treated as 1. */
float* start_update_instances(uint32_t instance_count);
/* lib/memory.c:250-267.  Publish the instances written since start_update_instances; they are
 * copied to the device at the next render_tick.  Returns 0, or -1. */
int32_t end_update_instances(uint32_t instance_count);
/* lib/entry.c:100-144.  Free everything entry() and later calls created. */
void cleanup(void);
/* Headless framebuffer readback (no counterpart in the reference, which presents to a window):
 * copies width*height RGBA8 pixels, row-major from the top row, into `rgba`. */
int32_t vt_framebuffer_download(uint8_t* rgba, uint64_t capacity_bytes);

#ifdef __cplusplus
}
#endif

#endif /* VTRACE_H */
