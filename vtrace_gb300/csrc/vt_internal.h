// vt_internal.h — shared host-side declarations of libvtrace (not part of the C ABI).
#pragma once

#include <stdint.h>

#include <functional>
#include <string>

#include "vtrace.h"

namespace vt {

// Records `msg` as the calling thread's last error and returns `code`.
int32_t fail(int32_t code, const std::string& msg);
void clear_error();

int32_t gen_palette(uint32_t seed, uint32_t* pal);
int32_t gen_terrain(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t octaves,
                    float occupancy, uint8_t* vox);
int32_t gen_shapes(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint32_t count,
                   float rmin, float rmax, uint8_t* vox);
int32_t gen_cave(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, float occupancy,
                 uint8_t* vox);
int32_t gen_rays_uniform(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, uint64_t n,
                         vt_ray* rays);

}  // namespace vt
