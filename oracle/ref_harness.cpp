/*
 * ref_harness.cpp — drives vtrace's own fragment shader (shaders/trace.frag, compiled as C++
 * through glsl_compat.hpp) over a ray list (TEST INFRASTRUCTURE ONLY).
 *
 * With identity projection, camera and model matrices the shader's ray recovery
 * (trace.frag:48-66) reduces to ray_dir = normalize(screen_position.xyz) and
 * model_ray_pos = (model_position.xyz + 0.5) * size, so the harness can aim the reference DDA
 * (trace.frag:68-89) at any entry point and direction.  The shader only outputs a colour; the
 * compat sampler's side channel gives the texel fetched last (the hit voxel) and the number of
 * fetches (loop iterations + 1 on a hit, loop iterations on a miss).
 */
#include "glsl_compat.hpp"
#undef in
#undef out
#undef main
#undef uniform
#undef sampler3D
#undef layout
#undef flat
#undef discard

extern vec4 screen_position, world_position, model_position;
extern uint object_id, texture_id;
extern mat4 model_matrix;
struct PushConstants {
    mat4 projection;
    mat4 camera;
};
extern PushConstants push;
extern vec4 color, history_write;
extern float gl_FragDepth;
void trace_frag_main();

sampler3D_t tex[1];
bool glsl_discarded;

static mat4 identity4() {
    mat4 m;
    for (int i = 0; i < 4; ++i) m.c[i].e[i] = 1.0f;
    return m;
}

extern "C" {

/* Per ray i: model-space entry point mp[3*i..] in [-0.5,0.5]^3 and direction s[3*i..] (the
 * shader normalises it).  out[5*i..] = {hit, x, y, z, fetches}; colour[4*i..] = shader output. */
int vtref_trace(const uint8_t* rgba, int nx, int ny, int nz, uint64_t n, const float* mp,
                const float* s, int32_t* out, float* colour) {
    tex[0].texels = rgba;
    tex[0].nx = nx;
    tex[0].ny = ny;
    tex[0].nz = nz;
    push.projection = identity4();
    push.camera = identity4();
    model_matrix = identity4();
    texture_id = 0;
    object_id = 0;
    for (uint64_t i = 0; i < n; ++i) {
        screen_position = vec4(s[3 * i], s[3 * i + 1], s[3 * i + 2], 1.0f);
        model_position = vec4(mp[3 * i], mp[3 * i + 1], mp[3 * i + 2], 1.0f);
        world_position = model_position;
        tex[0].fetches = 0;
        tex[0].last_x = tex[0].last_y = tex[0].last_z = -1;
        glsl_discarded = false;
        color = vec4(0.f, 0.f, 0.f, 0.f);
        trace_frag_main();
        int32_t* o = out + 5 * i;
        o[0] = glsl_discarded ? 0 : 1;
        o[1] = tex[0].last_x;
        o[2] = tex[0].last_y;
        o[3] = tex[0].last_z;
        o[4] = (int32_t)tex[0].fetches;
        if (colour) {
            for (int c = 0; c < 4; ++c) colour[4 * i + c] = glsl_discarded ? 0.f : color.e[c];
        }
    }
    return 0;
}

int vtref_b2f_select(void) { return VT_B2F_SELECT; }
}
