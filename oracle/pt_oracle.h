/*
 * pt_oracle.h -- C API of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This is a scalar CPU restatement of
 * hala-pathtracer's per-pixel integrator (shaders/src/hala-pathtracer/
 * pathtracer.rgen.glsl and everything it calls). The test suite, the smoke
 * check and the benchmark's CPU-baseline leg use it as the checker. The
 * product library (libhalapt) never links, loads or calls it.
 *
 * Scene data uses the structs of include/hala_pt.h (the boundary's data
 * contract), so one scene description feeds both sides.
 */
#ifndef PT_ORACLE_H
#define PT_ORACLE_H

#include "../include/hala_pt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_ctx or_ctx;

or_ctx* or_create(const pt_tracer_config* cfg);
void or_destroy(or_ctx* c);
int or_set_scene(or_ctx* c, const pt_scene_desc* scene);
int or_set_envmap(or_ctx* c, const float* rgb, uint32_t w, uint32_t h, float rotation_degrees);
void or_set_ground_color(or_ctx* c, const float rgba[4]);
void or_set_sky_color(or_ctx* c, const float rgba[4]);
void or_set_env_intensity(or_ctx* c, float v);
void or_set_exposure_value(or_ctx* c, float v);
void or_set_camera_index(or_ctx* c, uint32_t i);
/* The camera jitter's blue-noise texture: 1024 x 1024 RGBA8 texels, row 0
 * first (load_blue_noise_texture); NULL returns to the substitute table. */
void or_set_blue_noise(or_ctx* c, const uint8_t* rgba8);
/* Builds the BVH and the environment alias tables; picks the feature set. */
int or_commit(or_ctx* c);
uint32_t or_features(const or_ctx* c);

/* Progressive render of `frames` frames over every pixel, running mean in
 * FP32 exactly as pathtracer.rgen.glsl:259-304. threads <= 0: all cores. */
int or_render(or_ctx* c, uint32_t frames, int threads);
/* Same frames, but radiance accumulated as an FP64 sum (the converged
 * reference); or_read_image(PT_IMAGE_ACCUM) then returns sum / count. */
int or_render_fp64(or_ctx* c, uint32_t frames, int threads);
void or_reset(or_ctx* c);
/* which: PT_IMAGE_ACCUM/ALBEDO/NORMAL (RGBA32F) or PT_IMAGE_FINAL (RGBA8). */
int or_read_image(or_ctx* c, int which, void* out, size_t bytes);

/* Per-path outputs for a pixel list: frames [first_frame, first_frame+nframes),
 * radiance_out[(f * npix + k) * 3 + c], hash_out[f * npix + k]. Does not
 * touch the accumulation images. */
int or_trace_paths(or_ctx* c, uint32_t first_frame, uint32_t nframes, const uint32_t* pixels,
                   uint32_t npix, float* radiance_out, uint32_t* hash_out, int threads);

/* Geometry queries with the same ray/hit layout as pt_renderer_trace_rays. */
// Every ray one path traces: origin xyz, tmin, direction xyz, tmax, kind
// (0 closest, 1 any-hit), result bits (hit id / occluded), t; 11 floats each.
int or_trace_path_rays(or_ctx* c, uint32_t pixel, uint32_t frame, float* out, uint32_t cap, uint32_t* count);
// Paths traced against every triangle (1) instead of the BVH (0, the default).
void or_set_brute(or_ctx* c, int brute);
int or_trace_rays(or_ctx* c, const float* rays, uint32_t n, int any_hit, int brute_force,
                  uint32_t* hits, int threads);

/* Counters of the last or_render / or_trace_paths call. */
void or_counters(const or_ctx* c, uint64_t* paths, uint64_t* closest_rays, uint64_t* shadow_rays);

/* ---- unit-level known-answer entry points ------------------------------ */
void or_pcg4d(uint32_t v[4]);
/* n draws of rand() from a state seeded like rng_initialize(pixel, frame). */
void or_rand_seq(uint32_t px, uint32_t py, uint32_t frame, uint32_t n, float* out);
/* Blue-noise substitute texel (RGBA in [0,1]). */
void or_blue_noise(uint32_t x, uint32_t y, float out[4]);
/* BSDF evaluation in world space. kind: 0 diffuse dispatch, 1 Disney.
 * frame: T,B,N (9 floats). state_eta / depth / any_non_specular as in State.
 * Returns f (3 floats) and pdf. */
void or_bsdf_eval(int kind, const pt_material* m, const float tbn[9], float eta, uint32_t depth,
                  int any_non_specular, const float V[3], const float N[3], const float L[3],
                  float f_out[3], float* pdf_out);
/* BSDF sample with an RNG state s0 (4 words, updated). */
void or_bsdf_sample(int kind, const pt_material* m, const float tbn[9], float eta, uint32_t depth,
                    int any_non_specular, const float V[3], const float N[3], uint32_t s0[4],
                    float f_out[3], float L_out[3], float* pdf_out, uint32_t* flags_out);
/* Portable float32 math of the oracle (oracle/pmath.h), for accuracy tests:
 * fn 0 sin, 1 cos, 2 tan, 3 exp, 4 log, 5 pow(x, y), 6 acos, 7 atan2(y=x[i], x=y[i]). */
void or_pmath(int fn, const float* x, const float* y, float* out, uint32_t n);
/* Tonemap + exposure + sRGB of one linear colour (pathtracer.rgen.glsl:280-301). */
void or_tonemap(const float in[3], float ev, int enable, int aces, int simple, float out[3]);

#ifdef __cplusplus
}
#endif

#endif
