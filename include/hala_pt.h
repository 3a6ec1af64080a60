/*
 * hala_pt.h -- C ABI of the GB300 wavefront path tracer.
 *
 * This header is the drop-in boundary for the per-pixel path-tracing
 * integrator of hala-pathtracer. The reference drives its integrator through
 * the `HalaRenderer` operator surface (crate hala-renderer, called from
 * src/bin/hala-pathtracer.rs); every entry point below names the call it
 * replaces. The GLSL-side data contract (Camera, Light, Medium, Material,
 * Vertex, Primitive) is mirrored field by field from
 * shaders/src/hala-pathtracer/inc/types.glsl so that a host which already
 * fills those buffers can fill these structs unchanged.
 *
 * Conventions
 *   - Plain C types only; no CUDA or torch types cross this boundary.
 *   - The library owns all device memory behind opaque handles. Host arrays
 *     passed in are copied before the call returns.
 *   - Every call returns a pt_status. On failure the per-handle last-error
 *     string (pt_renderer_last_error) says why. No call aborts the process.
 *   - One host thread at a time per pt_renderer.
 */
#ifndef HALA_PT_H
#define HALA_PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_ABI_VERSION 1u

/* Limits and constants, shaders/src/hala-pathtracer/inc/constants.glsl:1-6 */
#define PT_MAX_CAMERAS 8u
#define PT_MAX_LIGHTS 16u
#define PT_INVALID_INDEX 0xFFFFFFFFu
/* side of the blue-noise texture the camera jitter reads (wltcRS.glsl:43-53) */
#define PT_BLUE_NOISE_SIZE 1024u

/* Light types, constants.glsl:14-18 */
#define PT_LIGHT_POINT 0
#define PT_LIGHT_DIRECTIONAL 1
#define PT_LIGHT_SPOT 2
#define PT_LIGHT_QUAD 3
#define PT_LIGHT_SPHERE 4

/* Medium types, constants.glsl:41-44 */
#define PT_MEDIUM_NONE 0u
#define PT_MEDIUM_ABSORB 1u
#define PT_MEDIUM_SCATTER 2u
#define PT_MEDIUM_EMISSIVE 3u

/* Material types: callable order src/bin/hala-pathtracer.rs:182-185 */
#define PT_MATERIAL_DIFFUSE 0u
#define PT_MATERIAL_DISNEY 1u

/* Camera types, inc/types.glsl:10 */
#define PT_CAMERA_PERSPECTIVE 0u
#define PT_CAMERA_ORTHOGRAPHIC 1u

typedef enum pt_status {
  PT_OK = 0,
  PT_ERR_INVALID_ARG = 1,
  PT_ERR_OOM = 2,
  PT_ERR_CUDA = 3,
  PT_ERR_TIMEOUT = 4,
  PT_ERR_NOT_READY = 5,
  PT_ERR_UNSUPPORTED = 6,
  PT_ERR_STATE = 7,
  PT_ERR_CANCELLED = 8,
  PT_ERR_TRAVERSAL = 9  /* a BVH traversal ran out of stack or hit its visit cap: the
                           images of that call may be wrong (no reference counterpart:
                           RT-core traversal has no such limit) */
} pt_status;

/* Camera, inc/types.glsl:2-11. `type` 0 = perspective, 1 = orthographic. */
typedef struct pt_camera {
  float position[3];
  float right[3];
  float up[3];
  float forward[3];
  float yfov;                    /* radians */
  float focal_distance_or_xmag;  /* focal distance (perspective) / xmag (orthographic) */
  float aperture_or_ymag;        /* aperture (perspective) / ymag (orthographic) */
  uint32_t type;
} pt_camera;

/* Light, inc/types.glsl:14-39. Field meaning per light type is the same. */
typedef struct pt_light {
  float intensity[3];
  float position[3];
  float u[3];
  float v[3];
  float radius;
  float area;
  int32_t type;
} pt_light;

/* Medium, inc/types.glsl:42-49 */
typedef struct pt_medium {
  float color[3];
  float density;
  float anisotropy;
  uint32_t type;
} pt_medium;

/* Material, inc/types.glsl:52-83. `ax`/`ay` are the preprocessed values the
 * shaders read: GGX alphas for Disney, Oren-Nayar A/B for diffuse. Use
 * pt_material_preprocess() to derive them from roughness/anisotropic. */
typedef struct pt_material {
  pt_medium medium;
  float base_color[3];
  float opacity;
  float emission[3];
  float anisotropic;
  float metallic;
  float roughness;
  float subsurface;
  float specular_tint;
  float sheen;
  float sheen_tint;
  float clearcoat;
  float clearcoat_roughness;
  float clearcoat_tint[3];
  float specular_transmission;
  float ior;
  float ax;
  float ay;
  uint32_t base_color_map_index;
  uint32_t normal_map_index;
  uint32_t metallic_roughness_map_index;
  uint32_t emission_map_index;
  uint32_t type;
} pt_material;

/* One mesh primitive, inc/types.glsl:86-110 (Vertex + Primitive).
 * `vertices` holds 11 floats per vertex in the Vertex order:
 * position xyz, normal xyz, tangent xyz, tex_coord xy.
 * `transform` is a column-major 4x4 object-to-world matrix (GLSL mat4). */
typedef struct pt_primitive {
  const float* vertices;
  uint32_t num_vertices;
  const uint32_t* indices;
  uint32_t num_indices;
  float transform[16];
  uint32_t material_index;
} pt_primitive;

/* RGBA32F texture for the material maps (bindless set 2, inc/global.glsl:48). */
typedef struct pt_texture {
  const float* rgba;
  uint32_t width;
  uint32_t height;
} pt_texture;

/* The CPU scene handed to set_scene (HalaScene in the reference). */
typedef struct pt_scene_desc {
  const pt_primitive* primitives;
  uint32_t num_primitives;
  const pt_material* materials;
  uint32_t num_materials;
  const pt_light* lights;
  uint32_t num_lights;
  const pt_camera* cameras;
  uint32_t num_cameras;
  const pt_texture* textures;
  uint32_t num_textures;
} pt_scene_desc;

/* Tracer configuration: the arguments of HalaRenderer::new,
 * src/bin/hala-pathtracer.rs:128-138, plus the output size (window size in
 * the reference, src/config/window.rs:5-9) and an RNG seed offset.
 * `seed` is added to the frame index when the per-pixel RNG is seeded
 * (common/wltcRS.glsl:9-19); 0 reproduces the reference exactly. */
typedef struct pt_tracer_config {
  uint32_t width;
  uint32_t height;
  uint32_t max_depth;
  uint32_t rr_depth;
  int32_t enable_tonemap;
  int32_t enable_aces;
  int32_t use_simple_aces;
  uint32_t seed;
  uint64_t max_samples;   /* 0 = unlimited */
  uint32_t wave_paths;    /* paths in flight per wavefront; 0 = as many as half the free device
                             memory holds at the first render, at most 1 << 27 (about 35 GB),
                             halved again while the allocation fails */
  uint32_t keep_samples;  /* 1 = keep per-path radiance and hit-sequence hash of the last render call */
} pt_tracer_config;

typedef enum pt_image {
  PT_IMAGE_ACCUM = 0,        /* RGBA32F running mean of radiance (g_accum_image) */
  PT_IMAGE_ALBEDO = 1,       /* RGBA32F running mean of first-hit albedo (g_albedo_image) */
  PT_IMAGE_NORMAL = 2,       /* RGBA32F running mean of first-hit normal (g_normal_image) */
  PT_IMAGE_FINAL = 3,        /* RGBA8 exposure + tonemap + sRGB (g_final_image) */
  PT_IMAGE_SAMPLE_RADIANCE = 4, /* float3 per path of the last render call (keep_samples) */
  PT_IMAGE_SAMPLE_HASH = 5      /* uint32 hit-sequence hash per path (keep_samples) */
} pt_image;

typedef struct pt_stats {
  uint64_t frame_index;      /* frames accumulated so far */
  uint64_t paths;            /* paths traced by the last render call */
  uint64_t closest_rays;     /* closest-hit rays traced by the last render call */
  uint64_t shadow_rays;      /* shadow / transmittance rays traced by the last render call */
  double render_ms;          /* device time of the last render call (CUDA events) */
  double trace_ms;           /* device time spent in the closest-hit kernel, last call */
  double bvh_build_ms;       /* device time of the last BVH build */
  uint64_t bvh_nodes;
  uint64_t triangles;
  uint32_t features;         /* PT_FEATURE_* chosen at commit */
  uint32_t max_bounces_seen;
  uint64_t trace_launches;   /* closest-hit kernel launches timed in the last render call */
  uint64_t trav_nodes;       /* BVH nodes visited by closest-hit rays (PT_PROFILE_COUNT) */
  uint64_t trav_tris;        /* triangle tests of closest-hit rays (PT_PROFILE_COUNT) */
  uint64_t kernel_launches;  /* kernels launched by the last render call */
  uint64_t cache_queries;        /* paths ended in the radiance cache, last render call */
  uint64_t cache_train_samples;  /* training samples gathered, last render call */
  uint64_t cache_train_steps;    /* optimiser steps, last render call */
  double cache_loss;             /* loss of the last training batch */
  uint64_t wave_paths;           /* wavefront capacity (paths) of the last render call */
  uint64_t bvh_binary_nodes;     /* nodes of the binary tree (2 x leaves - 1) before the 4-wide collapse */
} pt_stats;

/* Profiling switches for pt_renderer_set_profiling. */
#define PT_PROFILE_TRACE_TIMING 1u  /* CUDA events around every closest-hit launch */
#define PT_PROFILE_COUNT 2u         /* count traversal work (slower counting kernels) */
/* Any flag above, or this one, drives the bounce loop from the host (one
 * read-back of the live-path count per bounce) instead of launching each
 * wave's bounces as one CUDA graph; the images are the same either way. */
#define PT_PROFILE_HOST_LOOP 4u

#define PT_FEATURE_MEDIUM 1u
#define PT_FEATURE_VOL_MIS 2u
#define PT_FEATURE_TRANSPARENT 4u
#define PT_FEATURE_TEXTURED 8u  /* some material uses a texture map */

typedef struct pt_renderer pt_renderer;

/* ---- renderer lifecycle: HalaRenderer operator surface -------------------- */

/* HalaRenderer::new (src/bin/hala-pathtracer.rs:128-138). */
pt_status pt_renderer_create(const pt_tracer_config* config, pt_renderer** out);
/* Drop of HalaRenderer after wait_idle (src/bin/hala-pathtracer.rs:226-230). */
void pt_renderer_destroy(pt_renderer* r);
/* anyhow error text of the last failed call on this handle. */
const char* pt_renderer_last_error(const pt_renderer* r);

/* HalaRenderer::set_scene (src/bin/hala-pathtracer.rs:198): uploads geometry,
 * materials, lights and cameras. The BVH is built on the device at commit. */
pt_status pt_renderer_set_scene(pt_renderer* r, const pt_scene_desc* scene);
/* HalaScene::new(scene_file) + HalaRenderer::set_scene
 * (src/bin/hala-pathtracer.rs:97-99, :198) with the file itself: reads a
 * glTF 2.0 scene with pt_gltf_load and calls pt_renderer_set_scene with it.
 * Unreadable or malformed files return PT_ERR_INVALID_ARG with the reason. */
pt_status pt_renderer_set_scene_file(pt_renderer* r, const char* path);
/* HalaRenderer::set_envmap (src/bin/hala-pathtracer.rs:203): equirectangular
 * RGB32F pixels (row 0 = theta 0) and the hdri_rotation in degrees. */
pt_status pt_renderer_set_envmap(pt_renderer* r, const float* rgb, uint32_t width,
                                 uint32_t height, float rotation_degrees);
/* HalaRenderer::set_envmap(&hdri_file, rotation) (src/bin/hala-pathtracer.rs:203)
 * with the file itself: reads an OpenEXR image (single-part scanline; HALF,
 * FLOAT or UINT channels; NONE, RLE, ZIPS or ZIP compression; R, G, B or a
 * single Y channel) and calls pt_renderer_set_envmap with its pixels. NULL
 * clears the map like pt_renderer_set_envmap(r, NULL, ...). Unsupported or
 * corrupt files return PT_ERR_INVALID_ARG with the reason. */
pt_status pt_renderer_set_envmap_file(pt_renderer* r, const char* path, float rotation_degrees);
/* The OpenEXR reader behind pt_renderer_set_envmap_file: RGB float triples,
 * row 0 at the top. With rgb = NULL only *width and *height are set;
 * otherwise rgb must hold width * height * 3 floats. No counterpart in the
 * reference (its exr crate dependency, Cargo.lock:502-504). */
pt_status pt_exr_read_rgb(const char* path, float* rgb, size_t capacity_floats, uint32_t* width,
                          uint32_t* height, char* error_message, size_t error_capacity);
/* ---- glTF 2.0 scene files --------------------------------------------------
 * The reader behind pt_renderer_set_scene_file, for hosts that keep a scene
 * on the CPU (job server submissions, several renderers): .gltf with external
 * or data-URI buffers, or .glb. Every TRIANGLES primitive of the default
 * scene's mesh nodes (world matrix as the primitive transform; smooth normals
 * and orthogonal tangents where the file has none), pbrMetallicRoughness
 * materials with the emissive-strength, ior, transmission and clearcoat
 * extensions and the renderer's material `extras` (any pt_material field by
 * name, "type", "medium"), PNG textures baked as factor x texel,
 * KHR_lights_punctual lights with the rectangle / sphere area-light extras
 * {type, param0, param1}, perspective and orthographic cameras. The
 * reference's own reader is the `gltf` crate (1.4.1) inside its renderer
 * crate; this mapping is the library's. */
typedef struct pt_gltf_scene pt_gltf_scene;
pt_status pt_gltf_load(const char* path, pt_gltf_scene** out, char* error_message, size_t error_capacity);
/* The scene in pt_renderer_set_scene's form; its arrays live until pt_gltf_free. */
const pt_scene_desc* pt_gltf_scene_desc(const pt_gltf_scene* scene);
/* Images the reader left out (not PNG): the maps that named them stay unset. */
uint32_t pt_gltf_skipped_images(const pt_gltf_scene* scene);
void pt_gltf_free(pt_gltf_scene* scene);
/* HalaRenderer::load_blue_noise_texture (src/bin/hala-pathtracer.rs:195): the
 * RGBA8 texture the camera rays' jitter reads (rand4blue, wltcRS.glsl:43-53:
 * texel ((pixel + shift) % 1024), channels / 255). An 8-bit or palette PNG of
 * at least 1024 x 1024; its top-left 1024 x 1024 texels are used. Until one is
 * loaded, and after a NULL path, a deterministic substitute table is read
 * (the reference's assets/textures/blue_noise.png is not in its checkout).
 * Takes effect at the next render; no new commit is needed. */
pt_status pt_renderer_load_blue_noise_texture(pt_renderer* r, const char* path);
/* The same with texels the host decoded: PT_BLUE_NOISE_SIZE^2 RGBA8 texels,
 * row-major, row 0 first; NULL returns to the substitute. */
pt_status pt_renderer_set_blue_noise(pt_renderer* r, const uint8_t* rgba8);
/* The PNG reader behind pt_renderer_load_blue_noise_texture: RGBA8 bytes of an
 * 8-bit or palette PNG (grey and RGB get alpha 255), row 0 at the top. With
 * rgba = NULL only *width and *height are set. */
pt_status pt_png_read_rgba8(const char* path, uint8_t* rgba, size_t capacity_bytes, uint32_t* width,
                            uint32_t* height, char* error_message, size_t error_capacity);
/* HalaRenderer::set_ground_color / set_sky_color (src/bin/hala-pathtracer.rs:205-206). */
pt_status pt_renderer_set_ground_color(pt_renderer* r, const float rgba[4]);
pt_status pt_renderer_set_sky_color(pt_renderer* r, const float rgba[4]);
/* HalaRenderer::set_env_intensity (src/bin/hala-pathtracer.rs:208). */
pt_status pt_renderer_set_env_intensity(pt_renderer* r, float intensity);
/* HalaRenderer::set_exposure_value (src/bin/hala-pathtracer.rs:211). */
pt_status pt_renderer_set_exposure_value(pt_renderer* r, float ev);
/* MainUBO.camera_index (inc/global.glsl:16). */
pt_status pt_renderer_set_camera_index(pt_renderer* r, uint32_t index);
/* HalaRenderer::commit (src/bin/hala-pathtracer.rs:213): picks the feature
 * permutation (src/bin/hala-pathtracer.rs:101-114), builds the BVH on the
 * device and the environment alias tables. */
pt_status pt_renderer_commit(pt_renderer* r);
/* HalaRenderer::update + render (src/bin/hala-pathtracer.rs:264-285):
 * traces `frames` progressive frames of one sample per pixel each and
 * accumulates them (pathtracer.rgen.glsl:259-304). Stops at max_samples. */
pt_status pt_renderer_render(pt_renderer* r, uint32_t frames);
/* Restart accumulation at frame 0. */
pt_status pt_renderer_reset(pt_renderer* r);
/* Resumes a progressive render from saved accumulation: the accum, albedo
 * and normal images as pt_renderer_read_image returns them (RGBA32F,
 * width * height each) and the number of frames they hold
 * (pt_stats.frame_index). The random sequence of a pixel depends only on the
 * pixel and the frame, so frames rendered afterwards continue exactly where
 * the saved render stopped: the result is bit-identical to an uninterrupted
 * render. The final image is recomputed from accum. The three pointers may
 * be host memory or device memory of the renderer's device. No counterpart in
 * the reference, whose accumulation lives only in GPU images. */
pt_status pt_renderer_load_accumulation(pt_renderer* r, const float* accum, const float* albedo,
                                        const float* normal, uint64_t frame_index);
/* Copy of one image (the data HalaRenderer::save_images writes,
 * src/bin/hala-pathtracer.rs:251). `bytes` must equal the image size. For the
 * accum, albedo, normal and final images `host` may also be device memory of
 * the renderer's device (the copy direction follows unified addressing). */
pt_status pt_renderer_read_image(pt_renderer* r, pt_image which, void* host, size_t bytes);
/* HalaRenderer::save_images (src/bin/hala-pathtracer.rs:251): writes
 * <prefix>_color.pfm, <prefix>_albedo.pfm, <prefix>_normal.pfm (the files
 * denoise.py:11-19 expects) and <prefix>_final.ppm. */
pt_status pt_renderer_save_images(pt_renderer* r, const char* prefix);
/* HalaRenderer::wait_idle (src/bin/hala-pathtracer.rs:228). */
pt_status pt_renderer_wait_idle(pt_renderer* r);
pt_status pt_renderer_get_stats(const pt_renderer* r, pt_stats* out);
/* Turns the PT_PROFILE_* instrumentation on or off (off by default). No
 * counterpart in the reference, which has no GPU timers. */
pt_status pt_renderer_set_profiling(pt_renderer* r, uint32_t flags);
/* The CUDA stream (cudaStream_t) the renderer launches on, for event timing. */
pt_status pt_renderer_get_stream(const pt_renderer* r, void** stream);

/* ---- geometry queries on the committed scene ------------------------------
 * Replaces traceRayEXT (pathtracer.rgen.glsl:56-68 closest hit,
 * inc/lighting.glsl:119-130 shadow any-hit) for testing and external use.
 * rays: n x 8 floats (origin xyz, tmin, direction xyz, tmax).
 * hits: n x 4 words (t as float, u, v as float, id as uint32). id is the
 * global triangle index, 0x80000000|light for an analytic light,
 * 0xFFFFFFFF for a miss. For any_hit, only t/id are meaningful (id != miss
 * means occluded). brute_force = 1 tests every primitive (no BVH). */
pt_status pt_renderer_trace_rays(pt_renderer* r, const float* rays, uint32_t n,
                                 int32_t any_hit, int32_t brute_force, uint32_t* hits);

/* BVH builder used by the next pt_renderer_commit (no counterpart in the
 * reference, whose acceleration structures the Vulkan driver builds):
 * PT_BVH_BUILD_SAH (default) prices binned SAH planes at every node, the
 * tree that traces fastest; PT_BVH_BUILD_FAST builds a linear BVH over
 * Morton codes in a fixed number of passes, for geometry rebuilt every
 * frame. The images are the same either way (closest hits do not depend on
 * the tree); only the build and traversal times differ. */
#define PT_BVH_BUILD_SAH 0u
#define PT_BVH_BUILD_FAST 1u
pt_status pt_renderer_set_bvh_build(pt_renderer* r, uint32_t mode);

/* Wave tail (no counterpart in the reference): once at most `paths` paths
 * of a wavefront are still alive, their remaining bounces run as one kernel
 * launch, one thread carrying each path to its end, instead of one launch
 * chain per bounce whose time the slowest ray sets. 0 turns it off;
 * PT_TAIL_PATHS_AUTO (the default) picks 16384 when some material can
 * refract (a glass lobe) or the scene has media, whose long chains of
 * bounces keep one tail thread busy longest, else 65536. The bounce graph
 * switches at its grid sizes (4096 x 4^k
 * paths), so the threshold in effect there is the largest such size not
 * above `paths`. Images, ray counts and bounce counts are the same either
 * way (with a radiance cache attached, the cache's training samples are
 * gathered in another order, so its images agree to within its training
 * noise). The PT_PROFILE_TRACE_TIMING / PT_PROFILE_COUNT instrumentation
 * always uses the per-bounce launches. */
#define PT_TAIL_PATHS_AUTO 0xFFFFFFFFu
pt_status pt_renderer_set_tail_paths(pt_renderer* r, uint32_t paths);

/* Traversal limits of this renderer: stack entries per ray (1..96; 0 = 96)
 * and node visits per ray (0 = 2^22). A traversal that needs more stack than
 * `stack_entries` skips a subtree, and one that reaches `max_visits` stops;
 * either sets a device error word that the render call (or trace_rays) that
 * saw it turns into PT_ERR_TRAVERSAL. The defaults are never reached by a
 * tree the library builds; smaller values exist to exercise that report.
 * No counterpart in the reference (RT-core traversal has no user limits). */
pt_status pt_renderer_set_traversal_limits(pt_renderer* r, uint32_t stack_entries, uint32_t max_visits);

/* Per-path results of the last render call for selected paths, gathered on
 * the device (keep_samples must be on). paths: n indices k into that call's
 * paths (k = frame_local * width * height + pixel); radiance: 3 floats per
 * path; hash: the hit-sequence hash (either output may be NULL). The same
 * values PT_IMAGE_SAMPLE_RADIANCE / PT_IMAGE_SAMPLE_HASH return for those
 * paths, without copying all of them. No counterpart in the reference. */
pt_status pt_renderer_read_samples(pt_renderer* r, const uint64_t* paths, uint32_t n, float* radiance,
                                   uint32_t* hash);

/* ---- allocation-free BVH rebuild ------------------------------------------
 * No counterpart in the reference (its acceleration structures are built by
 * the Vulkan driver inside hala-renderer). Some callers may not call
 * cudaMalloc or cudaFree while they run -- engines that reserve all device
 * memory in their own pools at start-up and rebuild the BVH of animated
 * geometry every frame without touching the allocator. This entry point builds
 * the BVH of `num_triangles` world-space triangles into buffers the caller
 * owns, with the build's scratch in a fixed library-owned device array.
 *
 *   tri_v0/e1/e2    device float4[num_triangles]: first vertex and the two edge
 *                   vectors of each triangle (w ignored)
 *   nodes_out       device float4[4 * node_capacity], node_capacity >= 2 * n
 *   tri_sorted_out  device float4[3 * num_triangles]: triangles in leaf order
 *                   (v0 with the input index in w's bits, e1, e2)
 *   num_nodes_out   host: number of nodes written
 *   stream          cudaStream_t (NULL = default stream)
 *   error_message   optional host buffer for the reason of a failure
 *
 * Output layout: a binary tree, node 0 the root, 64 bytes (4 float4) per node:
 *   q0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)   child 0's box, x and y
 *   q1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)   child 1's box, x and y
 *   q2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)   both boxes, z
 *   q3 = (link0, link1, 0, 0) as int32: link >= 0 is an internal node index;
 *        link < 0 is a leaf of the triangles tri_sorted_out[start .. start +
 *        count), start = link & 0x03FFFFFF, count = (link >> 26) & 0x1F.
 * The boxes are widened by a few ulps so a slab test in float32 never misses
 * a triangle inside them. The tree is the one pt_renderer_commit builds for
 * the same triangles (same binned-SAH splits, same node count, same leaf
 * order); the renderer traverses its 4-wide collapse, which it builds itself,
 * so this output is for the caller's own traversal kernels (a pt_renderer
 * does not take an external BVH).
 *
 * Limits: at most PT_NOALLOC_MAX_TRIANGLES triangles (larger inputs return
 * PT_ERR_INVALID_ARG with that reason); the scratch (about 11.3 MB) stays
 * resident on every device that loads the library until the process exits.
 * It calls no cudaMalloc/cudaFree. The first call in a device's context looks
 * up the scratch array's device address (cudaGetSymbolAddress, repeated after
 * cudaDeviceReset gives the device a new context); make that first call
 * before any stream capture. The build runs level by level and reads each
 * level's task count back to the host: the call synchronises `stream` once per
 * tree level and returns when the build is complete. All calls share the one
 * array: calls that overlap on the GPU (other streams, other threads) race and
 * must be serialised. */
#define PT_NOALLOC_MAX_TRIANGLES 65536u
pt_status pt_bvh_build_noalloc(const void* tri_v0, const void* tri_e1, const void* tri_e2,
                               uint32_t num_triangles, void* nodes_out, uint32_t node_capacity,
                               void* tri_sorted_out, uint32_t* num_nodes_out, void* stream,
                               char* error_message, size_t error_capacity);

/* ---- job server: continuous batching of render jobs ------------------------
 * No counterpart in the reference, which renders one scene in one window
 * (src/bin/hala-pathtracer.rs:226-295). A job is one render of one scene --
 * what the reference does between set_scene and its last render() -- and the
 * server runs many at once: a scheduler thread admits queued jobs while their
 * estimated device memory fits the HBM budget and a job slot is free, keeps
 * each admitted job's scene, BVH and accumulators on the device, and packs the
 * paths of all admitted jobs with the same feature permutation into shared
 * wavefronts. Jobs join and leave at wavefront boundaries. A job's images do
 * not depend on which jobs it shared wavefronts with: they are bit-identical
 * to a pt_renderer render of the same scene and configuration.
 *
 * Thread safety: every pt_server_* call may come from any host thread. */
typedef struct pt_server pt_server;
typedef struct pt_cache_config pt_cache_config;

typedef struct pt_server_config {
  uint64_t hbm_budget_bytes; /* device bytes for admitted jobs; 0 = 80% of free memory at create */
  uint32_t max_jobs;         /* admitted (device-resident) jobs at most; 0 = 64 */
  uint32_t wave_paths;       /* shared wavefront capacity in paths; 0 = 1 << 25 */
  uint32_t quantum_paths;    /* paths a job gets per wavefront before the next job's turn; 0 = 1 << 18 */
  uint32_t use_graphs;       /* 1 = replay each bounce as a CUDA graph */
  uint64_t fail_admission_of_job; /* host-side fault injection: admission of this job id fails as if
                                     the device were out of memory; 0 = off */
} pt_server_config;

/* One render job: the calls a reference host makes for one image. Host
 * arrays are copied before pt_server_submit returns. */
typedef struct pt_job_desc {
  const pt_scene_desc* scene;   /* set_scene */
  pt_tracer_config config;      /* HalaRenderer::new; wave_paths and keep_samples are ignored */
  uint32_t frames;              /* render() calls = samples per pixel */
  uint32_t camera_index;
  const float* env_rgb;         /* set_envmap: RGB32F, env_width x env_height; NULL = sky */
  uint32_t env_width;
  uint32_t env_height;
  float env_rotation_deg;
  float ground_color[4];        /* set_ground_color */
  float sky_color[4];           /* set_sky_color */
  float env_intensity;          /* set_env_intensity */
  float exposure_value;         /* set_exposure_value */
  const pt_cache_config* cache; /* non-NULL: render with an online radiance cache of this
                                   configuration (pt_renderer_set_radiance_cache); such a job
                                   runs its passes on its own, between shared wavefronts */
} pt_job_desc;

typedef enum pt_job_state {
  PT_JOB_QUEUED = 0,     /* waiting for budget or a slot */
  PT_JOB_RUNNING = 1,    /* admitted: resident on the device, sharing wavefronts */
  PT_JOB_DONE = 2,       /* all frames accumulated and tonemapped; images readable */
  PT_JOB_FAILED = 3,     /* see pt_job_info.status and .error */
  PT_JOB_CANCELLED = 4
} pt_job_state;

typedef struct pt_job_info {
  uint64_t id;
  int32_t state;          /* pt_job_state */
  int32_t status;         /* pt_status of a failed job */
  uint64_t paths_total;   /* width * height * frames */
  uint64_t paths_done;
  uint64_t device_bytes;  /* admission estimate */
  double submit_ms;       /* host clock, ms since the server was created */
  double admit_ms;        /* admitted to the device (0 while queued) */
  double done_ms;         /* reached a final state (0 before) */
  char error[128];
} pt_job_info;

typedef struct pt_server_stats {
  uint64_t jobs_submitted;
  uint64_t jobs_done;
  uint64_t jobs_failed;
  uint64_t jobs_cancelled;
  uint64_t jobs_rejected;      /* refused at submit (invalid, or larger than the whole budget) */
  uint32_t jobs_queued;
  uint32_t jobs_running;
  uint64_t resident_bytes;     /* admission estimates of the admitted jobs */
  uint64_t peak_resident_bytes;
  uint64_t wavefronts;
  uint64_t paths;
  uint64_t closest_rays;
  uint64_t shadow_rays;
  uint64_t kernel_launches;
  uint64_t graph_launches;
  double busy_ms;              /* device time of all wavefronts (CUDA events) */
  double uptime_ms;
} pt_server_stats;

pt_status pt_server_create(const pt_server_config* config, pt_server** out);
/* Cancels what is still queued or running, waits for the scheduler, frees
 * everything. */
void pt_server_destroy(pt_server* s);
const char* pt_server_last_error(const pt_server* s);
/* Queues a job. PT_ERR_INVALID_ARG for an invalid scene or configuration,
 * PT_ERR_OOM when the job alone exceeds the whole budget; neither is queued. */
pt_status pt_server_submit(pt_server* s, const pt_job_desc* job, uint64_t* job_id);
pt_status pt_server_poll(pt_server* s, uint64_t job_id, pt_job_info* info);
/* Waits until the job reaches a final state: PT_OK, or PT_ERR_TIMEOUT after
 * timeout_ms (0 = no limit). */
pt_status pt_server_wait(pt_server* s, uint64_t job_id, uint32_t timeout_ms);
/* Images of a PT_JOB_DONE job (accum, albedo, normal, final). */
pt_status pt_server_read_image(pt_server* s, uint64_t job_id, pt_image which, void* host, size_t bytes);
/* A queued job is cancelled at once, a running one at the next wavefront
 * boundary. */
pt_status pt_server_cancel(pt_server* s, uint64_t job_id);
/* Frees a finished job's device memory and forgets it (a job that is not
 * finished is cancelled first). */
pt_status pt_server_release(pt_server* s, uint64_t job_id);
/* 1 = stop forming wavefronts (queued jobs are still admitted), 0 = go on. */
pt_status pt_server_pause(pt_server* s, int32_t paused);
pt_status pt_server_get_stats(pt_server* s, pt_server_stats* out);

/* ---- radiance cache --------------------------------------------------------
 * No counterpart in the reference (its integrator is the plain unbiased path
 * tracer of pathtracer.rgen.glsl). An online-trained neural radiance cache:
 * a multiresolution hash-grid encoding of the query position (16 levels,
 * 2^log2_table_size fp16 entries of 2 features per level) plus direction,
 * normal and material inputs, feeding an MLP with 5 hidden layers of 64 ReLU
 * units (BF16 weights, FP32 accumulation), trained with Adam on the relative
 * L2 loss. With a cache attached to a renderer, the vertex `query_depth` of
 * a path gets its emission and direct light as usual, and the light arriving
 * there through further bounces (the indirect part) is the cache's estimate:
 * the path ends at that vertex. 1 in 2^train_shift paths continue unbiased
 * and become training samples. Without a cache the renderer is the plain
 * tracer.
 *
 * Query record (16 floats): position xyz, outgoing direction xyz (towards
 * the previous vertex), shading normal xyz, base colour rgb, roughness,
 * metallic, specular transmission, 0. */
typedef struct pt_cache pt_cache;

struct pt_cache_config {
  uint32_t query_depth;     /* vertex index at which paths end in the cache (1 = first bounce) */
  uint32_t train_shift;     /* 1 in 2^train_shift paths trains the cache (5 = 1/32) */
  uint32_t batch_size;      /* training batch in samples (multiple of 16) */
  uint32_t log2_table_size; /* hash-table entries per level = 2^log2_table_size */
  float learning_rate;      /* Adam learning rate */
  uint32_t min_resolution;  /* coarsest grid level */
  uint32_t max_resolution;  /* finest grid level */
  uint32_t seed;            /* weight initialisation */
  uint32_t warmup_frames;   /* frames traced with every path training before the first query */
  uint32_t paths_per_pass;  /* wavefront size while a cache is attached: the cache trains
                               between wavefronts, so smaller passes adapt sooner */
  uint32_t steps_per_pass;  /* optimiser steps after each pass at least (batches cycle
                               through the pass's samples) */
  uint32_t weight_grad_kernel; /* weight gradients: 0 = tcgen05 tensor-core kernel with the
                                  accumulator in tensor memory, 1 = the warp-level mma.sync
                                  kernel (kept for comparison) */
  float min_roughness;      /* the cache vertex queries (or trains) the cache only where the
                               surface is diffuse, or Disney without a glass lobe and at least
                               this rough; elsewhere the path goes on unbiased. 0 = every vertex */
};

/* query_depth 1, 1/32 training paths, batch 65536, 2^19 entries, lr 1e-2,
 * resolutions 16..2048, seed 1, one warm-up frame, passes of 2^21 paths,
 * at least one optimiser step per pass, tcgen05 weight gradients, cache
 * vertices at least 0.3 rough. */
void pt_cache_config_default(pt_cache_config* config);
pt_status pt_cache_create(const pt_cache_config* config, pt_cache** out);
void pt_cache_destroy(pt_cache* cache);
const char* pt_cache_last_error(const pt_cache* cache);
/* Scene box mapped to the unit cube of the encoding. */
pt_status pt_cache_set_bounds(pt_cache* cache, const float lo[3], const float hi[3]);
/* Parameter counts: MLP weights (layer by layer, [in][out] row-major) and
 * hash-table floats ([level][entry][feature]). */
pt_status pt_cache_num_params(const pt_cache* cache, uint64_t* mlp, uint64_t* grid);
/* FP32 master parameters (either pointer may be NULL). */
pt_status pt_cache_get_params(pt_cache* cache, float* mlp, float* grid);
pt_status pt_cache_set_params(pt_cache* cache, const float* mlp, const float* grid);
/* Predicted RGB (3 floats per record) for n host records. */
pt_status pt_cache_infer(pt_cache* cache, const float* records, uint32_t n, float* out_rgb);
/* Loss and gradients of one batch without updating anything (gradient check). */
pt_status pt_cache_gradients(pt_cache* cache, const float* records, const float* targets_rgb, uint32_t n,
                             float* mlp_grad, float* grid_grad, float* loss);
/* `steps` passes of Adam over the n samples in batches of batch_size; the
 * loss of the last batch goes to *last_loss. */
pt_status pt_cache_train(pt_cache* cache, const float* records, const float* targets_rgb, uint32_t n,
                         uint32_t steps, float* last_loss);
/* Device-timed throughput of the cache kernels on n seeded records: mean
 * milliseconds of one inference over all n, and of one training pass over
 * them (batches of batch_size), over `iterations` repetitions. Trains the
 * cache on those records. */
pt_status pt_cache_benchmark(pt_cache* cache, uint32_t n, uint32_t iterations, double* infer_ms, double* train_ms);
/* Attaches a new cache to the renderer (NULL detaches it and renders
 * unbiased again). The renderer owns the cache; scenes with participating
 * media are refused (PT_ERR_UNSUPPORTED). */
pt_status pt_renderer_set_radiance_cache(pt_renderer* r, const pt_cache_config* config);

/* ---- helpers ------------------------------------------------------------- */

/* Fills ax/ay from roughness/anisotropic the way the shaders expect them
 * (inc/bxdf/disney.glsl:420, inc/bxdf/oren_nayar.glsl:35-46). */
void pt_material_preprocess(pt_material* m);
/* Default-initialised material (Disney-free diffuse white, opacity 1, ior 1.5,
 * no maps, no medium). */
void pt_material_default(pt_material* m);
uint32_t pt_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* HALA_PT_H */
