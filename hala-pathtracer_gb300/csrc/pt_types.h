// pt_types.h -- device data layout of the GB300 wavefront path tracer.
//
// HBM layout (one renderer):
//   scene    tri[3*slot]        float4 x3 per triangle in BVH leaf order:
//                               (v0.xyz, global id bits), e1, e2   -- 48 B
//            nodes[4*i]         binary BVH node, 64 B: child boxes + links
//            tri_vidx[3*id]     global vertex indices of triangle id
//            tri_mat[id]        material index of triangle id
//            vnorm/vtan[v]      float4 world-space (un-normalised) attributes
//            tri_shade[6*id]    float4 x6: the normals then the tangents of
//                               triangle id's three vertices (copies of
//                               vnorm/vtan; .w of the first = material index
//                               bits), one dependent fetch for shading -- 96 B
//            vuv[v]             float2
//            mats[]             pt_material (the std140 Material field set)
//            env_rgba[]         float4 per environment texel
//            alias rows/cols    uint2 (prob bits, alias index) per entry
//   wave     SoA path state sized for `wave_paths` paths (see PathState)
//   images   accum/albedo/normal float4 per pixel, final uchar4 per pixel
#pragma once

// Children per traversal node, 4 or 8 (compile time). Measured on the GB300
// (Disney grid): 8-wide nodes cut node visits per ray from 10.2 to 6.8 but
// made each visit dearer (two slab groups, a 19-comparator sort, spills at
// the traversal kernels' register cap): closest hit 6.07 -> 7.90 ms per
// launch. 4 is the default.
#ifndef HPT_BVH_WIDTH
#define HPT_BVH_WIDTH 4
#endif
#include <cstdint>

#include "../../include/hala_pt.h"

namespace hpt {

struct DevLight {  // inc/types.glsl:14-39, padded to 64 B
  float intensity[3];
  float position[3];
  float u[3];
  float v[3];
  float radius;
  float area;
  int32_t type;
  int32_t pad;
};

struct DevCamera {  // inc/types.glsl:2-11
  float position[3];
  float right[3];
  float up[3];
  float forward[3];
  float yfov, fd_or_xmag, ap_or_ymag;
  uint32_t type;
};

// Binary BVH node (64 B = 4 x 16 B loads):
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (link0, link1, 0, 0)
// link >= 0: internal node index; link < 0: leaf, start = link & 0x03FFFFFF
// (slot in tri[]), count = (link >> 26) & 0x1F. An empty child has an
// inverted box so it never intersects.
// Wide BVH node used by the traversal: BVH_WIDTH children in groups of 4,
// NODE_F4 16-byte words (32 B per child):
//   q[6g .. 6g+5]     = lo.x, hi.x, lo.y, hi.y, lo.z, hi.z of the four
//                       children of group g
//   q[6G + g]         = the four child links of group g (as above;
//                       EMPTY_LINK for an unused slot, whose box is +inf on
//                       every bound so that no ray enters it: both slab
//                       distances of an axis are then +inf or -inf)
//   q[7G .. 8G - 1]   = unused
// with G = BVH_WIDTH / 4 groups. It is collapsed from the binary tree:
// a node of width W replaces log2(W) binary levels, which shortens the
// chain of dependent node fetches a ray waits on.
constexpr int BVH_WIDTH = HPT_BVH_WIDTH;
constexpr int BVH_GROUPS = BVH_WIDTH / 4;
constexpr int NODE_F4 = 8 * BVH_GROUPS;
static_assert(BVH_WIDTH == 4 || BVH_WIDTH == 8, "4- or 8-wide nodes");
constexpr int32_t EMPTY_LINK = 0x7FFFFFFF;
constexpr int32_t LEAF_BIT = (int32_t)0x80000000u;
constexpr int LEAF_MAX = 8;

__host__ __device__ inline int32_t make_leaf_link(uint32_t start, uint32_t count) {
  return (int32_t)(0x80000000u | (count << 26) | start);
}

struct DevScene {
  const float4* tri;
  const float4* nodes;
  const uint32_t* tri_vidx;
  const uint32_t* tri_mat;
  const float4* vnorm;
  const float4* vtan;
  const float4* tri_shade;
  const float2* vuv;
  const pt_material* mats;
  // per material, which shading kernel takes its hits: MAT_CLASS_*
  const uint32_t* mat_class;
  uint32_t num_mats;
  uint32_t num_tris;
  uint32_t num_lights;
  uint32_t env_map;  // 0 = sky (ENV_TYPE_SKY), 1 = map
  DevLight lights[PT_MAX_LIGHTS];
  DevCamera cam;
  // environment, inc/global.glsl:11-24
  const float4* env_rgba;
  const uint2* alias_rows;  // (prob float bits, alias)
  const uint2* alias_cols;
  uint32_t env_w, env_h;
  float env_rotation, env_intensity, env_total_sum;
  float ground[3], sky[3];
  // tracer settings, MainUBO inc/global.glsl:11-30
  uint32_t width, height, max_depth, rr_depth, seed;
  uint32_t features;
  // material textures (g_textures, inc/global.glsl:48): texels of all maps
  // back to back, and per map (first texel, width, height, 0)
  const float4* tex_texels;
  const uint4* tex_info;
  uint32_t num_textures;
  // traversal limits (stack entries <= 96, node visits per ray) and the
  // device word their violations are reported in (TRAV_ERR_* bits)
  uint32_t trav_stack, trav_visits;
  uint32_t* err;
  // blue-noise texture of the camera jitter (PT_BLUE_NOISE_SIZE^2 RGBA8
  // texels), or null for the substitute table
  const uchar4* blue_noise;
};

// Structure-of-arrays path state of one wavefront (capacity P paths).
struct PathState {
  uint4* rng;        // s0 of the per-path RNG (s1 is only used by the camera)
  float4* ray_o;     // origin.xyz
  float4* ray_d;     // direction.xyz
  float4* hit;       // t, u, v, id bits (light hit: u = light pdf)
  float4* thr;       // throughput.xyz, state.pdf
  float4* rad;       // radiance.xyz, hash bits
  uint32_t* depth;   // state.depth (uint, wraps like the reference)
  uint32_t* flags;   // state.flags | ANS_BIT | IN_MEDIUM_BIT | DONE_BIT
  float4* albedo;    // first-hit albedo
  float4* normal;    // first-hit normal
  float4* med0;      // medium color.xyz, density
  float2* med1;      // medium anisotropy, type bits
  // pending next-event estimation: shadow rays + contributions. Surfaces
  // without media (k_shadow):
  float4* sh_o;      // scatter position, pending bits (1 env, 2 light) and events
  float4* sh_d0;     // env ray dir, tmax
  float4* sh_d1;     // light ray dir, tmax
  float4* sh_c0;     // env contribution, (unused)
  float4* sh_c1;     // light contribution, (unused)
  float4* sh_T;      // throughput at the NEE vertex
  // With media and no transparent material (k_transmit): sh_d0/sh_d1 hold
  // the ray direction and MIS weight, sh_c0/sh_c1 the light's radiance and
  // pdf, sh_f0/sh_f1 the BSDF or phase value and whether the sample adds
  // light when visible (media waves only).
  float4* sh_f0;
  float4* sh_f1;
  // shared wavefronts of several jobs (serving): per-path job slot and the
  // device table of the jobs' scene records; null for a single-scene render
  uint32_t* job;
  const struct DevScene* jobs;
  // radiance cache (all null when no cache is attached)
  float4* c_rec;       // query record of a path that ends in the cache (4 float4 per slot)
  float4* c_T;         // throughput arriving at the query vertex
  uint32_t* c_queue;   // slots waiting for a cache query
  uint32_t* c_counts;  // [0] queued queries, [1] training samples
  uint32_t* c_train;   // training-sample index of the slot, ~0u = none
  float4* t_rec;       // training samples: record (4 float4 each),
  float4* t_T;         //   throughput arriving at the vertex,
  float4* t_R;         //   radiance gathered up to the vertex's own emission and
                       //   direct light (NaN until the path leaves the vertex)
  uint32_t c_depth;    // vertex index of the query
  uint32_t c_mode;     // 1 = every path trains (warm-up), 2 = query, 1 in 2^c_shift trains
  uint32_t c_shift;
  float c_min_rough;   // cache vertices must be at least this rough (and not glass)
};

// One contiguous run of a job's paths inside a shared wavefront: wave slots
// [start, start + count) hold the job's global path indices g0 .. g0 + count.
struct WaveSegment {
  uint32_t slot;
  uint32_t start;
  uint32_t count;
  uint32_t pad;
  uint64_t g0;
};

constexpr uint32_t ANS_BIT = 0x100u;        // any_non_specular_bounce
constexpr uint32_t IN_MEDIUM_BIT = 0x200u;  // is_in_medium

// Shading kernel of a material (DevScene::mat_class; 0 = the surface-logic
// kernel: misses, lights, invalid materials). A Disney material whose glass
// lobe weight, (1 - metallic) * specular_transmission as the lobe
// probabilities compute it, is zero (or NaN) is shaded by a kernel built
// without that lobe.
constexpr uint32_t MAT_CLASS_DIFFUSE = 1, MAT_CLASS_DISNEY = 2, MAT_CLASS_GLASS = 3;
// Template argument of k_shade for the glass-capable Disney kernel.
constexpr int SHADE_DISNEY_GLASS = 2;

// Queue counters (device memory)
enum QueueSlot : int {
  Q_NEXT = 0,     // paths continuing to the next bounce
  // slot 1 unused (misses and emitter hits end in the closest-hit kernel)
  Q_DIFFUSE = 2,  // surface hits on diffuse materials
  Q_DISNEY = 3,   // surface hits on Disney materials without a glass lobe
  Q_SHADOW = 4,   // paths with pending shadow rays
  C_CLOSEST = 5,  // closest-hit rays traced (64-bit pair: 5,6)
  C_SHADOW = 7,   // shadow/transmittance rays traced (64-bit pair: 7,8)
  Q_GLASS = 9,    // surface hits on Disney materials whose glass lobe can be sampled
  Q_COUNT = 16
};

}  // namespace hpt
