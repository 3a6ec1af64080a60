// ref_harness.inl -- host stand-in for the Vulkan ray-tracing pipeline around
// the reference's own shaders (oracle/_ref, test infrastructure only).
//
// This file is appended to the translation unit that holds the reference's
// GLSL (compiled through glsl_shim.h). It provides what the RT pipeline and
// the missing hala-renderer crate provide on the GPU, with the conventions
// the CPU oracle and the CUDA library share:
//   * traceRayEXT: brute-force closest hit over world-space triangles,
//     lexicographic minimum of (t, global triangle id); the light
//     intersection shader lights.rint runs for every light and a light wins
//     only when strictly closer; hit, light-hit and miss shaders run as the
//     SBT would run them; payload locations 0/1/2 are routed to
//     g_ray_payload / g_shadow_ray_payload / g_trans_ray_payload;
//   * executeCallableEXT: the 15 callables in the SBT order of
//     src/bin/hala-pathtracer.rs:170-186;
//   * textures: the blue-noise texture (a loaded 1024 x 1024 RGBA8 table,
//     else the substitute: pcg4d of the texel coordinates read as RGBA8),
//     nearest-texel environment lookups (u wraps, v clamps), and the
//     two distribution textures realised by FP64 alias tables;
//   * images: the accumulation, albedo, normal and RGBA8 final images.
#include <atomic>
#include <thread>
#include <vector>

#include "../../include/hala_pt.h"

accelerationStructureEXT g_tlas{0};
image2D g_final_image{0};
image2D g_accum_image{1};
image2D g_albedo_image{2};
image2D g_normal_image{3};
texture2D g_blue_noise{0};
sampler2D g_env_map(0, 0);
texture2D g_env_map_dist[2] = {{0}, {1}};
sampler g_env_map_dist_sampler{0};
thread_local MainUBO g_main_ubo_inst;
CamerasBuffer g_cameras_buf_inst;
LightsBuffer g_lights_buf_inst;
MaterialBuffer* g_materials = nullptr;
PrimitivesBuffer* g_primitives = nullptr;
sampler2D* g_textures = nullptr;

thread_local LaunchID gl_LaunchIDEXT;
thread_local uint gl_InstanceCustomIndexEXT;
thread_local int gl_PrimitiveID;
thread_local float gl_HitTEXT;
thread_local uint gl_HitKindEXT;
thread_local vec3 gl_WorldRayOriginEXT;
thread_local vec3 gl_WorldRayDirectionEXT;
thread_local float gl_RayTminEXT;
thread_local float gl_RayTmaxEXT;
thread_local vec2 attribs;
thread_local LightHitAttribute g_light_hit_attribute;

namespace refh {

struct Tri {
  vec3 v0, e1, e2;
  uint prim, local;
};

struct Ctx {
  pt_tracer_config cfg{};
  std::vector<std::vector<Vertex>> verts;
  std::vector<std::vector<uint>> idx;
  std::vector<PrimitivesBuffer> prims;
  std::vector<MaterialBuffer> mats;
  std::vector<Tri> tris;
  uint num_lights = 0;
  MainUBO ubo{};
  bool env_map = false;
  std::vector<float> env_rgb;
  uint env_w = 0, env_h = 0;
  std::vector<float> prob_rows, prob_cols;
  std::vector<uint> alias_rows, alias_cols;
  std::vector<vec4> accum, albedo, normal;
  std::vector<unsigned char> final_img;
  uint64_t frame_index = 0;
  // material textures behind g_textures (sampler kind 3, id = index)
  std::vector<std::vector<float>> tex_rgba;
  std::vector<uint> tex_w, tex_h;
  std::vector<sampler2D> tex_samplers;
  // blue-noise texels (1024 x 1024 RGBA8) or empty: the substitute
  std::vector<unsigned char> blue_noise;
};

Ctx* g_ctx = nullptr;

// Moller-Trumbore on (v0, e1, e2), the same operations as the oracle.
inline bool tri_hit(const vec3& o, const vec3& d, const Tri& T, float tmin, float tmax, float& t, float& u, float& v) {
  vec3 pvec = cross(d, T.e2);
  float det = dot(T.e1, pvec);
  if (det == 0.0f) return false;
  float inv = 1.0f / det;
  vec3 tvec = o - T.v0;
  u = dot(tvec, pvec) * inv;
  if (u < 0.0f || u > 1.0f) return false;
  vec3 qvec = cross(tvec, T.e1);
  v = dot(d, qvec) * inv;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot(T.e2, qvec) * inv;
  if (t < tmin || t > tmax) return false;
  return true;
}

thread_local bool t_reported;
thread_local float t_rep_t;
thread_local uint t_rep_kind;

inline uint tex_index(float u, float v) {
  Ctx& c = *g_ctx;
  float fu = u - std::floor(u);
  if (!(fu >= 0.0f)) fu = 0.0f;
  float fv = v;
  if (!(fv >= 0.0f)) fv = 0.0f;
  if (fv > 1.0f) fv = 1.0f;
  uint ix = (uint)(fu * (float)c.env_w), iy = (uint)(fv * (float)c.env_h);
  if (ix > c.env_w - 1) ix = c.env_w - 1;
  if (iy > c.env_h - 1) iy = c.env_h - 1;
  return iy * c.env_w + ix;
}

inline uint alias_draw(const float* prob, const uint* alias, uint n, float s, float& frac) {
  float x = s * (float)n;
  uint k = (uint)x;
  if (k > n - 1) k = n - 1;
  float r = x - (float)k;
  float p = prob[k];
  if (p >= 1.0f) { frac = r; return k; }
  if (r < p) { frac = r / p; return k; }
  frac = (r - p) / (1.0f - p);
  return alias[k];
}

// Vose's alias method in FP64 with stack-ordered small/large lists.
void build_alias(const double* w, uint n, float* prob, uint* alias) {
  double total = 0.0;
  for (uint i = 0; i < n; ++i) total += w[i];
  if (!(total > 0.0)) {
    for (uint i = 0; i < n; ++i) { prob[i] = 1.0f; alias[i] = i; }
    return;
  }
  std::vector<double> q(n);
  std::vector<uint> small, large;
  for (uint i = 0; i < n; ++i) {
    q[i] = w[i] * (double)n / total;
    if (q[i] < 1.0) small.push_back(i);
    else large.push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    uint s = small.back(); small.pop_back();
    uint l = large.back(); large.pop_back();
    prob[s] = (float)q[s];
    alias[s] = l;
    q[l] = (q[l] + q[s]) - 1.0;
    if (q[l] < 1.0) small.push_back(l);
    else large.push_back(l);
  }
  while (!large.empty()) { uint l = large.back(); large.pop_back(); prob[l] = 1.0f; alias[l] = l; }
  while (!small.empty()) { uint s = small.back(); small.pop_back(); prob[s] = 1.0f; alias[s] = s; }
}

}  // namespace refh

using namespace refh;

vec4 texelFetch(const texture2D&, const ivec2& p, int) {  // g_blue_noise, the only texelFetch
  const Ctx& c = *g_ctx;
  if (!c.blue_noise.empty()) {  // RGBA8 UNORM
    const unsigned char* t = &c.blue_noise[4 * ((size_t)p.y * 1024 + (size_t)p.x)];
    return vec4((float)t[0] / 255.0f, (float)t[1] / 255.0f, (float)t[2] / 255.0f, (float)t[3] / 255.0f);
  }
  uvec4 v = uvec4((uint)p.x, (uint)p.y, 0x2545F491u, 0x9E3779B9u);
  pcg4d(v);  // the reference's own pcg4d (common/wltcRS.glsl)
  return vec4((float)(v.x >> 24) / 255.0f, (float)(v.y >> 24) / 255.0f, (float)(v.z >> 24) / 255.0f,
              (float)(v.w >> 24) / 255.0f);
}

vec4 textureLod(const sampler2D& s, const vec2& uv, float) {
  Ctx& c = *g_ctx;
  if (s.kind == 0) {
    const float* p = &c.env_rgb[3 * (size_t)tex_index(uv.x, uv.y)];
    return vec4(p[0], p[1], p[2], 1.0f);
  }
  if (s.kind == 1) {  // marginal: s = uv.y -> v
    float f;
    uint y = alias_draw(c.prob_rows.data(), c.alias_rows.data(), c.env_h, uv.y, f);
    return vec4(((float)y + f) / (float)c.env_h, 0.0f, 0.0f, 0.0f);
  }
  if (s.kind == 2) {  // conditional on the row of texel v: s = uv.x -> u
    uint y = (uint)(uv.y * (float)c.env_h);
    if (y > c.env_h - 1) y = c.env_h - 1;
    float f;
    uint x = alias_draw(&c.prob_cols[(size_t)y * c.env_w], &c.alias_cols[(size_t)y * c.env_w], c.env_w, uv.x, f);
    return vec4(((float)x + f) / (float)c.env_w, 0.0f, 0.0f, 0.0f);
  }
  if (s.kind == 3 && (size_t)s.id < c.tex_rgba.size()) {
    // material texture: bilinear, repeat, texel centres at half-integers
    // (the sampler the oracle and the CUDA path define)
    const uint w = c.tex_w[s.id], h = c.tex_h[s.id];
    float u = uv.x, v = uv.y;
    if (!(std::fabs(u) < 1e6f)) u = 0.0f;
    if (!(std::fabs(v) < 1e6f)) v = 0.0f;
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    auto wrap = [](long long i, uint n) {
      long long m = i % (long long)n;
      return (uint)(m < 0 ? m + n : m);
    };
    const uint ix0 = wrap((long long)x0, w), ix1 = wrap((long long)x0 + 1, w);
    const uint iy0 = wrap((long long)y0, h), iy1 = wrap((long long)y0 + 1, h);
    const float* T = c.tex_rgba[s.id].data();
    const float* a = T + 4 * ((size_t)iy0 * w + ix0);
    const float* b = T + 4 * ((size_t)iy0 * w + ix1);
    const float* cc = T + 4 * ((size_t)iy1 * w + ix0);
    const float* e = T + 4 * ((size_t)iy1 * w + ix1);
    float o[4];
    for (int k = 0; k < 4; ++k) {
      float top = a[k] + (b[k] - a[k]) * fx;
      float bot = cc[k] + (e[k] - cc[k]) * fx;
      o[k] = top + (bot - top) * fy;
    }
    return vec4(o[0], o[1], o[2], o[3]);
  }
  return vec4(1.0f, 1.0f, 1.0f, 1.0f);
}

vec4 imageLoad(const image2D& img, const ivec2& p) {
  Ctx& c = *g_ctx;
  size_t i = (size_t)p.y * c.cfg.width + (size_t)p.x;
  if (img.id == 1) return c.accum[i];
  if (img.id == 2) return c.albedo[i];
  if (img.id == 3) return c.normal[i];
  return vec4(0.0f);
}

inline unsigned char unorm8(float x) {
  float c = clamp(x, 0.0f, 1.0f);
  if (!(c == c)) c = 0.0f;
  return (unsigned char)std::floor(c * 255.0f + 0.5f);
}

void imageStore(const image2D& img, const ivec2& p, const vec4& v) {
  Ctx& c = *g_ctx;
  size_t i = (size_t)p.y * c.cfg.width + (size_t)p.x;
  if (img.id == 1) c.accum[i] = v;
  else if (img.id == 2) c.albedo[i] = v;
  else if (img.id == 3) c.normal[i] = v;
  else {
    c.final_img[4 * i] = unorm8(v.x);
    c.final_img[4 * i + 1] = unorm8(v.y);
    c.final_img[4 * i + 2] = unorm8(v.z);
    c.final_img[4 * i + 3] = 255;
  }
}

bool reportIntersectionEXT(float t, uint kind) {
  t_reported = true;
  t_rep_t = t;
  t_rep_kind = kind;
  return true;
}

void executeCallableEXT(uint sbt, int) {
  switch (sbt) {
    case 0: perspective_ray_rcall_main(); break;
    case 1: orthographic_ray_rcall_main(); break;
    case 2: env_sky_eval_rcall_main(); break;
    case 3: env_sky_sample_rcall_main(); break;
    case 4: env_map_eval_rcall_main(); break;
    case 5: env_map_sample_rcall_main(); break;
    case 6: point_light_sample_rcall_main(); break;
    case 7: directional_light_sample_rcall_main(); break;
    case 8: spot_light_sample_rcall_main(); break;
    case 9: quad_light_sample_rcall_main(); break;
    case 10: sphere_light_sample_rcall_main(); break;
    case 11: diffuse_bxdf_eval_rcall_main(); break;
    case 12: diffuse_bxdf_sample_rcall_main(); break;
    case 13: disney_bxdf_eval_rcall_main(); break;
    case 14: disney_bxdf_sample_rcall_main(); break;
    default: break;
  }
}

void traceRayEXT(const accelerationStructureEXT&, uint flags, uint, uint, uint, uint miss_index, const vec3& origin,
                 float tmin, const vec3& dir, float tmax, int payload) {
  Ctx& c = *g_ctx;
  const bool any = (flags & gl_RayFlagsTerminateOnFirstHitEXT) != 0;
  // light geometry through the reference's intersection shader
  bool light_found = false;
  float lt = 0.0f;
  uint lkind = 0;
  LightHitAttribute lattr{};
  for (uint i = 0; i < c.num_lights; ++i) {
    gl_PrimitiveID = (int)i;
    gl_WorldRayOriginEXT = origin;
    gl_WorldRayDirectionEXT = dir;
    gl_RayTminEXT = tmin;
    gl_RayTmaxEXT = tmax;
    t_reported = false;
    lights_rint_main();
    if (t_reported && (!light_found || t_rep_t < lt)) {
      light_found = true;
      lt = t_rep_t;
      lkind = t_rep_kind;
      lattr = g_light_hit_attribute;
    }
  }
  // triangles
  float best = tmax, bu = 0.0f, bv = 0.0f;
  uint best_id = 0xFFFFFFFFu;
  for (uint k = 0; k < (uint)c.tris.size(); ++k) {
    float t, u, v;
    if (tri_hit(origin, dir, c.tris[k], tmin, best, t, u, v) && (t < best || k < best_id)) {
      best = t;
      best_id = k;
      bu = u;
      bv = v;
      if (any) break;
    }
  }
  if (payload == 1) {  // shadow ray: TerminateOnFirstHit | SkipClosestHit
    if (!light_found && best_id == 0xFFFFFFFFu) shadow_ray_rmiss_main();
    return;
  }
  RayPayload saved;
  if (payload == 2) {
    saved = g_ray_payload;
    g_ray_payload = g_trans_ray_payload;
  }
  const bool light_wins = light_found && (best_id == 0xFFFFFFFFu || lt < best);
  if (light_wins) {
    g_light_hit_attribute = lattr;
    gl_HitTEXT = lt;
    gl_HitKindEXT = lkind;
    lights_rchit_main();
  } else if (best_id != 0xFFFFFFFFu) {
    gl_InstanceCustomIndexEXT = c.tris[best_id].prim;
    gl_PrimitiveID = (int)c.tris[best_id].local;
    gl_HitTEXT = best;
    attribs = vec2(bu, bv);
    triangles_rchit_main();
  } else if (miss_index == 0) {
    pathtracer_rmiss_main();
  } else {
    shadow_ray_rmiss_main();
  }
  if (payload == 2) {
    g_trans_ray_payload = g_ray_payload;
    g_ray_payload = saved;
  }
}

inline vec3 v3(const float* p) { return vec3(p[0], p[1], p[2]); }

extern "C" {

void* ref_create(const pt_tracer_config* cfg) {
  Ctx* c = new Ctx();
  c->cfg = *cfg;
  size_t n = (size_t)cfg->width * cfg->height;
  c->accum.assign(n, vec4(0.0f));
  c->albedo.assign(n, vec4(0.0f));
  c->normal.assign(n, vec4(0.0f));
  c->final_img.assign(4 * n, 0);
  MainUBO& u = c->ubo;
  u = MainUBO{};
  u.resolution = vec2((float)cfg->width, (float)cfg->height);
  u.max_depth = cfg->max_depth;
  u.rr_depth = cfg->rr_depth;
  u.enable_tonemap = cfg->enable_tonemap != 0;
  u.enable_aces = cfg->enable_aces != 0;
  u.use_simple_aces = cfg->use_simple_aces != 0;
  u.env_intensity = 1.0f;
  return c;
}

void ref_destroy(void* h) { delete static_cast<Ctx*>(h); }

int ref_set_scene(void* h, const pt_scene_desc* s) {
  Ctx& c = *static_cast<Ctx*>(h);
  c.verts.assign(s->num_primitives, {});
  c.idx.assign(s->num_primitives, {});
  c.prims.assign(s->num_primitives, PrimitivesBuffer{});
  c.tris.clear();
  for (uint p = 0; p < s->num_primitives; ++p) {
    const pt_primitive& P = s->primitives[p];
    c.verts[p].resize(P.num_vertices);
    std::memcpy(c.verts[p].data(), P.vertices, sizeof(float) * 11 * (size_t)P.num_vertices);
    c.idx[p].assign(P.indices, P.indices + P.num_indices);
    Primitive& pr = c.prims[p].data;
    for (int col = 0; col < 4; ++col)
      pr.transform.c[col] = vec4(P.transform[4 * col], P.transform[4 * col + 1], P.transform[4 * col + 2],
                                 P.transform[4 * col + 3]);
    pr.material_index = P.material_index;
    pr.vertices.data = c.verts[p].data();
    pr.indices.data = c.idx[p].data();
    const float* T = P.transform;
    std::vector<vec3> w(P.num_vertices);
    for (uint v = 0; v < P.num_vertices; ++v) {
      const float* q = P.vertices + 11 * (size_t)v;
      w[v] = vec3(((T[0] * q[0] + T[4] * q[1]) + T[8] * q[2]) + T[12],
                  ((T[1] * q[0] + T[5] * q[1]) + T[9] * q[2]) + T[13],
                  ((T[2] * q[0] + T[6] * q[1]) + T[10] * q[2]) + T[14]);
    }
    for (uint t = 0; t < P.num_indices / 3; ++t) {
      const vec3& a = w[P.indices[3 * t]];
      Tri tr;
      tr.v0 = a;
      tr.e1 = w[P.indices[3 * t + 1]] - a;
      tr.e2 = w[P.indices[3 * t + 2]] - a;
      tr.prim = p;
      tr.local = t;
      c.tris.push_back(tr);
    }
  }
  c.tex_rgba.assign(s->num_textures, {});
  c.tex_w.assign(s->num_textures, 0);
  c.tex_h.assign(s->num_textures, 0);
  c.tex_samplers.clear();
  for (uint i = 0; i < s->num_textures; ++i) {
    const pt_texture& t = s->textures[i];
    c.tex_rgba[i].assign(t.rgba, t.rgba + 4 * (size_t)t.width * t.height);
    c.tex_w[i] = t.width;
    c.tex_h[i] = t.height;
    c.tex_samplers.push_back(sampler2D((int)i, 3));
  }
  c.mats.assign(s->num_materials, MaterialBuffer{});
  for (uint i = 0; i < s->num_materials; ++i) {
    const pt_material& m = s->materials[i];
    Material& d = c.mats[i].data;
    d.medium.color = v3(m.medium.color);
    d.medium.density = m.medium.density;
    d.medium.anisotropy = m.medium.anisotropy;
    d.medium.type = m.medium.type;
    d.base_color = v3(m.base_color);
    d.opacity = m.opacity;
    d.emission = v3(m.emission);
    d.anisotropic = m.anisotropic;
    d.metallic = m.metallic;
    d.roughness = m.roughness;
    d.subsurface = m.subsurface;
    d.specular_tint = m.specular_tint;
    d.sheen = m.sheen;
    d.sheen_tint = m.sheen_tint;
    d.clearcoat = m.clearcoat;
    d.clearcoat_roughness = m.clearcoat_roughness;
    d.clearcoat_tint = v3(m.clearcoat_tint);
    d.specular_transmission = m.specular_transmission;
    d.ior = m.ior;
    d.ax = m.ax;
    d.ay = m.ay;
    d.base_color_map_index = m.base_color_map_index;
    d.normal_map_index = m.normal_map_index;
    d.metallic_roughness_map_index = m.metallic_roughness_map_index;
    d.emission_map_index = m.emission_map_index;
    d.type = m.type;
  }
  c.num_lights = s->num_lights;
  for (uint i = 0; i < MAX_LIGHTS; ++i) g_lights_buf_inst.lights[i] = Light{};
  for (uint i = 0; i < s->num_lights && i < MAX_LIGHTS; ++i) {
    const pt_light& l = s->lights[i];
    Light& d = g_lights_buf_inst.lights[i];
    d.intensity = v3(l.intensity);
    d.position = v3(l.position);
    d.u = v3(l.u);
    d.v = v3(l.v);
    d.radius = l.radius;
    d.area = l.area;
    d.type = l.type;
  }
  for (uint i = 0; i < s->num_cameras && i < MAX_CAMERAS; ++i) {
    const pt_camera& k = s->cameras[i];
    Camera& d = g_cameras_buf_inst.cameras[i];
    d.position = v3(k.position);
    d.right = v3(k.right);
    d.up = v3(k.up);
    d.forward = v3(k.forward);
    d.yfov = k.yfov;
    d.focal_distance_or_xmag = k.focal_distance_or_xmag;
    d.aperture_or_ymag = k.aperture_or_ymag;
    d.type = k.type;
  }
  c.ubo.num_of_lights = s->num_lights;
  return 0;
}

int ref_set_envmap(void* h, const float* rgb, uint w, uint hh, float rot_deg) {
  Ctx& c = *static_cast<Ctx*>(h);
  c.env_map = rgb && w && hh;
  if (!c.env_map) { c.ubo.env_type = 0; return 0; }
  c.env_rgb.assign(rgb, rgb + 3 * (size_t)w * hh);
  c.env_w = w;
  c.env_h = hh;
  c.ubo.env_type = 1;
  c.ubo.env_map_width = w;
  c.ubo.env_map_height = hh;
  c.ubo.env_rotation = rot_deg / 360.0f;
  return 0;
}

void ref_set_colors(void* h, const float ground[4], const float sky[4]) {
  Ctx& c = *static_cast<Ctx*>(h);
  c.ubo.ground_color = vec4(ground[0], ground[1], ground[2], ground[3]);
  c.ubo.sky_color = vec4(sky[0], sky[1], sky[2], sky[3]);
}
void ref_set_env_intensity(void* h, float v) { static_cast<Ctx*>(h)->ubo.env_intensity = v; }
void ref_set_blue_noise(void* h, const unsigned char* rgba8) {
  Ctx& c = *static_cast<Ctx*>(h);
  if (rgba8) c.blue_noise.assign(rgba8, rgba8 + 4 * 1024 * 1024);
  else c.blue_noise.clear();
}
void ref_set_exposure_value(void* h, float v) { static_cast<Ctx*>(h)->ubo.exposure_value = v; }

int ref_commit(void* h) {
  Ctx& c = *static_cast<Ctx*>(h);
  if (c.env_map) {
    const uint W = c.env_w, H = c.env_h;
    std::vector<double> w((size_t)W * H), rows(H);
    double total = 0.0;
    for (uint y = 0; y < H; ++y) {
      double rs = 0.0;
      for (uint x = 0; x < W; ++x) {
        const float* p = &c.env_rgb[3 * ((size_t)y * W + x)];
        double l = 0.212671 * (double)p[0] + 0.715160 * (double)p[1] + 0.072169 * (double)p[2];
        if (!(l > 0.0)) l = 0.0;
        w[(size_t)y * W + x] = l;
        rs += l;
      }
      rows[y] = rs;
      total += rs;
    }
    c.prob_rows.assign(H, 1.0f);
    c.alias_rows.assign(H, 0);
    c.prob_cols.assign((size_t)W * H, 1.0f);
    c.alias_cols.assign((size_t)W * H, 0);
    build_alias(rows.data(), H, c.prob_rows.data(), c.alias_rows.data());
    for (uint y = 0; y < H; ++y)
      build_alias(&w[(size_t)y * W], W, &c.prob_cols[(size_t)y * W], &c.alias_cols[(size_t)y * W]);
    c.ubo.env_total_sum = (float)(total * (double)c.ubo.env_intensity);
  }
  return 0;
}

int ref_render(void* h, uint frames, int threads) {
  Ctx& c = *static_cast<Ctx*>(h);
  g_ctx = &c;
  g_materials = c.mats.data();
  g_primitives = c.prims.data();
  g_textures = c.tex_samplers.data();
  const uint W = c.cfg.width, H = c.cfg.height;
  const uint64_t f0 = c.frame_index;
  std::atomic<uint> next{0};
  int T = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  if (T < 1) T = 1;
  std::vector<std::thread> ws;
  for (int t = 0; t < T; ++t)
    ws.emplace_back([&]() {
      g_main_ubo_inst = c.ubo;
      for (;;) {
        uint y = next.fetch_add(1);
        if (y >= H) break;
        for (uint x = 0; x < W; ++x)
          for (uint f = 0; f < frames; ++f) {
            g_main_ubo_inst.frame_index = (uint)(f0 + f);
            gl_LaunchIDEXT.x = x;
            gl_LaunchIDEXT.y = y;
            gl_LaunchIDEXT.z = 0;
            pathtracer_rgen_main();
          }
      }
    });
  for (auto& w : ws) w.join();
  c.frame_index += frames;
  return 0;
}

int ref_read_image(void* h, int which, void* out, size_t bytes) {
  Ctx& c = *static_cast<Ctx*>(h);
  size_t n = (size_t)c.cfg.width * c.cfg.height;
  if (which == PT_IMAGE_FINAL) {
    if (bytes != 4 * n) return PT_ERR_INVALID_ARG;
    std::memcpy(out, c.final_img.data(), bytes);
    return 0;
  }
  if (bytes != 16 * n) return PT_ERR_INVALID_ARG;
  const std::vector<vec4>& src = which == PT_IMAGE_ACCUM ? c.accum : (which == PT_IMAGE_ALBEDO ? c.albedo : c.normal);
  float* o = static_cast<float*>(out);
  for (size_t i = 0; i < n; ++i) {
    o[4 * i] = src[i].x;
    o[4 * i + 1] = src[i].y;
    o[4 * i + 2] = src[i].z;
    o[4 * i + 3] = src[i].w;
  }
  return 0;
}

}  // extern "C"
