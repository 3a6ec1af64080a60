// pt_oracle.cpp -- CPU restatement of hala-pathtracer's per-pixel integrator.
//
// TEST INFRASTRUCTURE ONLY: the checker the CUDA path is compared against,
// and the CPU baseline the benchmark times. The product library never links
// or loads this file.
//
// Each function names the reference GLSL it restates
// (paths relative to shaders/src/ of the reference project). Quirks of the
// reference are kept on purpose (they are listed where they occur).
//
// Conventions that the reference leaves to its missing hala-renderer crate
// and that this file fixes (the CUDA library uses the same ones):
//   * blue-noise texture: a pcg4d-hashed RGBA8 table (blue_noise_texel)
//   * geometry is flattened to world space at commit; closest hit is the
//     lexicographic minimum of (t, global triangle index); analytic lights
//     win only when strictly closer than the closest triangle
//   * environment map: nearest-texel lookup, u wraps, v clamps; importance
//     sampling through FP64-built alias tables (rows, then columns) with
//     the same pdf as inc/env_map.glsl:43-55; rotation = degrees / 360
#include "pt_oracle.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "pmath.h"
#include "vec.h"

namespace orc {

// common/common.glsl:6-15, hala-pathtracer/inc/constants.glsl:6-12
constexpr float PI = 3.14159265358979323846f;
constexpr float TWO_PI = 2.0f * PI;
constexpr float INV_PI = 1.0f / PI;
constexpr float INV_TWO_PI = 1.0f / TWO_PI;
constexpr float FOUR_PI = 4.0f * PI;
constexpr float INV_FOUR_PI = 1.0f / FOUR_PI;
constexpr float EPS = 0.0003f;
constexpr float INF = 1000000.0f;
constexpr float WORLD_SIZE = 10000.0f;
constexpr uint32_t INVALID_INDEX = 0xFFFFFFFFu;

constexpr uint32_t RAY_FLAGS_HIT = 0x1u;
constexpr uint32_t RAY_FLAGS_IS_EMITTER = 0x2u;
constexpr uint32_t RAY_FLAGS_SPECULAR = 0x4u;
constexpr uint32_t RAY_FLAGS_REFLECTION = 0x8u;
constexpr uint32_t RAY_FLAGS_TRANSMISSION = 0x10u;

constexpr uint32_t HIT_MISS = 0xFFFFFFFFu;
constexpr uint32_t HIT_LIGHT_BIT = 0x80000000u;

// ---------------------------------------------------------------- hashing
// Hit-sequence hash: FNV-1a over 32-bit event words. Two implementations
// that agree on every event of a path give the same hash.
inline void hmix(uint32_t& h, uint32_t x) { h = (h ^ x) * 16777619u; }
constexpr uint32_t HASH_INIT = 2166136261u;

// ---------------------------------------------------------------- RNG
// common/wltcRS.glsl:4-53
struct RNG {
  U4 s0, s1;
  int px, py;
};

inline void pcg4d(U4& v) {  // wltcRS.glsl:22-28
  v.x = v.x * 1664525u + 1013904223u;
  v.y = v.y * 1664525u + 1013904223u;
  v.z = v.z * 1664525u + 1013904223u;
  v.w = v.w * 1664525u + 1013904223u;
  v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
  v.x ^= v.x >> 16u; v.y ^= v.y >> 16u; v.z ^= v.z >> 16u; v.w ^= v.w >> 16u;
  v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
}

// float(u) / float(0xffffffffu): the divisor rounds to 2^32, so this is an
// exact scale of the rounded integer and can reach 1.0 (wltcRS.glsl:30-32).
inline float u2f(uint32_t u) { return (float)u * 2.3283064365386963e-10f; }

inline RNG rng_initialize(uint32_t px, uint32_t py, uint32_t frame) {  // wltcRS.glsl:9-19
  RNG r;
  r.s0 = {px, py, frame, px + py};
  r.s1 = {frame, frame * 15843u, frame * 31u + 4566u, frame * 2345u + 58585u};
  r.px = (int)px;
  r.py = (int)py;
  return r;
}
inline float rand1(RNG& r) { pcg4d(r.s0); return u2f(r.s0.x); }
inline V2 rand2(RNG& r) { pcg4d(r.s0); return V2(u2f(r.s0.x), u2f(r.s0.y)); }

// Substitute for assets/textures/blue_noise.png (absent from the reference
// snapshot): texel (x, y) = pcg4d(x, y, 0x2545F491, 0x9E3779B9), each
// channel the top byte of one word read as RGBA8 unorm (k / 255).
inline void blue_noise_texel(uint32_t x, uint32_t y, float out[4]) {
  U4 v = {x, y, 0x2545F491u, 0x9E3779B9u};
  pcg4d(v);
  out[0] = (float)(v.x >> 24) / 255.0f;
  out[1] = (float)(v.y >> 24) / 255.0f;
  out[2] = (float)(v.z >> 24) / 255.0f;
  out[3] = (float)(v.w >> 24) / 255.0f;
}

// shift2 + rand4blue, wltcRS.glsl:43-53: texelFetch of a loaded 1024 x 1024
// RGBA8 texture (UNORM, byte / 255) when `tex` is given, else the substitute
inline void rand4blue(RNG& r, const uint8_t* tex, float out[4]) {
  pcg4d(r.s1);
  int sx = (r.px + (int)(r.s1.x % 0x0fffffffu)) % 1024;
  int sy = (r.py + (int)(r.s1.y % 0x0fffffffu)) % 1024;
  if (tex) {
    const uint8_t* t = tex + 4 * ((size_t)sy * 1024 + (size_t)sx);
    for (int k = 0; k < 4; ++k) out[k] = (float)t[k] / 255.0f;
    return;
  }
  blue_noise_texel((uint32_t)sx, (uint32_t)sy, out);
}

// ---------------------------------------------------------------- small math
// common/common.glsl:26-71, common/sampling.glsl
inline float luminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
// Any component non-zero (NaN counts as non-zero).
inline bool nonzero(V3 c) { return c.x != 0.0f || c.y != 0.0f || c.z != 0.0f; }
inline V3 to_world(V3 X, V3 Y, V3 Z, V3 v) { return v.x * X + v.y * Y + v.z * Z; }
inline V3 to_local(V3 X, V3 Y, V3 Z, V3 v) { return V3(dot(v, X), dot(v, Y), dot(v, Z)); }
inline float sin2_theta(V3 w) { return std::fmax(0.0f, 1.0f - w.z * w.z); }
inline float sin_theta(V3 w) { return std::sqrt(sin2_theta(w)); }
inline float abs_cos_theta(V3 w) { return std::fabs(w.z); }
inline float cos_phi(V3 w) {
  float st = sin_theta(w);
  return (st == 0.0f) ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
inline float sin_phi(V3 w) {
  float st = sin_theta(w);
  return (st == 0.0f) ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}

inline float gtr1(float ndh, float a) {  // sampling.glsl:8-18
  if (a >= 1.0f) return INV_PI;
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * ndh * ndh;
  return (a2 - 1.0f) / (PI * pmath::log(a2) * t);
}
// sampling.glsl:25-44; the y component sin*sin is the reference's (kept).
inline V3 sample_gtr1(float roughness, float r1, float r2) {
  float a = std::fmax(0.001f, roughness);
  float a2 = a * a;
  float phi = r1 * TWO_PI;
  float ct = std::sqrt((1.0f - pmath::pow(a2, 1.0f - r2)) / (1.0f - a2));
  float st = clampf(std::sqrt(1.0f - (ct * ct)), 0.0f, 1.0f);
  float sp = pmath::sin(phi);
  (void)sp;
  float cp = pmath::cos(phi);
  return V3(st * cp, st * st, ct);
}
// sampling.glsl:120-136 (spherical-cap VNDF)
inline V3 sample_ggx_vndf(V3 wi, float ax, float ay, float r1, float r2) {
  V3 wiStd = normalize(V3(wi.x * ax, wi.y * ay, wi.z));
  float phi = (2.0f * r1 - 1.0f) * PI;
  float z = std::fma((1.0f - r2), (1.0f + wiStd.z), -wiStd.z);
  float sinTheta = std::sqrt(clampf(1.0f - z * z, 0.0f, 1.0f));
  float x = sinTheta * pmath::cos(phi);
  float y = sinTheta * pmath::sin(phi);
  V3 c(x, y, z);
  V3 wmStd = c + wiStd;
  return normalize(V3(wmStd.x * ax, wmStd.y * ay, wmStd.z));
}
inline float gtr2_aniso(float ndh, float hdx, float hdy, float ax, float ay) {  // sampling.glsl:146-154
  float a = hdx / ax;
  float b = hdy / ay;
  float c = a * a + b * b + ndh * ndh;
  return 1.0f / (PI * ax * ay * c * c);
}
inline float smith_g(float ndv, float alpha_g) {  // sampling.glsl:181-188
  float a = alpha_g * alpha_g;
  float b = ndv * ndv;
  return (2.0f * ndv) / (ndv + std::sqrt(a + b - a * b));
}
inline float smith_g_aniso(float ndv, float vdx, float vdy, float ax, float ay) {  // :193-202
  float a = vdx * ax;
  float b = vdy * ay;
  float c = ndv;
  return (2.0f * ndv) / (ndv + std::sqrt(a * a + b * b + c * c));
}
inline float schlick_weight(float u) {  // :207-211
  float m = clampf(1.0f - u, 0.0f, 1.0f);
  float m2 = m * m;
  return m2 * m2 * m;
}
inline float dielectric_fresnel(float cos_i, float eta) {  // :218-236
  float s2 = eta * eta * (1.0f - cos_i * cos_i);
  if (s2 > 1.0f) return 1.0f;
  float ct = std::sqrt(std::fmax(1.0f - s2, 0.0f));
  float rs = (eta * ct - cos_i) / (eta * ct + cos_i);
  float rp = (eta * cos_i - ct) / (eta * cos_i + ct);
  return 0.5f * (rs * rs + rp * rp);
}
inline V3 cosine_sample_hemisphere(float r1, float r2) {  // :252-260
  float r = std::sqrt(r1);
  float phi = TWO_PI * r2;
  float x = r * pmath::cos(phi);
  float y = r * pmath::sin(phi);
  float z = std::sqrt(std::fmax(0.0f, 1.0f - x * x - y * y));
  return V3(x, y, z);
}
inline V3 uniform_sample_hemisphere(float r1, float r2) {  // :266-270
  float r = std::sqrt(std::fmax(0.0f, 1.0f - r1 * r1));
  float phi = TWO_PI * r2;
  return V3(r * pmath::cos(phi), r * pmath::sin(phi), r1);
}
inline float power_heuristic(float a, float b) {  // :286-290
  a *= a;
  b *= b;
  return a / (a + b);
}
inline void onb(V3 N, V3& T, V3& B) {  // :296-300
  V3 up = std::fabs(N.z) < 0.9999999f ? V3(0, 0, 1) : V3(1, 0, 0);
  T = normalize(cross(up, N));
  B = cross(N, T);
}
inline V3 sample_hg(V3 V, float g, float r1, float r2) {  // :308-327
  float ct;
  if (std::fabs(g) < 0.001f) {
    ct = 1.0f - 2.0f * r2;
  } else {
    float sq = (1.0f - g * g) / (1.0f + g - 2.0f * g * r2);
    ct = -(1.0f + g * g - sq * sq) / (2.0f * g);
  }
  float phi = r1 * TWO_PI;
  float st = clampf(std::sqrt(1.0f - (ct * ct)), 0.0f, 1.0f);
  float sp = pmath::sin(phi);
  float cp = pmath::cos(phi);
  V3 v1, v2;
  onb(V, v1, v2);
  return st * cp * v1 + st * sp * v2 + ct * V;
}
inline float phase_hg(float ct, float g) {  // :333-336
  float denom = std::fmax(1.0f + g * g + 2.0f * g * ct, EPS);
  return INV_FOUR_PI * (1.0f - g * g) / (denom * std::sqrt(denom));
}

// ---------------------------------------------------------------- tonemap
// common/tonemap.glsl, common/common.glsl:26-39
inline float linear_2_srgb(float x) {
  if (x <= 0.0031308f) return 12.92f * x;
  return 1.055f * pmath::pow(x, 1.0f / 2.4f) - 0.055f;
}
// v * mat3(c0, c1, c2) = (dot(v, c0), dot(v, c1), dot(v, c2))
inline V3 aces_fitted(V3 c) {
  const V3 i0(0.59719f, 0.35458f, 0.04823f), i1(0.07600f, 0.90834f, 0.01566f),
      i2(0.02840f, 0.13383f, 0.83777f);
  const V3 o0(1.60475f, -0.53108f, -0.07367f), o1(-0.10208f, 1.10813f, -0.00605f),
      o2(-0.00327f, -0.07276f, 1.07602f);
  c = V3(dot(c, i0), dot(c, i1), dot(c, i2));
  V3 a = c * (c + V3(0.0245786f)) - V3(0.000090537f);
  V3 b = c * (0.983729f * c + V3(0.4329510f)) + V3(0.238081f);
  c = a / b;
  c = V3(dot(c, o0), dot(c, o1), dot(c, o2));
  return clamp(c, 0.0f, 1.0f);
}
inline V3 aces_simple(V3 c) {
  const float a = 2.51f, b = 0.03f, y = 2.43f, d = 0.59f, e = 0.14f;
  return clamp((c * (a * c + V3(b))) / (c * (y * c + V3(d)) + V3(e)), 0.0f, 1.0f);
}
inline V3 tonemap_lum(V3 c, float limit) { return c * 1.0f / (1.0f + luminance(c) / limit); }

// pathtracer.rgen.glsl:280-301
inline V3 finish_color(V3 accum, float ev, bool enable, bool aces, bool simple) {
  V3 c = accum;
  float exposure = pmath::pow(2.0f, ev);
  c = c * exposure;
  if (enable) {
    if (aces) c = simple ? aces_simple(c) : aces_fitted(c);
    else c = tonemap_lum(c, 1.5f);
  }
  return V3(linear_2_srgb(c.x), linear_2_srgb(c.y), linear_2_srgb(c.z));
}
inline uint8_t to_unorm8(float x) {
  float c = clampf(x, 0.0f, 1.0f);
  if (!(c == c)) c = 0.0f;
  return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

// ---------------------------------------------------------------- scene
struct Light {
  V3 intensity, position, u, v;
  float radius, area;
  int type;
};
struct Medium {
  V3 color;
  float density = 0.0f, anisotropy = 1.0f;
  uint32_t type = PT_MEDIUM_NONE;
};
struct Material {
  Medium medium;
  V3 base_color;
  float opacity;
  V3 emission;
  float anisotropic, metallic, roughness, subsurface, specular_tint, sheen, sheen_tint, clearcoat,
      clearcoat_roughness;
  V3 clearcoat_tint;
  float specular_transmission, ior, ax, ay;
  uint32_t base_color_map, normal_map, mr_map, emission_map, type;
};
struct Camera {
  V3 position, right, up, forward;
  float yfov, fd_or_xmag, ap_or_ymag;
  uint32_t type;
};
struct Texture {
  std::vector<float> rgba;
  uint32_t w = 0, h = 0;
};

inline V3 v3(const float* p) { return V3(p[0], p[1], p[2]); }

struct State {  // inc/types.glsl:129-145
  V3 first_hit_position, ffnormal, normal, tangent, bitangent;
  V2 tex_coord;
  float hit_distance = 0.0f, pdf = 1.0f, eta = 1.0f;
  uint32_t flags = 0, depth = 0;
  uint32_t material_index = INVALID_INDEX;
  Medium medium;
};

struct Ray {
  V3 o, d;
};

// ---------------------------------------------------------------- BVH
struct AABB {
  V3 lo, hi;
};
struct BNode {
  AABB box;
  int left = -1, right = -1;  // children (internal)
  int start = 0, count = 0;   // leaf range in tri_order
};

struct Ctx {
  pt_tracer_config cfg{};
  bool force_brute = false;  // paths traced against every triangle instead of the BVH (checks)
  // flattened geometry
  std::vector<V3> tv0, te1, te2;            // per triangle, world space
  std::vector<uint32_t> tidx;               // 3 global vertex indices per triangle
  std::vector<uint32_t> tmat;               // material index per triangle
  std::vector<V3> vnorm, vtan;              // world-transformed (not normalised)
  std::vector<V2> vuv;
  std::vector<Material> mats;
  std::vector<Light> lights;
  std::vector<Camera> cams;
  std::vector<Texture> texs;
  uint32_t camera_index = 0;
  std::vector<uint8_t> blue_noise;  // 1024 x 1024 RGBA8, or empty: the substitute
  // environment, inc/global.glsl:11-24
  bool env_map = false;
  std::vector<float> env_rgb;
  uint32_t env_w = 0, env_h = 0;
  float env_rotation = 0.0f, env_intensity = 1.0f, env_total_sum = 1.0f;
  std::vector<float> alias_prob_rows, alias_prob_cols;
  std::vector<uint32_t> alias_idx_rows, alias_idx_cols;
  V3 ground, sky;
  float exposure = 0.0f;
  // features, src/bin/hala-pathtracer.rs:101-114
  bool use_medium = false, use_vol_mis = false, use_transparent = false;
  // BVH
  std::vector<BNode> nodes;
  std::vector<uint32_t> tri_order;
  bool committed = false;
  // images
  std::vector<float> accum, albedo, normal;  // RGBA32F
  std::vector<double> accum64;
  uint64_t frame_index = 0;
  bool fp64_mode = false;
  std::atomic<uint64_t> n_paths{0}, n_closest{0}, n_shadow{0};
};

// Closest hit record
struct Hit {
  float t;
  float u, v;
  uint32_t id;  // triangle id, HIT_LIGHT_BIT|light, HIT_MISS
  V3 light_normal;
  float light_pdf;
};

// Moller-Trumbore on precomputed (v0, e1, e2). Valid when tmin <= t <= tmax.
// The device code performs exactly these IEEE operations in this order.
inline bool intersect_tri(const V3& o, const V3& d, const V3& v0, const V3& e1, const V3& e2,
                          float tmin, float tmax, float& t, float& u, float& v) {
  V3 pvec = cross(d, e2);
  float det = dot(e1, pvec);
  if (det == 0.0f) return false;
  float inv = 1.0f / det;
  V3 tvec = o - v0;
  u = dot(tvec, pvec) * inv;
  if (u < 0.0f || u > 1.0f) return false;
  V3 qvec = cross(tvec, e1);
  v = dot(d, qvec) * inv;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot(e2, qvec) * inv;
  if (t < tmin || t > tmax) return false;
  return true;
}

// Slab test; the far distance is widened by 2 ulp-ish so a box never misses
// a triangle it contains (Ize 2013). Same arithmetic on the device.
// Conservative slab test: a few ulps of slack on the slab interval, and
// 2^-12 relative slack on tmax (the best hit so far): a triangle's computed t
// can be early by many ulps when the ray grazes it or it is small against its
// distance, and its box must not be culled for that (the device traversal
// uses the same slack).
inline bool slab(const AABB& b, const V3& o, const V3& inv, float tmin, float tmax, float& tn) {
  float tx0 = (b.lo.x - o.x) * inv.x, tx1 = (b.hi.x - o.x) * inv.x;
  float ty0 = (b.lo.y - o.y) * inv.y, ty1 = (b.hi.y - o.y) * inv.y;
  float tz0 = (b.lo.z - o.z) * inv.z, tz1 = (b.hi.z - o.z) * inv.z;
  float tnear = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)),
                          std::fmax(std::fmin(tz0, tz1), tmin));
  float tfar = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmax(tz0, tz1));
  tfar = std::fmin(tfar * 1.0000005f, tmax * (1.0f + 1.0f / 4096.0f));
  tn = tnear;
  return tnear <= tfar;
}

static void build_bvh(Ctx& c) {
  const size_t n = c.tv0.size();
  c.nodes.clear();
  c.tri_order.resize(n);
  for (size_t i = 0; i < n; ++i) c.tri_order[i] = (uint32_t)i;
  if (n == 0) return;
  std::vector<AABB> tb(n);
  std::vector<V3> cen(n);
  for (size_t i = 0; i < n; ++i) {
    V3 a = c.tv0[i], b = a + c.te1[i], d = a + c.te2[i];
    tb[i].lo = V3(std::fmin(a.x, std::fmin(b.x, d.x)), std::fmin(a.y, std::fmin(b.y, d.y)),
                  std::fmin(a.z, std::fmin(b.z, d.z)));
    tb[i].hi = V3(std::fmax(a.x, std::fmax(b.x, d.x)), std::fmax(a.y, std::fmax(b.y, d.y)),
                  std::fmax(a.z, std::fmax(b.z, d.z)));
    cen[i] = (tb[i].lo + tb[i].hi) * 0.5f;
    // Widen by a few ulp so a box always contains every point the
    // intersection test can report for its triangle (device builder: same).
    for (int k = 0; k < 3; ++k) {
      float* lo = k == 0 ? &tb[i].lo.x : (k == 1 ? &tb[i].lo.y : &tb[i].lo.z);
      float* hi = k == 0 ? &tb[i].hi.x : (k == 1 ? &tb[i].hi.y : &tb[i].hi.z);
      *lo = *lo - (std::fabs(*lo) * 4.8e-7f + 1e-30f);
      *hi = *hi + (std::fabs(*hi) * 4.8e-7f + 1e-30f);
    }
  }
  auto grow = [](AABB& a, const AABB& b) {
    a.lo = V3(std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y), std::fmin(a.lo.z, b.lo.z));
    a.hi = V3(std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y), std::fmax(a.hi.z, b.hi.z));
  };
  auto area = [](const AABB& a) {
    V3 e = a.hi - a.lo;
    if (e.x < 0) return 0.0f;
    return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
  };
  const AABB empty{V3(1e30f), V3(-1e30f)};
  struct Task {
    int node, start, count;
  };
  c.nodes.reserve(2 * n);
  c.nodes.push_back(BNode());
  std::vector<Task> stack{{0, 0, (int)n}};
  constexpr int NB = 16;
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    AABB box = empty, cb = empty;
    for (int i = t.start; i < t.start + t.count; ++i) {
      uint32_t p = c.tri_order[i];
      grow(box, tb[p]);
      grow(cb, AABB{cen[p], cen[p]});
    }
    c.nodes[t.node].box = box;
    auto make_leaf = [&]() {
      c.nodes[t.node].start = t.start;
      c.nodes[t.node].count = t.count;
    };
    if (t.count <= 2) { make_leaf(); continue; }
    int best_axis = -1, best_bin = -1;
    float best_cost = 1e30f;
    for (int ax = 0; ax < 3; ++ax) {
      float lo = cb.lo[ax], hi = cb.hi[ax];
      if (!(hi > lo)) continue;
      AABB bb[NB];
      int bc[NB] = {0};
      for (int b = 0; b < NB; ++b) bb[b] = empty;
      float scale = NB / (hi - lo);
      for (int i = t.start; i < t.start + t.count; ++i) {
        uint32_t p = c.tri_order[i];
        int b = std::min(NB - 1, (int)((cen[p][ax] - lo) * scale));
        bc[b]++;
        grow(bb[b], tb[p]);
      }
      AABB racc = empty;
      float rarea[NB];
      int rcnt[NB];
      int acc = 0;
      for (int b = NB - 1; b > 0; --b) {
        grow(racc, bb[b]);
        acc += bc[b];
        rarea[b] = area(racc);
        rcnt[b] = acc;
      }
      AABB lacc = empty;
      int lc = 0;
      for (int b = 0; b < NB - 1; ++b) {
        grow(lacc, bb[b]);
        lc += bc[b];
        if (lc == 0 || rcnt[b + 1] == 0) continue;
        float cost = area(lacc) * lc + rarea[b + 1] * rcnt[b + 1];
        if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b; }
      }
    }
    int mid;
    if (best_axis < 0) {
      if (t.count <= 4) { make_leaf(); continue; }
      mid = t.start + t.count / 2;
    } else {
      float leaf_cost = area(box) * t.count;
      if (t.count <= 4 && leaf_cost <= best_cost + 0.5f * area(box)) { make_leaf(); continue; }
      float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
      float scale = NB / (hi - lo);
      auto it = std::stable_partition(
          c.tri_order.begin() + t.start, c.tri_order.begin() + t.start + t.count,
          [&](uint32_t p) { return std::min(NB - 1, (int)((cen[p][best_axis] - lo) * scale)) <= best_bin; });
      mid = (int)(it - c.tri_order.begin());
      if (mid == t.start || mid == t.start + t.count) mid = t.start + t.count / 2;
    }
    int l = (int)c.nodes.size();
    c.nodes.push_back(BNode());
    c.nodes.push_back(BNode());
    c.nodes[t.node].left = l;
    c.nodes[t.node].right = l + 1;
    stack.push_back({l, t.start, mid - t.start});
    stack.push_back({l + 1, mid, t.start + t.count - mid});
  }
}

// Light intersection, inc/light/quad.glsl:42-60, common/intersection.glsl:31-72
inline float rect_intersect(V3 pos, V3 u, V3 v, V3 n, float pw, const Ray& r) {
  float dt = dot(r.d, n);
  float t = (pw - dot(n, r.o)) / dt;
  if (t > EPS) {
    V3 p = r.o + r.d * t;
    V3 vi = p - pos;
    float a1 = dot(u, vi);
    if (a1 >= 0.0f && a1 <= 1.0f) {
      float a2 = dot(v, vi);
      if (a2 >= 0.0f && a2 <= 1.0f) return t;
    }
  }
  return INF;
}
inline float quad_intersect(const Light& L, const Ray& r, V3& normal, float& pdf) {
  normal = normalize(cross(L.v, L.u));
  float ct = dot(-r.d, normal);
  if (ct < 0.0f) return INF;
  float pw = dot(normal, L.position);
  V3 u = L.u / dot(L.u, L.u);
  V3 v = L.v / dot(L.v, L.v);
  float t = rect_intersect(L.position, u, v, normal, pw, r);
  if (t < 0.0f) return INF;
  pdf = (t * t) / (L.area * ct);
  return t;
}
// common/intersection.glsl:6-26
inline float sphere_intersect_raw(float rad, V3 pos, const Ray& r) {
  V3 op = pos - r.o;
  float b = dot(op, r.d);
  float det = b * b - dot(op, op) + rad * rad;
  if (det < 0.0f) return INF;
  det = std::sqrt(det);
  float t1 = b - det;
  if (t1 > EPS) return t1;
  float t2 = b + det;
  if (t2 > EPS) return t2;
  return INF;
}
// inc/light/sphere.glsl:50-65 (the reference leaves `normal` unassigned; 0 here)
inline float sphere_light_intersect(const Light& L, const Ray& r, V3& normal, float& pdf) {
  normal = V3(0.0f);
  float dist = length(L.position - r.o);
  if (dist < L.radius) return INF;
  float t = sphere_intersect_raw(L.radius, L.position, r);
  if (t < 0.0f) return INF;
  V3 hit = r.o + t * r.d;
  float ct = dot(-r.d, normalize(hit - L.position));
  pdf = (t * t) / (L.area * ct * 0.5f);
  return t;
}
// lights.rint.glsl:16-37
inline bool light_hit(const Light& L, const Ray& r, float tmin, float tmax, float& t, V3& n,
                      float& pdf) {
  t = INF;
  n = V3(0.0f);
  pdf = 1.0f;
  if (L.type == PT_LIGHT_QUAD) t = quad_intersect(L, r, n, pdf);
  else if (L.type == PT_LIGHT_SPHERE) t = sphere_light_intersect(L, r, n, pdf);
  else return false;
  return t >= tmin && t <= tmax;
}

static Hit trace_closest(const Ctx& c, const Ray& r, float tmin, float tmax, bool brute) {
  Hit h;
  h.t = INF;
  h.u = h.v = 0.0f;
  h.id = HIT_MISS;
  float best = tmax;
  uint32_t best_id = HIT_MISS;
  float bu = 0, bv = 0;
  auto test = [&](uint32_t p) {
    float t, u, v;
    if (intersect_tri(r.o, r.d, c.tv0[p], c.te1[p], c.te2[p], tmin, best, t, u, v)) {
      if (t < best || (t == best && p < best_id)) {
        best = t;
        best_id = p;
        bu = u;
        bv = v;
      }
    }
  };
  if (brute || c.nodes.empty()) {
    for (uint32_t p = 0; p < (uint32_t)c.tv0.size(); ++p) test(p);
  } else {
    V3 inv(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const BNode& nd = c.nodes[stack[--sp]];
      float tn;
      if (!slab(nd.box, r.o, inv, tmin, best, tn)) continue;
      if (nd.left < 0) {
        for (int i = nd.start; i < nd.start + nd.count; ++i) test(c.tri_order[i]);
      } else {
        stack[sp++] = nd.right;
        stack[sp++] = nd.left;
      }
    }
  }
  if (best_id != HIT_MISS) {
    h.t = best;
    h.id = best_id;
    h.u = bu;
    h.v = bv;
  }
  // Analytic light geometry (lights.rint.glsl): wins only when strictly closer.
  float lbest = (best_id != HIT_MISS) ? best : INF;
  for (uint32_t i = 0; i < (uint32_t)c.lights.size(); ++i) {
    float t, pdf;
    V3 n;
    if (light_hit(c.lights[i], r, tmin, tmax, t, n, pdf) && t < lbest) {
      lbest = t;
      h.t = t;
      h.id = HIT_LIGHT_BIT | i;
      h.light_normal = n;
      h.light_pdf = pdf;
      h.u = pdf;  // hit attribute of lights.rint.glsl: the light pdf
      h.v = 0.0f;
    }
  }
  return h;
}

// Any-hit occlusion (TerminateOnFirstHit | Opaque | SkipClosestHit):
// inc/lighting.glsl:116-130 and :203-216. Light geometry also occludes.
static bool trace_any(const Ctx& c, const Ray& r, float tmin, float tmax, bool brute) {
  for (uint32_t i = 0; i < (uint32_t)c.lights.size(); ++i) {
    float t, pdf;
    V3 n;
    if (light_hit(c.lights[i], r, tmin, tmax, t, n, pdf)) return true;
  }
  float t, u, v;
  if (brute || c.nodes.empty()) {
    for (uint32_t p = 0; p < (uint32_t)c.tv0.size(); ++p)
      if (intersect_tri(r.o, r.d, c.tv0[p], c.te1[p], c.te2[p], tmin, tmax, t, u, v)) return true;
    return false;
  }
  V3 inv(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& nd = c.nodes[stack[--sp]];
    float tn;
    if (!slab(nd.box, r.o, inv, tmin, tmax, tn)) continue;
    if (nd.left < 0) {
      for (int i = nd.start; i < nd.start + nd.count; ++i) {
        uint32_t p = c.tri_order[i];
        if (intersect_tri(r.o, r.d, c.tv0[p], c.te1[p], c.te2[p], tmin, tmax, t, u, v)) return true;
      }
    } else {
      stack[sp++] = nd.right;
      stack[sp++] = nd.left;
    }
  }
  return false;
}

// Closest hit -> State: triangles.rchit.glsl:13-76, lights.rchit.glsl:13-26,
// pathtracer.rmiss.glsl:12-14.
static void fill_state(const Ctx& c, const Ray& r, const Hit& h, State& s) {
  if (h.id == HIT_MISS) {
    s.flags &= ~RAY_FLAGS_HIT;
    return;
  }
  if (h.id & HIT_LIGHT_BIT) {
    s.flags |= (RAY_FLAGS_HIT | RAY_FLAGS_IS_EMITTER);
    s.material_index = h.id & ~HIT_LIGHT_BIT;
    s.hit_distance = h.t;
    s.first_hit_position = r.o + r.d * s.hit_distance;
    s.normal = h.light_normal;
    s.ffnormal = dot(s.normal, r.d) <= 0.0f ? s.normal : -s.normal;
    s.tangent = V3(0.0f);
    s.bitangent = V3(0.0f);
    s.tex_coord = V2(h.light_pdf, 0.0f);
    return;
  }
  uint32_t p = h.id;
  uint32_t i0 = c.tidx[3 * p], i1 = c.tidx[3 * p + 1], i2 = c.tidx[3 * p + 2];
  float b0 = 1.0f - h.u - h.v, b1 = h.u, b2 = h.v;
  V3 n = c.vnorm[i0] * b0 + c.vnorm[i1] * b1 + c.vnorm[i2] * b2;
  n = normalize(n);
  V3 tg = c.vtan[i0] * b0 + c.vtan[i1] * b1 + c.vtan[i2] * b2;
  tg = normalize(tg);
  V3 bt = cross(n, tg);
  V2 uv0 = c.vuv[i0], uv1 = c.vuv[i1], uv2 = c.vuv[i2];
  V2 uv(uv0.x * b0 + uv1.x * b1 + uv2.x * b2, uv0.y * b0 + uv1.y * b1 + uv2.y * b2);
  s.flags |= RAY_FLAGS_HIT;
  s.material_index = c.tmat[p];
  s.hit_distance = h.t;
  s.first_hit_position = r.o + r.d * s.hit_distance;
  s.normal = n;
  s.ffnormal = dot(n, r.d) <= 0.0f ? n : -n;
  s.tangent = tg;
  s.bitangent = bt;
  s.tex_coord = uv;
}

// ---------------------------------------------------------------- material textures
// pathtracer.rgen.glsl:121-145; textureLod with bilinear filtering, repeat
// wrapping, texel centres at half-integers, row 0 at v = 0 (the glTF default
// sampler; the reference's sampler object lives in its renderer crate).
inline uint32_t wrap_texel(long long i, uint32_t n) {
  long long m = i % (long long)n;
  return (uint32_t)(m < 0 ? m + n : m);
}
static void sample_texture(const Texture& t, float u, float v, float out[4]) {
  if (!(std::fabs(u) < 1e6f)) u = 0.0f;
  if (!(std::fabs(v) < 1e6f)) v = 0.0f;
  const float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
  const float x0 = std::floor(x), y0 = std::floor(y);
  const float fx = x - x0, fy = y - y0;
  const uint32_t ix0 = wrap_texel((long long)x0, t.w), ix1 = wrap_texel((long long)x0 + 1, t.w);
  const uint32_t iy0 = wrap_texel((long long)y0, t.h), iy1 = wrap_texel((long long)y0 + 1, t.h);
  const float* a = &t.rgba[4 * ((size_t)iy0 * t.w + ix0)];
  const float* b = &t.rgba[4 * ((size_t)iy0 * t.w + ix1)];
  const float* cc = &t.rgba[4 * ((size_t)iy1 * t.w + ix0)];
  const float* e = &t.rgba[4 * ((size_t)iy1 * t.w + ix1)];
  for (int k = 0; k < 4; ++k) {
    float top = a[k] + (b[k] - a[k]) * fx;
    float bot = cc[k] + (e[k] - cc[k]) * fx;
    out[k] = top + (bot - top) * fy;
  }
}

static void apply_maps(const Ctx& c, Material& m, State& st, const V3& dir) {
  const uint32_t nt = (uint32_t)c.texs.size();
  float t[4];
  if (m.base_color_map < nt) {
    sample_texture(c.texs[m.base_color_map], st.tex_coord.x, st.tex_coord.y, t);
    m.base_color = V3(t[0], t[1], t[2]);
  }
  if (m.mr_map < nt) {
    sample_texture(c.texs[m.mr_map], st.tex_coord.x, st.tex_coord.y, t);
    m.metallic = t[2];
    m.roughness = t[1];
  }
  if (m.emission_map < nt) {
    sample_texture(c.texs[m.emission_map], st.tex_coord.x, st.tex_coord.y, t);
    m.emission = V3(t[0], t[1], t[2]);
  }
  if (m.normal_map < nt) {
    sample_texture(c.texs[m.normal_map], st.tex_coord.x, st.tex_coord.y, t);
    V3 nts(t[0], t[1], t[2] * 5.0f);
    nts = normalize(nts * 2.0f - V3(1.0f));
    const V3 orig = st.normal;
    st.normal = normalize(st.tangent * nts.x + st.bitangent * nts.y + st.normal * nts.z);
    st.ffnormal = dot(orig, dir) <= 0.0f ? st.normal : -st.normal;
    st.bitangent = cross(st.normal, st.tangent);
  }
}

// ---------------------------------------------------------------- environment
// Nearest texel of the equirect map at (u, v): u wraps, v clamps, NaN -> 0.
inline uint32_t env_texel_index(const Ctx& c, float u, float v) {
  float fu = u - std::floor(u);
  if (!(fu >= 0.0f)) fu = 0.0f;
  float fv = v;
  if (!(fv >= 0.0f)) fv = 0.0f;
  if (fv > 1.0f) fv = 1.0f;
  uint32_t ix = (uint32_t)(fu * (float)c.env_w);
  uint32_t iy = (uint32_t)(fv * (float)c.env_h);
  if (ix > c.env_w - 1) ix = c.env_w - 1;
  if (iy > c.env_h - 1) iy = c.env_h - 1;
  return iy * c.env_w + ix;
}
inline V3 env_texel(const Ctx& c, uint32_t idx) {
  const float* p = &c.env_rgb[3 * (size_t)idx];
  return V3(p[0], p[1], p[2]);
}

// inc/env_map.glsl:43-55
inline float env_pdf(const Ctx& c, float u, float v, float theta) {
  float st = pmath::sin(theta);
  if (st > EPS) {
    V3 color = env_texel(c, env_texel_index(c, u, v)) * c.env_intensity;
    float pdf = luminance(color) / c.env_total_sum;
    if (pdf > EPS)
      return (pdf * (float)c.env_w * (float)c.env_h) / (TWO_PI * PI * st);
    return 0.0f;
  }
  return 0.0f;
}

// Alias table: Vose's method in FP64, small/large lists used as stacks.
// The device builder runs the same sequential algorithm per row.
static void build_alias(const double* w, uint32_t n, float* prob, uint32_t* alias) {
  double total = 0.0;
  for (uint32_t i = 0; i < n; ++i) total += w[i];
  std::vector<double> q(n);
  std::vector<uint32_t> small, large;
  small.reserve(n);
  large.reserve(n);
  if (!(total > 0.0)) {
    for (uint32_t i = 0; i < n; ++i) { prob[i] = 1.0f; alias[i] = i; }
    return;
  }
  for (uint32_t i = 0; i < n; ++i) {
    q[i] = w[i] * (double)n / total;
    if (q[i] < 1.0) small.push_back(i);
    else large.push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    uint32_t s = small.back(); small.pop_back();
    uint32_t l = large.back(); large.pop_back();
    prob[s] = (float)q[s];
    alias[s] = l;
    q[l] = (q[l] + q[s]) - 1.0;
    if (q[l] < 1.0) small.push_back(l);
    else large.push_back(l);
  }
  while (!large.empty()) { uint32_t l = large.back(); large.pop_back(); prob[l] = 1.0f; alias[l] = l; }
  while (!small.empty()) { uint32_t s = small.back(); small.pop_back(); prob[s] = 1.0f; alias[s] = s; }
}

static void build_env_tables(Ctx& c) {
  const uint32_t W = c.env_w, H = c.env_h;
  std::vector<double> w((size_t)W * H), rows(H);
  double total = 0.0;
  for (uint32_t y = 0; y < H; ++y) {
    double rs = 0.0;
    for (uint32_t x = 0; x < W; ++x) {
      const float* p = &c.env_rgb[3 * ((size_t)y * W + x)];
      double l = 0.212671 * (double)p[0] + 0.715160 * (double)p[1] + 0.072169 * (double)p[2];
      if (!(l > 0.0)) l = 0.0;
      w[(size_t)y * W + x] = l;
      rs += l;
    }
    rows[y] = rs;
    total += rs;
  }
  c.env_total_sum = (float)(total * (double)c.env_intensity);
  c.alias_prob_rows.assign(H, 1.0f);
  c.alias_idx_rows.assign(H, 0);
  c.alias_prob_cols.assign((size_t)W * H, 1.0f);
  c.alias_idx_cols.assign((size_t)W * H, 0);
  build_alias(rows.data(), H, c.alias_prob_rows.data(), c.alias_idx_rows.data());
  for (uint32_t y = 0; y < H; ++y)
    build_alias(&w[(size_t)y * W], W, &c.alias_prob_cols[(size_t)y * W], &c.alias_idx_cols[(size_t)y * W]);
}

// One alias draw: s in [0, 1] -> bin index and the position inside the bin.
inline uint32_t alias_draw(const float* prob, const uint32_t* alias, uint32_t n, float s,
                           float& frac) {
  float x = s * (float)n;
  uint32_t k = (uint32_t)x;
  if (k > n - 1) k = n - 1;
  float r = x - (float)k;
  float p = prob[k];
  if (p >= 1.0f) { frac = r; return k; }
  if (r < p) { frac = r / p; return k; }
  frac = (r - p) / (1.0f - p);
  return alias[k];
}

// inc/env_map.glsl:6-37 with alias tables in place of the inverse-CDF textures.
static V3 sample_env_map(const Ctx& c, RNG& rng, V3& color, float& pdf) {
  V2 s = rand2(rng);
  // v = marginal(s.x); u = conditional(s.y, v) on the row of texel v; the
  // colour is the nearest texel at (u, v) -- inc/env_map.glsl:7-12 with the
  // inverse-CDF textures realised as alias tables.
  float fv, fu;
  uint32_t yr = alias_draw(c.alias_prob_rows.data(), c.alias_idx_rows.data(), c.env_h, s.x, fv);
  float v = ((float)yr + fv) / (float)c.env_h;
  uint32_t y = (uint32_t)(v * (float)c.env_h);
  if (y > c.env_h - 1) y = c.env_h - 1;
  uint32_t x = alias_draw(&c.alias_prob_cols[(size_t)y * c.env_w], &c.alias_idx_cols[(size_t)y * c.env_w],
                          c.env_w, s.y, fu);
  float u = ((float)x + fu) / (float)c.env_w;
  color = env_texel(c, env_texel_index(c, u, v)) * c.env_intensity;
  pdf = luminance(color) / c.env_total_sum;
  float phi = (u + c.env_rotation) * TWO_PI;
  float theta = v * PI;
  float st = pmath::sin(theta);
  if (st <= EPS) pdf = 0.0f;
  V3 dir = normalize(V3(-st * pmath::cos(phi), st * pmath::sin(phi), pmath::cos(theta)));
  pdf = (pdf * (float)c.env_w * (float)c.env_h) / (TWO_PI * PI * st);
  return dir;
}

// env_map_eval.rcall.glsl:14-34 and env_sky_eval.rcall.glsl:12-15
static V3 eval_env(const Ctx& c, V3 dir, uint32_t depth, uint32_t flags, float state_pdf) {
  if (!c.env_map) {
    float a = std::fmax(dir.z, 0.0f);
    return mix(c.ground, c.sky, a) * c.env_intensity;
  }
  float theta = pmath::acos(dir.z);
  float u = -(PI + pmath::atan2(dir.y, dir.x)) * INV_TWO_PI - c.env_rotation;
  float v = theta * INV_PI;
  float mis = 1.0f;
  if (depth > 0 && (flags & RAY_FLAGS_SPECULAR) == 0) {
    float pdf = env_pdf(c, u, v, theta);
    mis = power_heuristic(state_pdf, pdf);
  }
  return mis * env_texel(c, env_texel_index(c, u, v)) * c.env_intensity;
}

// ---------------------------------------------------------------- lights
// inc/light/*.glsl. `nl` is num_of_lights (emission is scaled by it).
struct LightSample {
  V3 normal, emission, direction;
  float dist, pdf;
};
static LightSample sample_light(RNG& rng, const State& s, const Light& L, uint32_t nl) {
  LightSample o;
  float fn = (float)nl;
  switch (L.type) {
    case PT_LIGHT_POINT: {  // point.glsl:10-21
      V3 ld = L.position - s.first_hit_position;
      float d2 = dot(ld, ld);
      o.dist = std::sqrt(d2);
      ld = ld / o.dist;
      o.normal = -ld;
      o.emission = L.intensity * fn / d2;
      o.pdf = 1.0f;
      o.direction = ld;
      break;
    }
    case PT_LIGHT_DIRECTIONAL: {  // distant.glsl:10-35
      V3 dir = -L.u;
      float cos_alpha = L.v.x;
      if (cos_alpha > EPS) {
        V3 N = dir, T, B;
        onb(N, T, B);
        float r = rand1(rng);
        float phi = TWO_PI * rand1(rng);
        float z = (1.0f - r * (1.0f - cos_alpha));
        float radius = std::sqrt(1.0f - z * z);
        float x = radius * pmath::cos(phi);
        float y = radius * pmath::sin(phi);
        dir = to_world(T, B, N, V3(x, y, z));
      }
      o.normal = L.u;
      o.emission = L.intensity * fn;
      o.dist = WORLD_SIZE;
      o.pdf = 1.0f;
      o.direction = dir;
      break;
    }
    case PT_LIGHT_SPOT: {  // spot.glsl:10-21
      V3 ld = L.position - s.first_hit_position;
      float d2 = dot(ld, ld);
      o.dist = std::sqrt(d2);
      ld = ld / o.dist;
      o.normal = -ld;
      o.emission = smoothstepf(L.v.y, L.v.x, dot(-ld, L.u)) * L.intensity * fn / d2;
      o.pdf = 1.0f;
      o.direction = ld;
      break;
    }
    case PT_LIGHT_QUAD: {  // quad.glsl:10-34 (cos uses the unnormalised direction, as the reference)
      float r1 = rand1(rng);
      float r2 = rand1(rng);
      V3 lp = L.position + L.u * r1 + L.v * r2;
      V3 ld = lp - s.first_hit_position;
      o.normal = normalize(cross(L.v, L.u));
      float ct = dot(-ld, o.normal);
      if (ct < 0.0f) {
        o.emission = V3(0.0f);
        o.dist = 0.0f;
        o.pdf = 0.0f;
        o.direction = V3(0.0f);
        break;
      }
      float d2 = dot(ld, ld);
      o.dist = std::sqrt(d2);
      ld /= o.dist;
      o.emission = L.intensity * fn;
      o.pdf = d2 / (L.area * std::fabs(ct));
      o.direction = ld;
      break;
    }
    case PT_LIGHT_SPHERE: {  // sphere.glsl:10-42
      float r1 = rand1(rng);
      float r2 = rand1(rng);
      V3 cs = s.first_hit_position - L.position;
      float dc = length(cs);
      cs /= dc;
      if (dc < L.radius) {
        o.normal = cs;
        o.emission = V3(0.0f);
        o.dist = dc;
        o.pdf = 0.0f;
        o.direction = V3(0.0f);
        break;
      }
      V3 sd = uniform_sample_hemisphere(r1, r2);
      V3 T, B;
      onb(cs, T, B);
      sd = T * sd.x + B * sd.y + cs * sd.z;
      V3 lp = L.position + sd * L.radius;
      V3 ld = lp - s.first_hit_position;
      float d2 = dot(ld, ld);
      o.dist = std::sqrt(d2);
      ld = ld / o.dist;
      o.normal = normalize(lp - L.position);
      o.emission = L.intensity * fn;
      o.pdf = d2 / (L.area * 0.5f * std::fabs(dot(o.normal, ld)));
      o.direction = ld;
      break;
    }
    default: {
      o.normal = o.emission = o.direction = V3(0.0f);
      o.dist = 0.0f;
      o.pdf = 0.0f;
    }
  }
  return o;
}

// ---------------------------------------------------------------- BSDFs
// inc/bxdf/lambert.glsl:37-42
inline V3 lambert_eval(const Material& m, V3 N, V3 L, float& pdf) {
  float ndl = dot(N, L);
  pdf = ndl * INV_PI;
  return m.base_color * ndl * INV_PI;
}
// inc/bxdf/oren_nayar.glsl:7-51
inline V3 oren_nayar_f(const Material& m, V3 wo, V3 wi) {
  float sti = sin_theta(wi), sto = sin_theta(wo);
  float max_cos = 0.0f;
  if (sti > EPS && sto > EPS) {
    float spi = sin_phi(wi), cpi = cos_phi(wi);
    float spo = sin_phi(wo), cpo = cos_phi(wo);
    float dcos = cpi * cpo + spi * spo;
    max_cos = std::fmax(0.0f, dcos);
  }
  float sin_alpha, tan_beta;
  if (abs_cos_theta(wi) > abs_cos_theta(wo)) {
    sin_alpha = sto;
    tan_beta = sti / abs_cos_theta(wi);
  } else {
    sin_alpha = sti;
    tan_beta = sto / abs_cos_theta(wo);
  }
  float A = m.ax, B = m.ay;
  return m.base_color * INV_PI * (A + B * max_cos * sin_alpha * tan_beta);
}
inline V3 oren_nayar_eval(const State& s, const Material& m, V3 V, V3 N, V3 L, float& pdf) {
  L = to_local(s.tangent, s.bitangent, N, L);
  V = to_local(s.tangent, s.bitangent, N, V);
  pdf = L.z * INV_PI;
  return oren_nayar_f(m, V, L) * L.z;
}
// diffuse_bxdf_eval.rcall.glsl:15-20
inline V3 diffuse_eval(const State& s, const Material& m, V3 V, V3 N, V3 L, float& pdf) {
  if (m.roughness > EPS) return oren_nayar_eval(s, m, V, N, L, pdf);
  return lambert_eval(m, N, L, pdf);
}
// diffuse_bxdf_sample.rcall.glsl:15-38, lambert.glsl:15-27, oren_nayar.glsl:67-79
inline V3 diffuse_sample(RNG& rng, bool& ans, const State& s, const Material& m, V3 V, V3 N, V3& L,
                         float& pdf, uint32_t& flags) {
  float r1 = rand1(rng);
  float r2 = rand1(rng);
  L = cosine_sample_hemisphere(r1, r2);
  L = to_world(s.tangent, s.bitangent, N, L);
  ans = true;
  flags = RAY_FLAGS_REFLECTION;
  return diffuse_eval(s, m, V, N, L, pdf);
}

// inc/bxdf/disney.glsl
inline void tint_colors(V3 base, float spec_tint, float sheen_tint, float eta, float& F0,
                        V3& c_sheen, V3& c_spec0) {  // :9-32
  float lum = luminance(base);
  V3 ctint = lum > 0.0f ? base / lum : V3(1.0f);
  F0 = (1.0f - eta) / (1.0f + eta);
  F0 *= F0;
  c_spec0 = F0 * mix(V3(1.0f), ctint, spec_tint);
  c_sheen = mix(V3(1.0f), ctint, sheen_tint);
}
inline float diffuse_directional_albedo(float th, float ax, float ay, float e0) {  // :34-37
  return mixf(e0 + (1.0f - e0) * pmath::pow(std::fabs(1.0f - th), 5.0f), 0.04762f + 0.95238f * e0,
              1.0f - pmath::pow(std::fabs(1.0f - ax * ay), 5.0f));
}
inline float diffuse_average_albedo(float ax, float ay, float e0) {  // :39-41
  return e0 + (-0.33263f * ax * ay - 0.072359f) * (1.0f - e0) * e0;
}
inline float coupled_diffuse(float ax, float ay, float wi, float wo, float e0) {  // :43-48
  float Ewi = diffuse_directional_albedo(wi, ax, ay, e0);
  float Ewo = diffuse_directional_albedo(wo, ax, ay, e0);
  float Eavg = diffuse_average_albedo(ax, ay, e0);
  return (1.0f - Ewo) * (1.0f - Ewi) / (PI * (1.0f - Eavg));
}
inline float sheen_directional_albedo(float ct, float alpha) {  // :50-54
  float c = 1.0f - ct;
  float c3 = c * c * c;
  return 0.65584461f * c3 + 1.0f / (4.16526551f + pmath::exp(-7.97291361f * std::sqrt(alpha) + 6.33516894f));
}
inline V3 eval_disney_diffuse(float ax, float ay, float F0, float spec_tint, V3 base, float rough,
                              float subsurface, float sheen, V3 c_sheen, V3 V, V3 L, V3 H,
                              float& pdf) {  // :71-113
  pdf = 0.0f;
  if (L.z <= 0.0f) return V3(0.0f);
  float LdH = dot(L, H);
  float retro = 2.0f * rough * LdH * LdH;
  float fL = schlick_weight(L.z);
  float fV = schlick_weight(V.z);
  float f_retro = retro * (fL + fV + fL * fV * (retro - 1.0f));
  float f_d = (1.0f - 0.5f * fL) * (1.0f - 0.5f * fV);
  float coupled = coupled_diffuse(ax, ay, std::fabs(V.z), std::fabs(L.z), F0 * spec_tint);
  float f_ss90 = 0.5f * retro;
  float f_ss = mixf(1.0f, f_ss90, fL) * mixf(1.0f, f_ss90, fV);
  float ss = 1.25f * (f_ss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
  float fH = schlick_weight(LdH);
  V3 f_sheen = fH * sheen * c_sheen;
  float alpha = std::fmax(rough, 0.07f);
  alpha = alpha * alpha;
  float Ewi = max3(c_sheen) * sheen_directional_albedo(std::fabs(V.z), alpha);
  float Ewo = max3(c_sheen) * sheen_directional_albedo(std::fabs(L.z), alpha);
  float sheen_weight = std::fmin(1.0f - Ewi, 1.0f - Ewo);
  pdf = L.z * INV_PI;
  return INV_PI * base * mixf(f_d * coupled * PI + f_retro, ss, subsurface) + f_sheen * sheen_weight;
}
inline V3 eval_microfacet_reflection(float ax, float ay, V3 V, V3 L, V3 H, V3 F, float& pdf) {  // :124-143
  pdf = 0.0f;
  if (L.z <= 0.0f) return V3(0.0f);
  float D = gtr2_aniso(H.z, H.x, H.y, ax, ay);
  float G1 = smith_g_aniso(std::fabs(V.z), V.x, V.y, ax, ay);
  float G2 = G1 * smith_g_aniso(std::fabs(L.z), L.x, L.y, ax, ay);
  pdf = G1 * D / (4.0f * V.z);
  return F * D * G2 / (4.0f * L.z * V.z);
}
inline float specular_directional_albedo(float alpha, float ct) {  // :145-149
  return 1.0f - 1.45940f * alpha * (-0.20276f + alpha * (2.77203f + (-2.61748f + 0.73343f * alpha) * alpha)) *
                    ct * (3.09507f + ct * (-9.11368f + ct * (15.88844f + ct * (-13.70343f + 4.51786f * ct))));
}
inline float specular_average_albedo(float alpha) {  // :151-153
  return 1.0f + alpha * (-0.11304f + alpha * (-1.86947f + (2.22682f - 0.83397f * alpha) * alpha));
}
inline V3 eval_microfacet_ms(float ax, float ay, V3 V, V3 L, V3 F0) {  // :168-177
  float alpha = std::sqrt(ax * ay);
  float Ewi = specular_directional_albedo(alpha, std::fabs(V.z));
  float Ewo = specular_directional_albedo(alpha, std::fabs(L.z));
  float Eavg = specular_average_albedo(alpha);
  float ms = (1.0f - Ewo) * (1.0f - Ewi) / (PI * (1.0f - Eavg));
  V3 Favg = (20.0f / 21.0f) * F0 + (1.0f / 21.0f) * V3(1.0f);
  V3 f = (Favg * Favg * Eavg) / (V3(1.0f) - Favg * (1.0f - Eavg));
  return ms * f;
}
inline V3 eval_microfacet_refraction(float ax, float ay, V3 base, float eta, V3 V, V3 L, V3 H, V3 F,
                                     float& pdf) {  // :190-219
  pdf = 0.0f;
  if (L.z >= 0.0f) return V3(0.0f);
  float ldh = dot(L, H);
  float vdh = dot(V, H);
  float D = gtr2_aniso(H.z, H.x, H.y, ax, ay);
  float G1 = smith_g_aniso(std::fabs(V.z), V.x, V.y, ax, ay);
  float G2 = G1 * smith_g_aniso(std::fabs(L.z), L.x, L.y, ax, ay);
  float denom = ldh + vdh * eta;
  denom *= denom;
  float eta2 = eta * eta;
  float jac = std::fabs(ldh) / denom;
  pdf = G1 * std::fmax(0.0f, vdh) * D * jac / V.z;
  return V3(pmath::pow(base.x, 0.5f), pmath::pow(base.y, 0.5f), pmath::pow(base.z, 0.5f)) * (V3(1.0f) - F) * D * G2 * std::fabs(vdh) * jac * eta2 / std::fabs(L.z * V.z);
}
inline V3 eval_clearcoat(float ccr, V3 V, V3 L, V3 H, float& pdf) {  // :229-252
  pdf = 0.0f;
  if (L.z <= 0.0f) return V3(0.0f);
  float vdh = dot(V, H);
  float F = mixf(0.04f, 1.0f, schlick_weight(vdh));
  float D = gtr1(H.z, ccr);
  float G = smith_g(L.z, 0.25f) * smith_g(V.z, 0.25f);
  float jac = 1.0f / (4.0f * vdh);
  pdf = D * H.z * jac;
  return V3(F) * D * G;
}

struct LobeProbs {
  float F0;
  V3 c_sheen, c_spec0;
  float dielectric_wt, metal_wt, glass_wt;
  float diffuse_pr, dielectric_pr, metal_pr, glass_pr, clearcoat_pr;
};
inline LobeProbs lobe_probs(const Material& m, float eta, float Vz) {  // :300-331, :433-464
  LobeProbs p;
  tint_colors(m.base_color, m.specular_tint, m.sheen_tint, eta, p.F0, p.c_sheen, p.c_spec0);
  p.dielectric_wt = (1.0f - m.metallic) * (1.0f - m.specular_transmission);
  p.metal_wt = m.metallic;
  p.glass_wt = (1.0f - m.metallic) * m.specular_transmission;
  float sw = schlick_weight(Vz);
  p.diffuse_pr = p.dielectric_wt * luminance(m.base_color);
  p.dielectric_pr = p.dielectric_wt * luminance(mix(p.c_spec0, V3(1.0f), sw));
  p.metal_pr = p.metal_wt * luminance(mix(m.base_color, V3(1.0f), sw));
  p.glass_pr = p.glass_wt;
  p.clearcoat_pr = 0.25f * m.clearcoat;
  float inv = 1.0f / (p.diffuse_pr + p.dielectric_pr + p.metal_pr + p.glass_pr + p.clearcoat_pr);
  p.diffuse_pr *= inv;
  p.dielectric_pr *= inv;
  p.metal_pr *= inv;
  p.glass_pr *= inv;
  p.clearcoat_pr *= inv;
  return p;
}

// disney.glsl:264-390 (ROUGHNESS_REGULARIZE_EVAL on, make_shaders.yaml:4)
static V3 disney_eval(bool ans, const State& s, const Material& m, V3 V, V3 N, V3 L, float& pdf) {
  float ax = m.ax, ay = m.ay;
  if (s.depth > 0 && ans) {
    if (ax < 0.3f) ax = clampf(2.0f * ax, 0.1f, 0.3f);
    if (ay < 0.3f) ay = clampf(2.0f * ay, 0.1f, 0.3f);
  }
  pdf = 0.0f;
  V3 f(0.0f);
  V = to_local(s.tangent, s.bitangent, N, V);
  L = to_local(s.tangent, s.bitangent, N, L);
  V3 H;
  if (L.z > 0.0f) H = normalize(L + V);
  else H = normalize(L + V * s.eta);
  if (H.z < 0.0f) H = -H;
  LobeProbs p = lobe_probs(m, s.eta, V.z);
  bool refl = L.z * V.z > 0.0f;
  float tmp = 0.0f;
  float vdh = std::fabs(dot(V, H));
  if (p.diffuse_pr > 0.0f && refl) {
    f += eval_disney_diffuse(ax, ay, p.F0, m.specular_tint, m.base_color, m.roughness, m.subsurface,
                             m.sheen, p.c_sheen, V, L, H, tmp) * p.dielectric_wt;
    pdf += tmp * p.diffuse_pr;
  }
  if (p.dielectric_pr > 0.0f && refl) {
    float F = (dielectric_fresnel(vdh, s.eta) - p.F0) / (1.0f - p.F0);
    f += eval_microfacet_reflection(ax, ay, V, L, H, mix(p.c_spec0, V3(1.0f), F), tmp) * p.dielectric_wt;
    f += eval_microfacet_ms(ax, ay, V, L, p.c_spec0) * p.dielectric_wt;
    pdf += tmp * p.dielectric_pr;
  }
  if (p.metal_pr > 0.0f && refl) {
    V3 F = mix(m.base_color, V3(1.0f), schlick_weight(vdh));
    f += eval_microfacet_reflection(ax, ay, V, L, H, F, tmp) * p.metal_wt;
    f += eval_microfacet_ms(ax, ay, V, L, m.base_color) * p.metal_wt;
    pdf += tmp * p.metal_pr;
  }
  if (p.glass_pr > 0.0f) {
    float F = dielectric_fresnel(vdh, s.eta);
    if (refl) {
      f += eval_microfacet_reflection(ax, ay, V, L, H, V3(F), tmp) * p.glass_wt;
      f += eval_microfacet_ms(ax, ay, V, L, p.c_spec0) * p.glass_wt;
      pdf += tmp * p.glass_pr * F;
    } else {
      f += eval_microfacet_refraction(ax, ay, m.base_color, s.eta, V, L, H, V3(F), tmp) * p.glass_wt;
      pdf += tmp * p.glass_pr * (1.0f - F);
    }
  }
  if (p.clearcoat_pr > 0.0f && refl) {
    f += eval_clearcoat(m.clearcoat_roughness, V, L, H, tmp) * m.clearcoat_tint * 0.25f * m.clearcoat;
    pdf += tmp * p.clearcoat_pr;
  }
  return f * std::fabs(L.z);
}

// disney.glsl:405-531
static V3 disney_sample(RNG& rng, bool& ans, const State& s, const Material& m, V3 V, V3 N, V3& L,
                        float& pdf, uint32_t& flags) {
  float ax = m.ax, ay = m.ay;
  ans = true;
  pdf = 0.0f;
  float r1 = rand1(rng);
  float r2 = rand1(rng);
  V = to_local(s.tangent, s.bitangent, N, V);
  LobeProbs p = lobe_probs(m, s.eta, V.z);
  float cdf0 = p.diffuse_pr;
  float cdf1 = cdf0 + p.dielectric_pr;
  float cdf2 = cdf1 + p.metal_pr;
  float cdf3 = cdf2 + p.glass_pr;
  float r3 = rand1(rng);
  // flags bits 8..10 carry the sampled lobe (0 diffuse, 1 dielectric/metal,
  // 2 glass reflection, 3 glass refraction, 4 clearcoat) for the path hash
  if (r3 < cdf0) {
    L = cosine_sample_hemisphere(r1, r2);
    flags = RAY_FLAGS_REFLECTION;
  } else if (r3 < cdf2) {
    V3 H = sample_ggx_vndf(V, ax, ay, r1, r2);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect(-V, H));
    flags = RAY_FLAGS_REFLECTION | (1u << 8);
  } else if (r3 < cdf3) {
    V3 H = sample_ggx_vndf(V, ax, ay, r1, r2);
    float F = dielectric_fresnel(std::fabs(dot(V, H)), s.eta);
    if (H.z < 0.0f) H = -H;
    r3 = (r3 - cdf2) / (cdf3 - cdf2);
    if (r3 < F) {
      L = normalize(reflect(-V, H));
      flags = RAY_FLAGS_REFLECTION | (2u << 8);
    } else {
      L = normalize(refract(-V, H, s.eta));
      flags = RAY_FLAGS_TRANSMISSION | (3u << 8);
    }
  } else {
    V3 H = sample_gtr1(m.clearcoat_roughness, r1, r2);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect(-V, H));
    flags = RAY_FLAGS_REFLECTION | (4u << 8);
  }
  L = to_world(s.tangent, s.bitangent, N, L);
  V = to_world(s.tangent, s.bitangent, N, V);
  return disney_eval(ans, s, m, V, N, L, pdf);
}

inline V3 bsdf_eval(const State& s, const Material& m, bool ans, V3 V, V3 N, V3 L, float& pdf) {
  if (m.type == PT_MATERIAL_DISNEY) return disney_eval(ans, s, m, V, N, L, pdf);
  return diffuse_eval(s, m, V, N, L, pdf);
}
inline V3 bsdf_sample(RNG& rng, bool& ans, const State& s, const Material& m, V3 V, V3 N, V3& L,
                      float& pdf, uint32_t& flags) {
  if (m.type == PT_MATERIAL_DISNEY) return disney_sample(rng, ans, s, m, V, N, L, pdf, flags);
  return diffuse_sample(rng, ans, s, m, V, N, L, pdf, flags);
}

// ---------------------------------------------------------------- integrator
struct PathOut {
  V3 radiance, albedo, normal;
  uint32_t hash;
  uint32_t closest, shadow;
};

struct Tracer {
  const Ctx& c;
  RNG rng;
  State st;
  Ray ray;
  uint32_t hash = HASH_INIT;
  uint32_t n_closest = 0, n_shadow = 0;
  // optional record of every ray the path traces (or_trace_path_rays):
  // origin xyz, tmin, direction xyz, tmax, kind (0 closest, 1 any-hit), hit id / occluded, t
  std::vector<float>* rec = nullptr;

  explicit Tracer(const Ctx& cc) : c(cc) {}

  void record(const Ray& r, float tmax, uint32_t kind, uint32_t result, float t) {
    if (!rec) return;
    const float v[11] = {r.o.x, r.o.y, r.o.z, 0.0f, r.d.x, r.d.y, r.d.z, tmax, (float)kind, 0.0f, t};
    rec->insert(rec->end(), v, v + 11);
    std::memcpy(&(*rec)[rec->size() - 2], &result, 4);
  }

  Hit closest(const Ray& r) {
    ++n_closest;
    Hit h = trace_closest(c, r, 0.0f, WORLD_SIZE, c.force_brute);
    record(r, WORLD_SIZE, 0, h.id, h.t);
    return h;
  }

  // inc/lighting.glsl:7-61 (MEDIUM && VOL_MIS); draws from the main path RNG.
  V3 eval_transmittance(Ray r) {
    State ts;
    ts.flags = 0;
    ts.pdf = 1.0f;
    ts.eta = 1.0f;
    ts.material_index = INVALID_INDEX;
    V3 T(1.0f);
    for (int depth = 0; depth < (int)c.cfg.max_depth; ++depth) {
      ++n_shadow;
      Hit h = trace_closest(c, r, 0.0f, WORLD_SIZE, c.force_brute);
      record(r, WORLD_SIZE, 0, h.id, h.t);
      fill_state(c, r, h, ts);
      if ((ts.flags & RAY_FLAGS_HIT) == 0 || (ts.flags & RAY_FLAGS_IS_EMITTER) != 0) break;
      if (ts.material_index >= c.mats.size()) return V3(0.0f);
      const Material& m = c.mats[ts.material_index];
      bool transparent = false;
      if (c.use_transparent) transparent = m.opacity == 0.0f || rand1(rng) > m.opacity;
      bool refractive = (1.0f - m.metallic) * m.specular_transmission > 0.0f;
      if (!(transparent || refractive)) return V3(0.0f);
      if (dot(r.d, ts.normal) > 0.0f && m.medium.type != PT_MEDIUM_NONE) {
        V3 col = m.medium.type == PT_MEDIUM_ABSORB ? V3(1.0f) - m.medium.color : V3(1.0f);
        T *= vexp(-col * m.medium.density * ts.hit_distance);
      }
      r.o = ts.first_hit_position + r.d * EPS;
    }
    return T;
  }

  bool occluded(const Ray& r, float tmax) {
    ++n_shadow;
    const bool occ = trace_any(c, r, 0.0f, tmax, c.force_brute);
    record(r, tmax, 1, occ ? 1u : 0u, 0.0f);
    return occ;
  }

  // inc/lighting.glsl:69-244
  V3 direct_lighting(const Material& mat, bool is_surface, bool ans) {
    V3 Ld(0.0f), Li(0.0f);
    V3 scatter_pos = st.first_hit_position + st.ffnormal * EPS;
    if (c.env_map) {
      V3 em;
      float light_pdf;
      V3 light_dir = sample_env_map(c, rng, em, light_pdf);
      Li = em;
      Ray sr{scatter_pos, light_dir};
      if (light_pdf > 0.0f) {
        if (c.use_vol_mis) {
          V3 T = eval_transmittance(sr);
          bool vis = luminance(T) > 0.0f;
          hmix(hash, 0x40000000u | (vis ? 1u : 0u));
          if (vis) {
            Li *= T;
            float pdf = 0.0f;
            V3 f(0.0f);
            if (is_surface) {
              f = bsdf_eval(st, mat, ans, -ray.d, st.ffnormal, light_dir, pdf);
            } else {
              pdf = phase_hg(dot(-ray.d, light_dir), st.medium.anisotropy);
              f = V3(pdf);
            }
            if (pdf > 0.0f) {
              float w = power_heuristic(light_pdf, pdf);
              if (w > 0.0f) Ld += w * Li * f / light_pdf;
            }
          }
        } else {
          // The reference traces the shadow ray and adds the contribution
          // when it is visible; a zero contribution leaves Ld unchanged
          // either way, so it is not traced and not hashed (the GPU path
          // does the same).
          float pdf;
          V3 f = bsdf_eval(st, mat, ans, -ray.d, st.ffnormal, light_dir, pdf);
          V3 contrib(0.0f);
          if (pdf > 0.0f) {
            float w = power_heuristic(light_pdf, pdf);
            if (w > 0.0f) contrib = w * Li * f / light_pdf;
          }
          if (nonzero(contrib)) {
            bool occ = occluded(sr, WORLD_SIZE);
            hmix(hash, 0x40000000u | (occ ? 0u : 1u));
            if (!occ) Ld += contrib;
          }
        }
      }
    }
    uint32_t nl = (uint32_t)c.lights.size();
    if (nl > 0) {
      int li = (int)(rand1(rng) * (float)nl);
      Light L{};
      L.type = PT_LIGHT_POINT;  // out-of-range pick (rand == 1.0) reads an empty light
      if (li >= 0 && li < (int)nl) L = c.lights[li];
      LightSample ls = sample_light(rng, st, L, nl);
      Ray sr{scatter_pos, ls.direction};
      float light_pdf = ls.pdf;
      Li = ls.emission;
      if (light_pdf > 0.0f && dot(ls.direction, ls.normal) < 0.0f) {
        if (c.use_vol_mis) {
          V3 T = eval_transmittance(sr);
          bool vis = luminance(T) > 0.0f;
          hmix(hash, 0x50000000u | (vis ? 1u : 0u));
          if (vis) {
            Li *= T;
            float pdf = 0.0f;
            V3 f(0.0f);
            if (is_surface) {
              f = bsdf_eval(st, mat, ans, -ray.d, st.ffnormal, ls.direction, pdf);
            } else {
              pdf = phase_hg(dot(-ray.d, ls.direction), st.medium.anisotropy);
              f = V3(pdf);
            }
            if (pdf > 0.0f) {
              float w = 1.0f;
              if (L.area > 0.0f) w = power_heuristic(light_pdf, pdf);
              if (w > 0.0f) Ld += w * Li * f / light_pdf;
            }
          }
        } else {
          float pdf;
          V3 f = bsdf_eval(st, mat, ans, -ray.d, st.ffnormal, ls.direction, pdf);
          V3 contrib(0.0f);
          if (pdf > 0.0f) {
            float w = 1.0f;
            if (L.area > 0.0f) w = power_heuristic(light_pdf, pdf);
            if (w > 0.0f) contrib = w * Li * f / light_pdf;
          }
          if (nonzero(contrib)) {
            bool occ = occluded(sr, ls.dist - 2.0f * EPS);
            hmix(hash, 0x50000000u | (occ ? 0u : 1u));
            if (!occ) Ld += contrib;
          }
        }
      }
    }
    return Ld;
  }

  // perspective_ray.rcall.glsl:12-65, orthographic_ray.rcall.glsl:12-46
  void gen_camera_ray(uint32_t px, uint32_t py) {
    const Camera& cam = c.cams[c.camera_index < c.cams.size() ? c.camera_index : 0];
    float r[4];
    rand4blue(rng, c.blue_noise.empty() ? nullptr : c.blue_noise.data(), r);
    float r1 = 2.0f * r[0], r2 = 2.0f * r[1];
    float jx = r1 < 1.0f ? std::sqrt(r1) - 1.0f : 1.0f - std::sqrt(2.0f - r1);
    float jy = r2 < 1.0f ? std::sqrt(r2) - 1.0f : 1.0f - std::sqrt(2.0f - r2);
    float W = (float)c.cfg.width, Hh = (float)c.cfg.height;
    jx /= (W * 0.5f);
    jy /= (Hh * 0.5f);
    float sx = (float)px / W, sy = (Hh - (float)py) / Hh;
    float dx = (2.0f * sx - 1.0f) + jx;
    float dy = (2.0f * sy - 1.0f) + jy;
    if (cam.type == PT_CAMERA_ORTHOGRAPHIC) {
      ray.d = normalize(cam.forward);
      ray.o = cam.position + cam.right * (dx * cam.fd_or_xmag) + cam.up * (dy * cam.ap_or_ymag);
      return;
    }
    float scale = pmath::tan(cam.yfov * 0.5f);
    dx *= scale * W / Hh;
    dy *= scale;
    V3 rd = normalize(cam.right * dx + cam.up * dy + cam.forward);
    V3 fd = rd, fo = cam.position;
    float aperture = cam.ap_or_ymag;
    if (aperture > 0.0f) {
      V3 focal = cam.fd_or_xmag * rd;
      float c1 = r[2] * TWO_PI;
      float c2 = r[3] * aperture;
      V3 ap = (pmath::cos(c1) * cam.right + pmath::sin(c1) * cam.up) * std::sqrt(c2);
      fd = normalize(focal - ap);
      fo = fo + ap;
    }
    ray.d = fd;
    ray.o = fo;
  }

  // pathtracer.rgen.glsl:22-257
  PathOut run(uint32_t px, uint32_t py, uint32_t frame) {
    rng = rng_initialize(px, py, frame + c.cfg.seed);
    hash = HASH_INIT;
    n_closest = n_shadow = 0;
    gen_camera_ray(px, py);
    st = State();
    st.flags = 0;
    st.pdf = 1.0f;
    st.eta = 1.0f;
    st.material_index = INVALID_INDEX;
    st.medium.type = PT_MEDIUM_NONE;
    st.medium.density = 0.0f;
    st.medium.anisotropy = 1.0f;
    V3 radiance(0.0f), throughput(1.0f);
    bool in_medium = false, medium_sampled = false;
    bool ans = false;
    V3 albedo(0.0f), normal(0.0f, 0.0f, 1.0f);
    const uint32_t max_depth = c.cfg.max_depth, rr_depth = c.cfg.rr_depth;
    for (st.depth = 0;; st.depth++) {
      Hit h = closest(ray);
      fill_state(c, ray, h, st);
      hmix(hash, h.id);
      if ((st.flags & RAY_FLAGS_HIT) == 0) {
        radiance += throughput * eval_env(c, ray.d, st.depth, st.flags, st.pdf);
        if (st.depth == 0) {
          albedo = radiance;
          normal = -ray.d;
        }
        break;
      }
      if ((st.flags & RAY_FLAGS_IS_EMITTER) != 0) {
        const Light& L = c.lights[st.material_index];
        float light_pdf = st.tex_coord.x;
        float w = 1.0f;
        if (st.depth > 0) w = power_heuristic(st.pdf, light_pdf);
        radiance += w * L.intensity * throughput;
        break;
      }
      if (st.material_index == INVALID_INDEX || st.material_index >= c.mats.size()) {
        radiance = V3(0.7f, 0.0f, 0.7f);
        break;
      }
      Material mat = c.mats[st.material_index];
      st.eta = dot(ray.d, st.normal) < 0.0f ? (1.0f / mat.ior) : mat.ior;
      apply_maps(c, mat, st, ray.d);
      if (st.depth == 0) {
        albedo = mat.base_color;
        normal = st.normal;
      }
      radiance += throughput * mat.emission;
      if (c.use_medium) {
        medium_sampled = false;
        if (in_medium) {
          if (st.medium.type == PT_MEDIUM_ABSORB) {
            throughput *= vexp(-(V3(1.0f) - st.medium.color) * st.hit_distance * st.medium.density);
          } else if (st.medium.type == PT_MEDIUM_EMISSIVE) {
            radiance += st.medium.color * st.hit_distance * st.medium.density * throughput;
          } else {
            float sd = std::fmin(-pmath::log(rand1(rng)) / st.medium.density, st.hit_distance);
            medium_sampled = sd < st.hit_distance;
            if (medium_sampled) {
              hmix(hash, 0x70000001u);
              throughput *= st.medium.color;
              ray.o = ray.o + ray.d * sd;
              st.first_hit_position = ray.o;
              radiance += direct_lighting(mat, false, ans) * throughput;
              float q1 = rand1(rng);
              float q2 = rand1(rng);
              V3 sdir = sample_hg(-ray.d, st.medium.anisotropy, q1, q2);
              st.pdf = phase_hg(dot(-ray.d, sdir), st.medium.anisotropy);
              ray.d = sdir;
            }
          }
        }
      }
      if (!medium_sampled) {
        bool skip = false;
        if (c.use_transparent) {
          if (mat.opacity == 0.0f || rand1(rng) > mat.opacity) {
            st.depth--;  // uint: wraps at depth 0, which then ends the path below
            skip = true;
            hmix(hash, 0x71000000u);
          }
        }
        bool stop = false;
        if (!skip) {
          radiance += throughput * direct_lighting(mat, true, ans);
          V3 L;
          float pdf;
          uint32_t sflags = 0;
          V3 f = bsdf_sample(rng, ans, st, mat, -ray.d, st.ffnormal, L, pdf, sflags);
          ray.d = L;
          st.pdf = pdf;
          st.flags |= sflags & 0xFFu;
          hmix(hash, 0x60000000u | sflags);
          if (st.pdf > 0.0f) {
            throughput *= f / st.pdf;
          } else {
            hmix(hash, 0x61000000u);
            stop = true;
          }
        }
        if (stop) break;
        ray.o = st.first_hit_position + ray.d * EPS;
        if (c.use_medium) {
          if (dot(ray.d, st.normal) < 0.0f && mat.medium.type != PT_MEDIUM_NONE) {
            in_medium = true;
            st.medium = mat.medium;
          } else {
            in_medium = false;
            st.medium.type = PT_MEDIUM_NONE;
          }
        }
      }
      if (st.depth >= max_depth) break;
      if (st.depth >= rr_depth && rr_depth > 0) {
        float q = std::fmin(std::fmax(throughput.x, std::fmax(throughput.y, throughput.z)) + 0.001f, 0.95f);
        if (rand1(rng) > q) {
          hmix(hash, 0x72000000u);
          break;
        }
        throughput /= q;
      }
    }
    PathOut o;
    o.radiance = radiance;
    o.albedo = albedo;
    o.normal = normal;
    o.hash = hash;
    o.closest = n_closest;
    o.shadow = n_shadow;
    return o;
  }
};

static Material to_mat(const pt_material& m) {
  Material o;
  o.medium.color = v3(m.medium.color);
  o.medium.density = m.medium.density;
  o.medium.anisotropy = m.medium.anisotropy;
  o.medium.type = m.medium.type;
  o.base_color = v3(m.base_color);
  o.opacity = m.opacity;
  o.emission = v3(m.emission);
  o.anisotropic = m.anisotropic;
  o.metallic = m.metallic;
  o.roughness = m.roughness;
  o.subsurface = m.subsurface;
  o.specular_tint = m.specular_tint;
  o.sheen = m.sheen;
  o.sheen_tint = m.sheen_tint;
  o.clearcoat = m.clearcoat;
  o.clearcoat_roughness = m.clearcoat_roughness;
  o.clearcoat_tint = v3(m.clearcoat_tint);
  o.specular_transmission = m.specular_transmission;
  o.ior = m.ior;
  o.ax = m.ax;
  o.ay = m.ay;
  o.base_color_map = m.base_color_map_index;
  o.normal_map = m.normal_map_index;
  o.mr_map = m.metallic_roughness_map_index;
  o.emission_map = m.emission_map_index;
  o.type = m.type;
  return o;
}

// Upper-left 3x3 inverse transpose by cofactors (column-major input). The
// library's host code computes the same matrix with the same float ops.
static void normal_matrix(const float* T, float N[9]) {
  auto M = [&](int r, int c) { return T[c * 4 + r]; };
  float C00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
  float C01 = -(M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0));
  float C02 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
  float C10 = -(M(0, 1) * M(2, 2) - M(0, 2) * M(2, 1));
  float C11 = M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0);
  float C12 = -(M(0, 0) * M(2, 1) - M(0, 1) * M(2, 0));
  float C20 = M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1);
  float C21 = -(M(0, 0) * M(1, 2) - M(0, 2) * M(1, 0));
  float C22 = M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0);
  float det = M(0, 0) * C00 + M(0, 1) * C01 + M(0, 2) * C02;
  float C[9] = {C00, C01, C02, C10, C11, C12, C20, C21, C22};
  for (int i = 0; i < 9; ++i) N[i] = C[i] / det;  // row-major N[r*3+c]
}
inline V3 xform_point(const float* T, V3 p) {
  return V3(((T[0] * p.x + T[4] * p.y) + T[8] * p.z) + T[12],
            ((T[1] * p.x + T[5] * p.y) + T[9] * p.z) + T[13],
            ((T[2] * p.x + T[6] * p.y) + T[10] * p.z) + T[14]);
}
inline V3 xform_dir3(const float* N, V3 v) {
  return V3((N[0] * v.x + N[1] * v.y) + N[2] * v.z, (N[3] * v.x + N[4] * v.y) + N[5] * v.z,
            (N[6] * v.x + N[7] * v.y) + N[8] * v.z);
}

}  // namespace orc

using namespace orc;

static int nthreads(int t) {
  if (t > 0) return t;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

template <class F>
static void parallel_for(uint32_t n, int threads, F fn) {
  std::atomic<uint32_t> next{0};
  int T = nthreads(threads);
  std::vector<std::thread> ws;
  for (int t = 0; t < T; ++t)
    ws.emplace_back([&]() {
      for (;;) {
        uint32_t i = next.fetch_add(1);
        if (i >= n) break;
        fn(i);
      }
    });
  for (auto& w : ws) w.join();
}


struct or_ctx {
  Ctx c;
};

extern "C" {

or_ctx* or_create(const pt_tracer_config* cfg) {
  if (!cfg || cfg->width == 0 || cfg->height == 0) return nullptr;
  or_ctx* o = new or_ctx();
  o->c.cfg = *cfg;
  size_t n = (size_t)cfg->width * cfg->height * 4;
  o->c.accum.assign(n, 0.0f);
  o->c.albedo.assign(n, 0.0f);
  o->c.normal.assign(n, 0.0f);
  o->c.ground = V3(0.0f);
  o->c.sky = V3(0.0f);
  return o;
}
void or_destroy(or_ctx* c) { delete c; }

int or_set_scene(or_ctx* o, const pt_scene_desc* s) {
  if (!o || !s) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  c.tv0.clear(); c.te1.clear(); c.te2.clear(); c.tidx.clear(); c.tmat.clear();
  c.vnorm.clear(); c.vtan.clear(); c.vuv.clear();
  for (uint32_t pi = 0; pi < s->num_primitives; ++pi) {
    const pt_primitive& p = s->primitives[pi];
    if (p.num_indices % 3 != 0) return PT_ERR_INVALID_ARG;
    uint32_t vbase = (uint32_t)c.vnorm.size();
    float N[9];
    normal_matrix(p.transform, N);
    std::vector<V3> wp(p.num_vertices);
    for (uint32_t v = 0; v < p.num_vertices; ++v) {
      const float* q = p.vertices + 11 * (size_t)v;
      wp[v] = xform_point(p.transform, V3(q[0], q[1], q[2]));
      c.vnorm.push_back(xform_dir3(N, V3(q[3], q[4], q[5])));
      c.vtan.push_back(xform_dir3(N, V3(q[6], q[7], q[8])));
      c.vuv.push_back(V2(q[9], q[10]));
    }
    for (uint32_t t = 0; t < p.num_indices / 3; ++t) {
      uint32_t a = p.indices[3 * t], b = p.indices[3 * t + 1], d = p.indices[3 * t + 2];
      if (a >= p.num_vertices || b >= p.num_vertices || d >= p.num_vertices) return PT_ERR_INVALID_ARG;
      c.tv0.push_back(wp[a]);
      c.te1.push_back(wp[b] - wp[a]);
      c.te2.push_back(wp[d] - wp[a]);
      c.tidx.push_back(vbase + a);
      c.tidx.push_back(vbase + b);
      c.tidx.push_back(vbase + d);
      c.tmat.push_back(p.material_index);
    }
  }
  c.mats.clear();
  for (uint32_t i = 0; i < s->num_materials; ++i) c.mats.push_back(to_mat(s->materials[i]));
  c.texs.assign(s->num_textures, Texture{});
  for (uint32_t i = 0; i < s->num_textures; ++i) {
    const pt_texture& t = s->textures[i];
    if (!t.rgba || t.width == 0 || t.height == 0) return PT_ERR_INVALID_ARG;
    c.texs[i].w = t.width;
    c.texs[i].h = t.height;
    c.texs[i].rgba.assign(t.rgba, t.rgba + 4 * (size_t)t.width * t.height);
  }
  c.lights.clear();
  for (uint32_t i = 0; i < s->num_lights && i < PT_MAX_LIGHTS; ++i) {
    const pt_light& l = s->lights[i];
    Light L;
    L.intensity = v3(l.intensity);
    L.position = v3(l.position);
    L.u = v3(l.u);
    L.v = v3(l.v);
    L.radius = l.radius;
    L.area = l.area;
    L.type = l.type;
    c.lights.push_back(L);
  }
  c.cams.clear();
  for (uint32_t i = 0; i < s->num_cameras && i < PT_MAX_CAMERAS; ++i) {
    const pt_camera& k = s->cameras[i];
    Camera C;
    C.position = v3(k.position);
    C.right = v3(k.right);
    C.up = v3(k.up);
    C.forward = v3(k.forward);
    C.yfov = k.yfov;
    C.fd_or_xmag = k.focal_distance_or_xmag;
    C.ap_or_ymag = k.aperture_or_ymag;
    C.type = k.type;
    c.cams.push_back(C);
  }
  if (c.cams.empty()) return PT_ERR_INVALID_ARG;
  c.committed = false;
  return PT_OK;
}

int or_set_envmap(or_ctx* o, const float* rgb, uint32_t w, uint32_t h, float rot_deg) {
  if (!o) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  if (!rgb || w == 0 || h == 0) {
    c.env_map = false;
    return PT_OK;
  }
  c.env_map = true;
  c.env_rgb.assign(rgb, rgb + 3 * (size_t)w * h);
  c.env_w = w;
  c.env_h = h;
  c.env_rotation = rot_deg / 360.0f;
  c.committed = false;
  return PT_OK;
}
void or_set_ground_color(or_ctx* o, const float v[4]) { o->c.ground = V3(v[0], v[1], v[2]); }
void or_set_sky_color(or_ctx* o, const float v[4]) { o->c.sky = V3(v[0], v[1], v[2]); }
void or_set_env_intensity(or_ctx* o, float v) { o->c.env_intensity = v; o->c.committed = false; }
void or_set_exposure_value(or_ctx* o, float v) { o->c.exposure = v; }
void or_set_camera_index(or_ctx* o, uint32_t i) { o->c.camera_index = i; }

void or_set_blue_noise(or_ctx* o, const uint8_t* rgba8) {
  if (rgba8) o->c.blue_noise.assign(rgba8, rgba8 + 4 * 1024 * 1024);
  else o->c.blue_noise.clear();
}

int or_commit(or_ctx* o) {
  if (!o) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  c.use_medium = false;
  c.use_transparent = false;
  for (const Material& m : c.mats) {
    if (m.medium.type != PT_MEDIUM_NONE) c.use_medium = true;
    if (m.opacity < 1.0f) c.use_transparent = true;
  }
  c.use_vol_mis = c.use_medium;
  build_bvh(c);
  if (c.env_map) build_env_tables(c);
  c.committed = true;
  return PT_OK;
}
uint32_t or_features(const or_ctx* o) {
  uint32_t f = 0;
  if (o->c.use_medium) f |= PT_FEATURE_MEDIUM;
  if (o->c.use_vol_mis) f |= PT_FEATURE_VOL_MIS;
  if (o->c.use_transparent) f |= PT_FEATURE_TRANSPARENT;
  return f;
}

static int render_impl(or_ctx* o, uint32_t frames, int threads, bool fp64) {
  if (!o) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  if (!c.committed) return PT_ERR_STATE;
  const uint32_t W = c.cfg.width, H = c.cfg.height;
  uint64_t f0 = c.frame_index;
  uint32_t nf = frames;
  if (c.cfg.max_samples > 0) {
    if (f0 >= c.cfg.max_samples) nf = 0;
    else if (f0 + nf > c.cfg.max_samples) nf = (uint32_t)(c.cfg.max_samples - f0);
  }
  if (fp64 && c.accum64.size() != (size_t)W * H * 3) c.accum64.assign((size_t)W * H * 3, 0.0);
  c.n_paths = 0;
  c.n_closest = 0;
  c.n_shadow = 0;
  parallel_for(H, threads, [&](uint32_t y) {
    Tracer tr(c);
    uint64_t nc = 0, ns = 0;
    for (uint32_t x = 0; x < W; ++x) {
      size_t pix = (size_t)y * W + x;
      for (uint32_t k = 0; k < nf; ++k) {
        uint32_t f = (uint32_t)(f0 + k);
        PathOut p = tr.run(x, y, f);
        nc += p.closest;
        ns += p.shadow;
        float* a = &c.accum[4 * pix];
        float* b = &c.albedo[4 * pix];
        float* n = &c.normal[4 * pix];
        // pathtracer.rgen.glsl:259-278
        if (f == 0) {
          a[0] = p.radiance.x; a[1] = p.radiance.y; a[2] = p.radiance.z;
          b[0] = p.albedo.x; b[1] = p.albedo.y; b[2] = p.albedo.z;
          n[0] = p.normal.x; n[1] = p.normal.y; n[2] = p.normal.z;
        } else {
          float t = 1.0f / ((float)f + 1.0f);
          V3 na = mix(V3(a[0], a[1], a[2]), p.radiance, t);
          V3 nb = mix(V3(b[0], b[1], b[2]), p.albedo, t);
          V3 nn = mix(V3(n[0], n[1], n[2]), p.normal, t);
          a[0] = na.x; a[1] = na.y; a[2] = na.z;
          b[0] = nb.x; b[1] = nb.y; b[2] = nb.z;
          n[0] = nn.x; n[1] = nn.y; n[2] = nn.z;
        }
        a[3] = b[3] = n[3] = 1.0f;
        if (fp64) {
          double* s = &c.accum64[3 * pix];
          s[0] += (double)p.radiance.x;
          s[1] += (double)p.radiance.y;
          s[2] += (double)p.radiance.z;
        }
      }
    }
    c.n_paths += (uint64_t)W * nf;
    c.n_closest += nc;
    c.n_shadow += ns;
  });
  c.frame_index = f0 + nf;
  c.fp64_mode = fp64;
  return PT_OK;
}

int or_render(or_ctx* o, uint32_t frames, int threads) { return render_impl(o, frames, threads, false); }
int or_render_fp64(or_ctx* o, uint32_t frames, int threads) { return render_impl(o, frames, threads, true); }

void or_reset(or_ctx* o) {
  Ctx& c = o->c;
  c.frame_index = 0;
  std::fill(c.accum.begin(), c.accum.end(), 0.0f);
  std::fill(c.albedo.begin(), c.albedo.end(), 0.0f);
  std::fill(c.normal.begin(), c.normal.end(), 0.0f);
  c.accum64.clear();
  c.fp64_mode = false;
}

int or_read_image(or_ctx* o, int which, void* out, size_t bytes) {
  if (!o || !out) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  size_t np = (size_t)c.cfg.width * c.cfg.height;
  if (which == PT_IMAGE_FINAL) {
    if (bytes != np * 4) return PT_ERR_INVALID_ARG;
    uint8_t* p = (uint8_t*)out;
    for (size_t i = 0; i < np; ++i) {
      V3 a(c.accum[4 * i], c.accum[4 * i + 1], c.accum[4 * i + 2]);
      V3 f = finish_color(a, c.exposure, c.cfg.enable_tonemap != 0, c.cfg.enable_aces != 0,
                          c.cfg.use_simple_aces != 0);
      p[4 * i] = to_unorm8(f.x);
      p[4 * i + 1] = to_unorm8(f.y);
      p[4 * i + 2] = to_unorm8(f.z);
      p[4 * i + 3] = 255;
    }
    return PT_OK;
  }
  if (bytes != np * 16) return PT_ERR_INVALID_ARG;
  float* p = (float*)out;
  if (which == PT_IMAGE_ACCUM) {
    if (c.fp64_mode && c.frame_index > 0) {
      for (size_t i = 0; i < np; ++i) {
        for (int k = 0; k < 3; ++k) p[4 * i + k] = (float)(c.accum64[3 * i + k] / (double)c.frame_index);
        p[4 * i + 3] = 1.0f;
      }
    } else {
      std::memcpy(p, c.accum.data(), bytes);
    }
    return PT_OK;
  }
  if (which == PT_IMAGE_ALBEDO) { std::memcpy(p, c.albedo.data(), bytes); return PT_OK; }
  if (which == PT_IMAGE_NORMAL) { std::memcpy(p, c.normal.data(), bytes); return PT_OK; }
  return PT_ERR_INVALID_ARG;
}

int or_trace_paths(or_ctx* o, uint32_t first_frame, uint32_t nframes, const uint32_t* pixels,
                   uint32_t npix, float* rad, uint32_t* hash, int threads) {
  if (!o || !pixels) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  if (!c.committed) return PT_ERR_STATE;
  c.n_paths = (uint64_t)npix * nframes;
  c.n_closest = 0;
  c.n_shadow = 0;
  parallel_for(npix, threads, [&](uint32_t k) {
    Tracer tr(c);
    uint32_t pix = pixels[k];
    uint32_t x = pix % c.cfg.width, y = pix / c.cfg.width;
    uint64_t nc = 0, ns = 0;
    for (uint32_t f = 0; f < nframes; ++f) {
      PathOut p = tr.run(x, y, first_frame + f);
      size_t i = (size_t)f * npix + k;
      if (rad) { rad[3 * i] = p.radiance.x; rad[3 * i + 1] = p.radiance.y; rad[3 * i + 2] = p.radiance.z; }
      if (hash) hash[i] = p.hash;
      nc += p.closest;
      ns += p.shadow;
    }
    c.n_closest += nc;
    c.n_shadow += ns;
  });
  return PT_OK;
}

// Every ray of one path (pixel, frame), 11 floats each (see Tracer::record);
// *count receives the number of rays, at most `cap` are written.
int or_trace_path_rays(or_ctx* o, uint32_t pixel, uint32_t frame, float* out, uint32_t cap, uint32_t* count) {
  if (!o || !out || !count) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  if (!c.committed) return PT_ERR_STATE;
  std::vector<float> rec;
  Tracer tr(c);
  tr.rec = &rec;
  tr.run(pixel % c.cfg.width, pixel / c.cfg.width, frame);
  const uint32_t n = (uint32_t)(rec.size() / 11);
  *count = n;
  std::memcpy(out, rec.data(), sizeof(float) * 11 * std::min(n, cap));
  return PT_OK;
}

// Paths traced against every triangle (1) or through the BVH (0, default).
void or_set_brute(or_ctx* o, int brute) {
  if (o) o->c.force_brute = brute != 0;
}

int or_trace_rays(or_ctx* o, const float* rays, uint32_t n, int any_hit, int brute, uint32_t* hits,
                  int threads) {
  if (!o || !rays || !hits) return PT_ERR_INVALID_ARG;
  Ctx& c = o->c;
  if (!c.committed) return PT_ERR_STATE;
  parallel_for((n + 255) / 256, threads, [&](uint32_t blk) {
    for (uint32_t i = blk * 256; i < std::min(n, blk * 256 + 256); ++i) {
      const float* r = rays + 8 * (size_t)i;
      Ray ray{V3(r[0], r[1], r[2]), V3(r[4], r[5], r[6])};
      uint32_t* hOut = hits + 4 * (size_t)i;
      if (any_hit) {
        bool occ = trace_any(c, ray, r[3], r[7], brute != 0);
        float t = occ ? 0.0f : INF;
        std::memcpy(&hOut[0], &t, 4);
        hOut[1] = hOut[2] = 0;
        hOut[3] = occ ? 0u : HIT_MISS;
      } else {
        Hit h = trace_closest(c, ray, r[3], r[7], brute != 0);
        std::memcpy(&hOut[0], &h.t, 4);
        std::memcpy(&hOut[1], &h.u, 4);
        std::memcpy(&hOut[2], &h.v, 4);
        hOut[3] = h.id;
      }
    }
  });
  return PT_OK;
}

void or_counters(const or_ctx* o, uint64_t* p, uint64_t* cl, uint64_t* sh) {
  if (p) *p = o->c.n_paths;
  if (cl) *cl = o->c.n_closest;
  if (sh) *sh = o->c.n_shadow;
}

void or_pcg4d(uint32_t v[4]) {
  U4 u = {v[0], v[1], v[2], v[3]};
  pcg4d(u);
  v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
}
void or_rand_seq(uint32_t px, uint32_t py, uint32_t frame, uint32_t n, float* out) {
  RNG r = rng_initialize(px, py, frame);
  for (uint32_t i = 0; i < n; ++i) out[i] = rand1(r);
}
void or_blue_noise(uint32_t x, uint32_t y, float out[4]) { blue_noise_texel(x, y, out); }

static State kat_state(const float tbn[9], float eta, uint32_t depth) {
  State s;
  s.tangent = V3(tbn[0], tbn[1], tbn[2]);
  s.bitangent = V3(tbn[3], tbn[4], tbn[5]);
  s.normal = V3(tbn[6], tbn[7], tbn[8]);
  s.ffnormal = s.normal;
  s.eta = eta;
  s.depth = depth;
  return s;
}
void or_bsdf_eval(int kind, const pt_material* m, const float tbn[9], float eta, uint32_t depth,
                  int ans, const float V[3], const float N[3], const float L[3], float f_out[3],
                  float* pdf_out) {
  State s = kat_state(tbn, eta, depth);
  Material mm = to_mat(*m);
  mm.type = kind == 1 ? PT_MATERIAL_DISNEY : PT_MATERIAL_DIFFUSE;
  float pdf = 0.0f;
  V3 f = bsdf_eval(s, mm, ans != 0, v3(V), v3(N), v3(L), pdf);
  f_out[0] = f.x; f_out[1] = f.y; f_out[2] = f.z;
  *pdf_out = pdf;
}
void or_bsdf_sample(int kind, const pt_material* m, const float tbn[9], float eta, uint32_t depth,
                    int ans, const float V[3], const float N[3], uint32_t s0[4], float f_out[3],
                    float L_out[3], float* pdf_out, uint32_t* flags_out) {
  State s = kat_state(tbn, eta, depth);
  Material mm = to_mat(*m);
  mm.type = kind == 1 ? PT_MATERIAL_DISNEY : PT_MATERIAL_DIFFUSE;
  RNG r;
  r.s0 = {s0[0], s0[1], s0[2], s0[3]};
  r.s1 = {0, 0, 0, 0};
  r.px = r.py = 0;
  bool a = ans != 0;
  V3 L;
  float pdf = 0.0f;
  uint32_t flags = 0;
  V3 f = bsdf_sample(r, a, s, mm, v3(V), v3(N), L, pdf, flags);
  s0[0] = r.s0.x; s0[1] = r.s0.y; s0[2] = r.s0.z; s0[3] = r.s0.w;
  f_out[0] = f.x; f_out[1] = f.y; f_out[2] = f.z;
  L_out[0] = L.x; L_out[1] = L.y; L_out[2] = L.z;
  *pdf_out = pdf;
  *flags_out = flags;
}
void or_pmath(int fn, const float* x, const float* y, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = pmath::sin(x[i]); break;
      case 1: out[i] = pmath::cos(x[i]); break;
      case 2: out[i] = pmath::tan(x[i]); break;
      case 3: out[i] = pmath::exp(x[i]); break;
      case 4: out[i] = pmath::log(x[i]); break;
      case 5: out[i] = pmath::pow(x[i], y[i]); break;
      case 6: out[i] = pmath::acos(x[i]); break;
      default: out[i] = pmath::atan2(x[i], y[i]); break;
    }
  }
}

void or_tonemap(const float in[3], float ev, int enable, int aces, int simple, float out[3]) {
  V3 c = finish_color(v3(in), ev, enable != 0, aces != 0, simple != 0);
  out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

}  // extern "C"
