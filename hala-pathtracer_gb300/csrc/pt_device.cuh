// pt_device.cuh -- device-side shading math of the GB300 wavefront tracer.
//
// Every function restates the reference GLSL it names (paths relative to
// shaders/src/ of hala-pathtracer). Operation order follows the GLSL so the
// CPU oracle and this code round the same way: plain IEEE arithmetic (this
// code is compiled without FMA contraction), correctly rounded division and
// square root, and the portable transcendental functions below.
#pragma once
#include <cstdint>

#include "pt_types.h"

namespace hpt {

// common/common.glsl:6-15, inc/constants.glsl:6-12
constexpr float PI = 3.14159265358979323846f;
constexpr float TWO_PI = 2.0f * PI;
constexpr float INV_PI = 1.0f / PI;
constexpr float INV_TWO_PI = 1.0f / TWO_PI;
constexpr float FOUR_PI = 4.0f * PI;
constexpr float INV_FOUR_PI = 1.0f / FOUR_PI;
constexpr float EPS = 0.0003f;
constexpr float INF = 1000000.0f;
constexpr float WORLD_SIZE = 10000.0f;

constexpr uint32_t RAY_FLAGS_HIT = 0x1u;
constexpr uint32_t RAY_FLAGS_IS_EMITTER = 0x2u;
constexpr uint32_t RAY_FLAGS_SPECULAR = 0x4u;
constexpr uint32_t RAY_FLAGS_REFLECTION = 0x8u;
constexpr uint32_t RAY_FLAGS_TRANSMISSION = 0x10u;

// ------------------------------------------------------------------ portable math
// float32 sin/cos/tan/exp/log/pow/acos/atan2 with a fixed operation order
// (explicit fused multiply-adds only): Cody-Waite argument reduction with
// three-part constants, then polynomial kernels fitted by iteratively
// reweighted least squares in relative error and rounded to float32. The CPU
// oracle evaluates the same algorithm, so both round identically; accuracy
// against 40-digit references: <= 1.5 ulp (sin, cos, exp, log, acos),
// <= 2.6 ulp (tan, atan2), pow = exp(y log x) within GLSL's pow precision.
constexpr float PM_TWO_OVER_PI = 0.6366197466850281f;
constexpr float PM_PIO2_HI = 1.5707963705062866f, PM_PIO2_MID = -4.371138828673793e-08f,
                PM_PIO2_LO = -1.7151245100058819e-15f;
constexpr float PM_PIO4_HI = 0.7853981852531433f, PM_PIO4_MID = -2.1855694143368964e-08f;
constexpr float PM_PI_HI = 3.1415927410125732f, PM_PI_MID = -8.742277657347586e-08f;
constexpr float PM_LOG2E = 1.4426950216293335f;
constexpr float PM_LN2_HI = 0.6931471824645996f, PM_LN2_MID = -1.9046542121259336e-09f;

__device__ __forceinline__ void pm_sincos(float x, float& s, float& c) {
  if (!(fabsf(x) <= 1.0e6f)) {
    s = c = __int_as_float(0x7fc00000);
    return;
  }
  float k = rintf(x * PM_TWO_OVER_PI);
  float r = fmaf(-k, PM_PIO2_HI, x);
  r = fmaf(-k, PM_PIO2_MID, r);
  r = fmaf(-k, PM_PIO2_LO, r);
  int q = (int)k;
  float z = r * r;
  float sp = fmaf(fmaf(fmaf(2.7249013783148257e-06f, z, -0.00019840076856780797f), z, 0.008333331905305386f), z,
                  -0.1666666716337204f);
  float sr = fmaf(r * z, sp, r);
  float cp = fmaf(fmaf(fmaf(-2.730170649556385e-07f, z, 2.480060538800899e-05f), z, -0.00138888880610466f), z,
                  0.0416666679084301f);
  float cr = fmaf(z * z, cp, fmaf(-0.5f, z, 1.0f));
  switch (q & 3) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
  }
}
__device__ __forceinline__ float pm_sin(float x) { float s, c; pm_sincos(x, s, c); return s; }
__device__ __forceinline__ float pm_cos(float x) { float s, c; pm_sincos(x, s, c); return c; }
__device__ __forceinline__ float pm_tan(float x) { float s, c; pm_sincos(x, s, c); return s / c; }

__device__ __forceinline__ float pm_exp(float x) {
  if (x != x) return x;
  if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
  if (x < -103.97208404541016f) return 0.0f;
  float k = rintf(x * PM_LOG2E);
  float r = fmaf(-k, PM_LN2_HI, x);
  r = fmaf(-k, PM_LN2_MID, r);
  float p = fmaf(fmaf(fmaf(fmaf(fmaf(0.00019924867956433445f, r, 0.0013933534501120448f), r, 0.008333264850080013f), r,
                           0.041666463017463684f), r, 0.1666666716337204f), r, 0.5f);
  float er = fmaf(r * r, p, r) + 1.0f;
  int ki = (int)k;
  int k1 = ki / 2, k2 = ki - k1;
  return (er * __uint_as_float((uint32_t)(k1 + 127) << 23)) * __uint_as_float((uint32_t)(k2 + 127) << 23);
}

__device__ __forceinline__ float pm_log(float x) {
  if (x != x || x < 0.0f) return __int_as_float(0x7fc00000);
  if (x == 0.0f) return __int_as_float(0xff800000);
  if (x == __int_as_float(0x7f800000)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) {
    x *= 8388608.0f;
    e = -23;
  }
  uint32_t b = __float_as_uint(x);
  e += (int)((b >> 23) & 0xffu) - 127;
  float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) {
    m *= 0.5f;
    e += 1;
  }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float p = fmaf(fmaf(fmaf(0.23334167897701263f, z, 0.28550657629966736f), z, 0.4000012278556824f), z,
                 0.6666666865348816f);
  float lm = fmaf(-s, fmaf(-z, p, f), f);
  float fe = (float)e;
  return fmaf(fe, PM_LN2_HI, fmaf(fe, PM_LN2_MID, lm));
}

__device__ __forceinline__ float pm_pow(float x, float y) {
  if (y == 0.0f || x == 1.0f) return 1.0f;
  if (x != x || y != y || x < 0.0f) return __int_as_float(0x7fc00000);
  if (x == 0.0f) return y > 0.0f ? 0.0f : __int_as_float(0x7f800000);
  return pm_exp(y * pm_log(x));
}

__device__ __forceinline__ float pm_asin_k(float x) {
  float z = x * x;
  float p = fmaf(fmaf(fmaf(fmaf(fmaf(0.034081507474184036f, z, 0.01690877228975296f), z, 0.031152866780757904f), z,
                           0.044594623148441315f), z, 0.07500111311674118f), z, 0.1666666567325592f);
  return fmaf(x * z, p, x);
}
__device__ __forceinline__ float pm_acos(float x) {
  if (x != x || fabsf(x) > 1.0f) return __int_as_float(0x7fc00000);
  if (fabsf(x) <= 0.5f) return PM_PIO2_HI - (pm_asin_k(x) - PM_PIO2_MID);
  if (x > 0.0f) return 2.0f * pm_asin_k(sqrtf((1.0f - x) * 0.5f));
  return PM_PI_HI - (2.0f * pm_asin_k(sqrtf((1.0f + x) * 0.5f)) - PM_PI_MID);
}

__device__ __forceinline__ float pm_atan_k(float t) {
  float z = t * t;
  float p = fmaf(fmaf(fmaf(fmaf(fmaf(0.05074314400553703f, z, -0.08635549992322922f), z, 0.11072912812232971f), z,
                           -0.1428423672914505f), z, 0.19999979436397552f), z, -0.3333333432674408f);
  return fmaf(t * z, p, t);
}
__device__ __forceinline__ float pm_atan2(float y, float x) {
  if (x != x || y != y) return __int_as_float(0x7fc00000);
  float ax = fabsf(x), ay = fabsf(y);
  float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  float r;
  if (mx == 0.0f) {
    r = 0.0f;
  } else {
    float t = (mx == __int_as_float(0x7f800000)) ? (mn == mx ? 1.0f : 0.0f) : mn / mx;
    if (t > 0.41421356f) r = PM_PIO4_HI + (pm_atan_k((t - 1.0f) / (t + 1.0f)) + PM_PIO4_MID);
    else r = pm_atan_k(t);
  }
  if (ay > ax) r = (PM_PIO2_HI - r) + PM_PIO2_MID;
  if (x < 0.0f) r = (PM_PI_HI - r) + PM_PI_MID;
  return (y < 0.0f) ? -r : r;
}

// ------------------------------------------------------------------ float3
__device__ __forceinline__ float3 f3(float s) { return make_float3(s, s, s); }
__device__ __forceinline__ float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ void operator+=(float3& a, float3 b) { a = a + b; }
__device__ __forceinline__ void operator*=(float3& a, float3 b) { a = a * b; }
__device__ __forceinline__ void operator*=(float3& a, float s) { a = a * s; }
__device__ __forceinline__ void operator/=(float3& a, float s) { a = a / s; }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float3 mix(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float3 clamp3(float3 v, float lo, float hi) {
  return make_float3(clampf(v.x, lo, hi), clampf(v.y, lo, hi), clampf(v.z, lo, hi));
}
__device__ __forceinline__ float3 vexp(float3 v) { return make_float3(pm_exp(v.x), pm_exp(v.y), pm_exp(v.z)); }
__device__ __forceinline__ float max3(float3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - 2.0f * dot(n, i) * n; }
__device__ __forceinline__ float3 refract3(float3 i, float3 n, float eta) {
  float d = dot(n, i);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return f3(0.0f);
  return eta * i - (eta * d + sqrtf(k)) * n;
}
__device__ __forceinline__ float luminance(float3 c) {  // common/common.glsl:69-71
  return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z;
}
__device__ __forceinline__ float3 to_world(float3 X, float3 Y, float3 Z, float3 v) {
  return v.x * X + v.y * Y + v.z * Z;
}
__device__ __forceinline__ float3 to_local(float3 X, float3 Y, float3 Z, float3 v) {
  return make_float3(dot(v, X), dot(v, Y), dot(v, Z));
}

// ------------------------------------------------------------------ hashing
// Hit-sequence hash, FNV-1a over event words (same events as the oracle).
constexpr uint32_t HASH_INIT = 2166136261u;
__device__ __forceinline__ void hmix(uint32_t& h, uint32_t x) { h = (h ^ x) * 16777619u; }

// ------------------------------------------------------------------ RNG
// common/wltcRS.glsl:9-53
__device__ __forceinline__ void pcg4d(uint4& v) {
  v.x = v.x * 1664525u + 1013904223u;
  v.y = v.y * 1664525u + 1013904223u;
  v.z = v.z * 1664525u + 1013904223u;
  v.w = v.w * 1664525u + 1013904223u;
  v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
  v.x ^= v.x >> 16u; v.y ^= v.y >> 16u; v.z ^= v.z >> 16u; v.w ^= v.w >> 16u;
  v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
}
// float(u) / float(0xffffffffu) == rn(u) * 2^-32 exactly; may equal 1.0.
__device__ __forceinline__ float u2f(uint32_t u) { return __uint2float_rn(u) * 2.3283064365386963e-10f; }
__device__ __forceinline__ float rand1(uint4& s) { pcg4d(s); return u2f(s.x); }
__device__ __forceinline__ float2 rand2(uint4& s) { pcg4d(s); return make_float2(u2f(s.x), u2f(s.y)); }
__device__ __forceinline__ uint4 rng_seed_s0(uint32_t px, uint32_t py, uint32_t frame) {
  return make_uint4(px, py, frame, px + py);
}
__device__ __forceinline__ uint4 rng_seed_s1(uint32_t frame) {
  return make_uint4(frame, frame * 15843u, frame * 31u + 4566u, frame * 2345u + 58585u);
}
// Blue-noise substitute: RGBA8 texel = top bytes of pcg4d(x, y, 0x2545F491, 0x9E3779B9).
__device__ __forceinline__ float4 blue_noise_texel(uint32_t x, uint32_t y) {
  uint4 v = make_uint4(x, y, 0x2545F491u, 0x9E3779B9u);
  pcg4d(v);
  return make_float4((float)(v.x >> 24) / 255.0f, (float)(v.y >> 24) / 255.0f,
                     (float)(v.z >> 24) / 255.0f, (float)(v.w >> 24) / 255.0f);
}
// shift2 + rand4blue, wltcRS.glsl:43-53: texelFetch of the loaded RGBA8
// texture (UNORM: byte / 255), or the substitute when none is loaded
__device__ __forceinline__ float4 rand4blue(uint4& s1, int px, int py, const uchar4* tex) {
  pcg4d(s1);
  int sx = (px + (int)(s1.x % 0x0fffffffu)) % 1024;
  int sy = (py + (int)(s1.y % 0x0fffffffu)) % 1024;
  if (tex) {
    const uchar4 t = tex[(uint32_t)sy * 1024u + (uint32_t)sx];
    return make_float4((float)t.x / 255.0f, (float)t.y / 255.0f, (float)t.z / 255.0f, (float)t.w / 255.0f);
  }
  return blue_noise_texel((uint32_t)sx, (uint32_t)sy);
}

// ------------------------------------------------------------------ sampling utils
// common/common.glsl:79-186, common/sampling.glsl
__device__ __forceinline__ float sin2_theta(float3 w) { return fmaxf(0.0f, 1.0f - w.z * w.z); }
__device__ __forceinline__ float sin_theta(float3 w) { return sqrtf(sin2_theta(w)); }
__device__ __forceinline__ float abs_cos_theta(float3 w) { return fabsf(w.z); }
__device__ __forceinline__ float cos_phi(float3 w) {
  float st = sin_theta(w);
  return (st == 0.0f) ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
__device__ __forceinline__ float sin_phi(float3 w) {
  float st = sin_theta(w);
  return (st == 0.0f) ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}
__device__ __forceinline__ float gtr1(float ndh, float a) {  // sampling.glsl:8-18
  if (a >= 1.0f) return INV_PI;
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * ndh * ndh;
  return (a2 - 1.0f) / (PI * pm_log(a2) * t);
}
// sampling.glsl:25-44 (y = sin*sin as the reference)
__device__ __forceinline__ float3 sample_gtr1(float roughness, float r1, float r2) {
  float a = fmaxf(0.001f, roughness);
  float a2 = a * a;
  float phi = r1 * TWO_PI;
  float ct = sqrtf((1.0f - pm_pow(a2, 1.0f - r2)) / (1.0f - a2));
  float st = clampf(sqrtf(1.0f - (ct * ct)), 0.0f, 1.0f);
  float cp = pm_cos(phi);
  return make_float3(st * cp, st * st, ct);
}
// sampling.glsl:120-136
__device__ __forceinline__ float3 sample_ggx_vndf(float3 wi, float ax, float ay, float r1, float r2) {
  float3 wiStd = normalize(make_float3(wi.x * ax, wi.y * ay, wi.z));
  float phi = (2.0f * r1 - 1.0f) * PI;
  float z = fmaf((1.0f - r2), (1.0f + wiStd.z), -wiStd.z);
  float sinTheta = sqrtf(clampf(1.0f - z * z, 0.0f, 1.0f));
  float x = sinTheta * pm_cos(phi);
  float y = sinTheta * pm_sin(phi);
  float3 wmStd = make_float3(x, y, z) + wiStd;
  return normalize(make_float3(wmStd.x * ax, wmStd.y * ay, wmStd.z));
}
__device__ __forceinline__ float gtr2_aniso(float ndh, float hdx, float hdy, float ax, float ay) {
  float a = hdx / ax;
  float b = hdy / ay;
  float c = a * a + b * b + ndh * ndh;
  return 1.0f / (PI * ax * ay * c * c);
}
__device__ __forceinline__ float smith_g(float ndv, float alpha_g) {
  float a = alpha_g * alpha_g;
  float b = ndv * ndv;
  return (2.0f * ndv) / (ndv + sqrtf(a + b - a * b));
}
__device__ __forceinline__ float smith_g_aniso(float ndv, float vdx, float vdy, float ax, float ay) {
  float a = vdx * ax;
  float b = vdy * ay;
  float c = ndv;
  return (2.0f * ndv) / (ndv + sqrtf(a * a + b * b + c * c));
}
__device__ __forceinline__ float schlick_weight(float u) {
  float m = clampf(1.0f - u, 0.0f, 1.0f);
  float m2 = m * m;
  return m2 * m2 * m;
}
__device__ __forceinline__ float dielectric_fresnel(float cos_i, float eta) {
  float s2 = eta * eta * (1.0f - cos_i * cos_i);
  if (s2 > 1.0f) return 1.0f;
  float ct = sqrtf(fmaxf(1.0f - s2, 0.0f));
  float rs = (eta * ct - cos_i) / (eta * ct + cos_i);
  float rp = (eta * cos_i - ct) / (eta * cos_i + ct);
  return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ float3 cosine_sample_hemisphere(float r1, float r2) {
  float r = sqrtf(r1);
  float phi = TWO_PI * r2;
  float x = r * pm_cos(phi);
  float y = r * pm_sin(phi);
  float z = sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y));
  return make_float3(x, y, z);
}
__device__ __forceinline__ float3 uniform_sample_hemisphere(float r1, float r2) {
  float r = sqrtf(fmaxf(0.0f, 1.0f - r1 * r1));
  float phi = TWO_PI * r2;
  return make_float3(r * pm_cos(phi), r * pm_sin(phi), r1);
}
__device__ __forceinline__ float power_heuristic(float a, float b) {
  a *= a;
  b *= b;
  return a / (a + b);
}
__device__ __forceinline__ void onb(float3 N, float3& T, float3& B) {
  float3 up = fabsf(N.z) < 0.9999999f ? make_float3(0, 0, 1) : make_float3(1, 0, 0);
  T = normalize(cross(up, N));
  B = cross(N, T);
}
__device__ __forceinline__ float3 sample_hg(float3 V, float g, float r1, float r2) {
  float ct;
  if (fabsf(g) < 0.001f) {
    ct = 1.0f - 2.0f * r2;
  } else {
    float sq = (1.0f - g * g) / (1.0f + g - 2.0f * g * r2);
    ct = -(1.0f + g * g - sq * sq) / (2.0f * g);
  }
  float phi = r1 * TWO_PI;
  float st = clampf(sqrtf(1.0f - (ct * ct)), 0.0f, 1.0f);
  float sp = pm_sin(phi);
  float cp = pm_cos(phi);
  float3 v1, v2;
  onb(V, v1, v2);
  return st * cp * v1 + st * sp * v2 + ct * V;
}
__device__ __forceinline__ float phase_hg(float ct, float g) {
  float denom = fmaxf(1.0f + g * g + 2.0f * g * ct, EPS);
  return INV_FOUR_PI * (1.0f - g * g) / (denom * sqrtf(denom));
}

// ------------------------------------------------------------------ tonemap
// common/tonemap.glsl, common/common.glsl:26-39, pathtracer.rgen.glsl:280-301
__device__ __forceinline__ float linear_2_srgb(float x) {
  if (x <= 0.0031308f) return 12.92f * x;
  return 1.055f * pm_pow(x, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ float3 aces_fitted(float3 c) {
  const float3 i0 = f3(0.59719f, 0.35458f, 0.04823f), i1 = f3(0.07600f, 0.90834f, 0.01566f),
               i2 = f3(0.02840f, 0.13383f, 0.83777f);
  const float3 o0 = f3(1.60475f, -0.53108f, -0.07367f), o1 = f3(-0.10208f, 1.10813f, -0.00605f),
               o2 = f3(-0.00327f, -0.07276f, 1.07602f);
  c = make_float3(dot(c, i0), dot(c, i1), dot(c, i2));
  float3 a = c * (c + f3(0.0245786f)) - f3(0.000090537f);
  float3 b = c * (0.983729f * c + f3(0.4329510f)) + f3(0.238081f);
  c = a / b;
  c = make_float3(dot(c, o0), dot(c, o1), dot(c, o2));
  return clamp3(c, 0.0f, 1.0f);
}
__device__ __forceinline__ float3 aces_simple(float3 c) {
  const float a = 2.51f, b = 0.03f, y = 2.43f, d = 0.59f, e = 0.14f;
  return clamp3((c * (a * c + f3(b))) / (c * (y * c + f3(d)) + f3(e)), 0.0f, 1.0f);
}
__device__ __forceinline__ float3 finish_color(float3 c, float ev, bool enable, bool aces, bool simple) {
  float exposure = pm_pow(2.0f, ev);
  c = c * exposure;
  if (enable) {
    if (aces) c = simple ? aces_simple(c) : aces_fitted(c);
    else c = c * 1.0f / (1.0f + luminance(c) / 1.5f);
  }
  return make_float3(linear_2_srgb(c.x), linear_2_srgb(c.y), linear_2_srgb(c.z));
}
__device__ __forceinline__ unsigned char to_unorm8(float x) {
  float c = clampf(x, 0.0f, 1.0f);
  if (!(c == c)) c = 0.0f;
  return (unsigned char)floorf(c * 255.0f + 0.5f);
}

// ------------------------------------------------------------------ BSDFs
struct ShadeFrame {  // the State fields a BSDF reads (inc/types.glsl:129-145)
  float3 tangent, bitangent;
  float eta;
  uint32_t depth;
};

// inc/bxdf/lambert.glsl:37-42
__device__ __forceinline__ float3 lambert_eval(const pt_material& m, float3 N, float3 L, float& pdf) {
  float ndl = dot(N, L);
  pdf = ndl * INV_PI;
  return f3(m.base_color) * ndl * INV_PI;
}
// inc/bxdf/oren_nayar.glsl:7-51, 103-117
__device__ __forceinline__ float3 oren_nayar_eval(const ShadeFrame& s, const pt_material& m, float3 V,
                                                  float3 N, float3 L, float& pdf) {
  float3 wi = to_local(s.tangent, s.bitangent, N, L);
  float3 wo = to_local(s.tangent, s.bitangent, N, V);
  pdf = wi.z * INV_PI;
  float sti = sin_theta(wi), sto = sin_theta(wo);
  float max_cos = 0.0f;
  if (sti > EPS && sto > EPS) {
    float spi = sin_phi(wi), cpi = cos_phi(wi);
    float spo = sin_phi(wo), cpo = cos_phi(wo);
    float dcos = cpi * cpo + spi * spo;
    max_cos = fmaxf(0.0f, dcos);
  }
  float sin_alpha, tan_beta;
  if (abs_cos_theta(wi) > abs_cos_theta(wo)) {
    sin_alpha = sto;
    tan_beta = sti / abs_cos_theta(wi);
  } else {
    sin_alpha = sti;
    tan_beta = sto / abs_cos_theta(wo);
  }
  float3 f = f3(m.base_color) * INV_PI * (m.ax + m.ay * max_cos * sin_alpha * tan_beta);
  return f * wi.z;
}
// diffuse_bxdf_eval.rcall.glsl:15-20
__device__ __forceinline__ float3 diffuse_eval(const ShadeFrame& s, const pt_material& m, float3 V, float3 N,
                                               float3 L, float& pdf) {
  if (m.roughness > EPS) return oren_nayar_eval(s, m, V, N, L, pdf);
  return lambert_eval(m, N, L, pdf);
}
// diffuse_bxdf_sample.rcall.glsl, lambert.glsl:15-27, oren_nayar.glsl:67-79
__device__ __forceinline__ float3 diffuse_sample(uint4& rng, bool& ans, const ShadeFrame& s, const pt_material& m,
                                                 float3 V, float3 N, float3& L, float& pdf, uint32_t& flags) {
  float r1 = rand1(rng);
  float r2 = rand1(rng);
  L = cosine_sample_hemisphere(r1, r2);
  L = to_world(s.tangent, s.bitangent, N, L);
  ans = true;
  flags = RAY_FLAGS_REFLECTION;
  return diffuse_eval(s, m, V, N, L, pdf);
}

// inc/bxdf/disney.glsl
__device__ __forceinline__ float diffuse_directional_albedo(float th, float ax, float ay, float e0) {
  return mixf(e0 + (1.0f - e0) * pm_pow(fabsf(1.0f - th), 5.0f), 0.04762f + 0.95238f * e0,
              1.0f - pm_pow(fabsf(1.0f - ax * ay), 5.0f));
}
__device__ __forceinline__ float coupled_diffuse(float ax, float ay, float wi, float wo, float e0) {
  float Ewi = diffuse_directional_albedo(wi, ax, ay, e0);
  float Ewo = diffuse_directional_albedo(wo, ax, ay, e0);
  float Eavg = e0 + (-0.33263f * ax * ay - 0.072359f) * (1.0f - e0) * e0;
  return (1.0f - Ewo) * (1.0f - Ewi) / (PI * (1.0f - Eavg));
}
__device__ __forceinline__ float sheen_directional_albedo(float ct, float alpha) {
  float c = 1.0f - ct;
  float c3 = c * c * c;
  return 0.65584461f * c3 + 1.0f / (4.16526551f + pm_exp(-7.97291361f * sqrtf(alpha) + 6.33516894f));
}
__device__ __forceinline__ float3 eval_disney_diffuse(float ax, float ay, float F0, const pt_material& m,
                                                      float3 c_sheen, float3 V, float3 L, float3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3(0.0f);
  float LdH = dot(L, H);
  float retro = 2.0f * m.roughness * LdH * LdH;
  float fL = schlick_weight(L.z);
  float fV = schlick_weight(V.z);
  float f_retro = retro * (fL + fV + fL * fV * (retro - 1.0f));
  float f_d = (1.0f - 0.5f * fL) * (1.0f - 0.5f * fV);
  float coupled = coupled_diffuse(ax, ay, fabsf(V.z), fabsf(L.z), F0 * m.specular_tint);
  float f_ss90 = 0.5f * retro;
  float f_ss = mixf(1.0f, f_ss90, fL) * mixf(1.0f, f_ss90, fV);
  float ss = 1.25f * (f_ss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
  float fH = schlick_weight(LdH);
  float3 f_sheen = fH * m.sheen * c_sheen;
  float alpha = fmaxf(m.roughness, 0.07f);
  alpha = alpha * alpha;
  float Ewi = max3(c_sheen) * sheen_directional_albedo(fabsf(V.z), alpha);
  float Ewo = max3(c_sheen) * sheen_directional_albedo(fabsf(L.z), alpha);
  float sheen_weight = fminf(1.0f - Ewi, 1.0f - Ewo);
  pdf = L.z * INV_PI;
  return INV_PI * f3(m.base_color) * mixf(f_d * coupled * PI + f_retro, ss, m.subsurface) + f_sheen * sheen_weight;
}
__device__ __forceinline__ float3 eval_microfacet_reflection(float ax, float ay, float3 V, float3 L, float3 H,
                                                             float3 F, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3(0.0f);
  float D = gtr2_aniso(H.z, H.x, H.y, ax, ay);
  float G1 = smith_g_aniso(fabsf(V.z), V.x, V.y, ax, ay);
  float G2 = G1 * smith_g_aniso(fabsf(L.z), L.x, L.y, ax, ay);
  pdf = G1 * D / (4.0f * V.z);
  return F * D * G2 / (4.0f * L.z * V.z);
}
__device__ __forceinline__ float specular_directional_albedo(float alpha, float ct) {
  return 1.0f - 1.45940f * alpha * (-0.20276f + alpha * (2.77203f + (-2.61748f + 0.73343f * alpha) * alpha)) *
                    ct * (3.09507f + ct * (-9.11368f + ct * (15.88844f + ct * (-13.70343f + 4.51786f * ct))));
}
__device__ __forceinline__ float3 eval_microfacet_ms(float ax, float ay, float3 V, float3 L, float3 F0) {
  float alpha = sqrtf(ax * ay);
  float Ewi = specular_directional_albedo(alpha, fabsf(V.z));
  float Ewo = specular_directional_albedo(alpha, fabsf(L.z));
  float Eavg = 1.0f + alpha * (-0.11304f + alpha * (-1.86947f + (2.22682f - 0.83397f * alpha) * alpha));
  float ms = (1.0f - Ewo) * (1.0f - Ewi) / (PI * (1.0f - Eavg));
  float3 Favg = (20.0f / 21.0f) * F0 + (1.0f / 21.0f) * f3(1.0f);
  float3 f = (Favg * Favg * Eavg) / (f3(1.0f) - Favg * (1.0f - Eavg));
  return ms * f;
}
__device__ __forceinline__ float3 eval_microfacet_refraction(float ax, float ay, float3 base, float eta, float3 V,
                                                             float3 L, float3 H, float3 F, float& pdf) {
  pdf = 0.0f;
  if (L.z >= 0.0f) return f3(0.0f);
  float ldh = dot(L, H);
  float vdh = dot(V, H);
  float D = gtr2_aniso(H.z, H.x, H.y, ax, ay);
  float G1 = smith_g_aniso(fabsf(V.z), V.x, V.y, ax, ay);
  float G2 = G1 * smith_g_aniso(fabsf(L.z), L.x, L.y, ax, ay);
  float denom = ldh + vdh * eta;
  denom *= denom;
  float eta2 = eta * eta;
  float jac = fabsf(ldh) / denom;
  pdf = G1 * fmaxf(0.0f, vdh) * D * jac / V.z;
  return make_float3(pm_pow(base.x, 0.5f), pm_pow(base.y, 0.5f), pm_pow(base.z, 0.5f)) * (f3(1.0f) - F) * D * G2 *
         fabsf(vdh) * jac * eta2 / fabsf(L.z * V.z);
}
__device__ __forceinline__ float3 eval_clearcoat(float ccr, float3 V, float3 L, float3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3(0.0f);
  float vdh = dot(V, H);
  float F = mixf(0.04f, 1.0f, schlick_weight(vdh));
  float D = gtr1(H.z, ccr);
  float G = smith_g(L.z, 0.25f) * smith_g(V.z, 0.25f);
  float jac = 1.0f / (4.0f * vdh);
  pdf = D * H.z * jac;
  return f3(F) * D * G;
}

struct LobeProbs {
  float F0;
  float3 c_sheen, c_spec0;
  float dielectric_wt, metal_wt, glass_wt;
  float diffuse_pr, dielectric_pr, metal_pr, glass_pr, clearcoat_pr;
};
// disney.glsl:9-32 (tint_colors), :312-331 (lobe probabilities)
__device__ __forceinline__ LobeProbs lobe_probs(const pt_material& m, float eta, float Vz) {
  LobeProbs p;
  float3 base = f3(m.base_color);
  float lum = luminance(base);
  float3 ctint = lum > 0.0f ? base / lum : f3(1.0f);
  p.F0 = (1.0f - eta) / (1.0f + eta);
  p.F0 *= p.F0;
  p.c_spec0 = p.F0 * mix(f3(1.0f), ctint, m.specular_tint);
  p.c_sheen = mix(f3(1.0f), ctint, m.sheen_tint);
  p.dielectric_wt = (1.0f - m.metallic) * (1.0f - m.specular_transmission);
  p.metal_wt = m.metallic;
  p.glass_wt = (1.0f - m.metallic) * m.specular_transmission;
  float sw = schlick_weight(Vz);
  p.diffuse_pr = p.dielectric_wt * lum;
  p.dielectric_pr = p.dielectric_wt * luminance(mix(p.c_spec0, f3(1.0f), sw));
  p.metal_pr = p.metal_wt * luminance(mix(base, f3(1.0f), sw));
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

// disney.glsl:264-390 (ROUGHNESS_REGULARIZE_EVAL)
// GLASS = false leaves out the glass lobe, for materials whose glass weight
// is zero: its branches are then never taken, so the result is the same.
template <bool GLASS>
static __device__ __forceinline__ float3 disney_eval_body(bool ans, const ShadeFrame& s, const pt_material& m,
                                                          float3 V, float3 N, float3 L, float& pdf) {
  float ax = m.ax, ay = m.ay;
  if (s.depth > 0 && ans) {
    if (ax < 0.3f) ax = clampf(2.0f * ax, 0.1f, 0.3f);
    if (ay < 0.3f) ay = clampf(2.0f * ay, 0.1f, 0.3f);
  }
  pdf = 0.0f;
  float3 f = f3(0.0f);
  V = to_local(s.tangent, s.bitangent, N, V);
  L = to_local(s.tangent, s.bitangent, N, L);
  float3 H;
  if (L.z > 0.0f) H = normalize(L + V);
  else H = normalize(L + V * s.eta);
  if (H.z < 0.0f) H = -H;
  LobeProbs p = lobe_probs(m, s.eta, V.z);
  bool refl = L.z * V.z > 0.0f;
  float tmp = 0.0f;
  float vdh = fabsf(dot(V, H));
  float3 base = f3(m.base_color);
  if (p.diffuse_pr > 0.0f && refl) {
    f += eval_disney_diffuse(ax, ay, p.F0, m, p.c_sheen, V, L, H, tmp) * p.dielectric_wt;
    pdf += tmp * p.diffuse_pr;
  }
  if (p.dielectric_pr > 0.0f && refl) {
    float F = (dielectric_fresnel(vdh, s.eta) - p.F0) / (1.0f - p.F0);
    f += eval_microfacet_reflection(ax, ay, V, L, H, mix(p.c_spec0, f3(1.0f), F), tmp) * p.dielectric_wt;
    f += eval_microfacet_ms(ax, ay, V, L, p.c_spec0) * p.dielectric_wt;
    pdf += tmp * p.dielectric_pr;
  }
  if (p.metal_pr > 0.0f && refl) {
    float3 F = mix(base, f3(1.0f), schlick_weight(vdh));
    f += eval_microfacet_reflection(ax, ay, V, L, H, F, tmp) * p.metal_wt;
    f += eval_microfacet_ms(ax, ay, V, L, base) * p.metal_wt;
    pdf += tmp * p.metal_pr;
  }
  if (GLASS && p.glass_pr > 0.0f) {
    float F = dielectric_fresnel(vdh, s.eta);
    if (refl) {
      f += eval_microfacet_reflection(ax, ay, V, L, H, f3(F), tmp) * p.glass_wt;
      f += eval_microfacet_ms(ax, ay, V, L, p.c_spec0) * p.glass_wt;
      pdf += tmp * p.glass_pr * F;
    } else {
      f += eval_microfacet_refraction(ax, ay, base, s.eta, V, L, H, f3(F), tmp) * p.glass_wt;
      pdf += tmp * p.glass_pr * (1.0f - F);
    }
  }
  if (p.clearcoat_pr > 0.0f && refl) {
    f += eval_clearcoat(m.clearcoat_roughness, V, L, H, tmp) * f3(m.clearcoat_tint) * 0.25f * m.clearcoat;
    pdf += tmp * p.clearcoat_pr;
  }
  return f * fabsf(L.z);
}

// One out-of-line copy per kernel instead of one per call site. The kernels of
// scenes with media ran faster with it (media box +4%, measured while they
// also held the transmittance traversal that k_transmit now runs for scenes
// without transparent materials), the others with the body inlined (Disney
// grid +2%).
template <bool GLASS>
static __device__ __noinline__ float3 disney_eval_call(bool ans, const ShadeFrame& s, const pt_material& m, float3 V,
                                                       float3 N, float3 L, float& pdf) {
  return disney_eval_body<GLASS>(ans, s, m, V, N, L, pdf);
}

template <bool GLASS, bool INLINE>
__device__ __forceinline__ float3 disney_eval(bool ans, const ShadeFrame& s, const pt_material& m, float3 V, float3 N,
                                              float3 L, float& pdf) {
  if (INLINE) return disney_eval_body<GLASS>(ans, s, m, V, N, L, pdf);
  return disney_eval_call<GLASS>(ans, s, m, V, N, L, pdf);
}

// disney.glsl:405-531 (GLASS and INLINE as for disney_eval)
template <bool GLASS, bool INLINE>
__device__ __forceinline__ float3 disney_sample(uint4& rng, bool& ans, const ShadeFrame& s, const pt_material& m,
                                                float3 V, float3 N, float3& L, float& pdf, uint32_t& flags) {
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
  // flags bits 8..10: sampled lobe (hash only; the state keeps the low byte)
  if (r3 < cdf0) {
    L = cosine_sample_hemisphere(r1, r2);
    flags = RAY_FLAGS_REFLECTION;
  } else if (r3 < cdf2) {
    float3 H = sample_ggx_vndf(V, ax, ay, r1, r2);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect3(-V, H));
    flags = RAY_FLAGS_REFLECTION | (1u << 8);
  } else if (GLASS && r3 < cdf3) {
    float3 H = sample_ggx_vndf(V, ax, ay, r1, r2);
    float F = dielectric_fresnel(fabsf(dot(V, H)), s.eta);
    if (H.z < 0.0f) H = -H;
    r3 = (r3 - cdf2) / (cdf3 - cdf2);
    if (r3 < F) {
      L = normalize(reflect3(-V, H));
      flags = RAY_FLAGS_REFLECTION | (2u << 8);
    } else {
      L = normalize(refract3(-V, H, s.eta));
      flags = RAY_FLAGS_TRANSMISSION | (3u << 8);
    }
  } else {
    float3 H = sample_gtr1(m.clearcoat_roughness, r1, r2);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect3(-V, H));
    flags = RAY_FLAGS_REFLECTION | (4u << 8);
  }
  L = to_world(s.tangent, s.bitangent, N, L);
  V = to_world(s.tangent, s.bitangent, N, V);
  return disney_eval<GLASS, INLINE>(ans, s, m, V, N, L, pdf);
}

template <int MAT, bool INLINE>
__device__ __forceinline__ float3 bsdf_eval(const ShadeFrame& s, const pt_material& m, bool ans, float3 V, float3 N,
                                            float3 L, float& pdf) {
  if (MAT == SHADE_DISNEY_GLASS) return disney_eval<true, INLINE>(ans, s, m, V, N, L, pdf);
  if (MAT == PT_MATERIAL_DISNEY) return disney_eval<false, INLINE>(ans, s, m, V, N, L, pdf);
  return diffuse_eval(s, m, V, N, L, pdf);
}
template <int MAT, bool INLINE>
__device__ __forceinline__ float3 bsdf_sample(uint4& rng, bool& ans, const ShadeFrame& s, const pt_material& m,
                                              float3 V, float3 N, float3& L, float& pdf, uint32_t& flags) {
  if (MAT == SHADE_DISNEY_GLASS) return disney_sample<true, INLINE>(rng, ans, s, m, V, N, L, pdf, flags);
  if (MAT == PT_MATERIAL_DISNEY) return disney_sample<false, INLINE>(rng, ans, s, m, V, N, L, pdf, flags);
  return diffuse_sample(rng, ans, s, m, V, N, L, pdf, flags);
}

}  // namespace hpt
