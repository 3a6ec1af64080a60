// glsl_shim.h -- just enough GLSL on top of C++ to compile the reference's
// ray-tracing shaders as host code (oracle/_ref, test infrastructure only).
//
// Vector/matrix types with the swizzles the shaders read, the GLSL built-in
// functions they call, and empty macros for the storage qualifiers. The
// arithmetic follows GLSL: component-wise float32 operations, mix(x, y, a) =
// x (1 - a) + y a, clamp = min(max()), normalize = v * (1 / sqrt(dot(v, v))).
// Transcendental built-ins use the portable float32 functions of the oracle
// (GLSL leaves their precision to the implementation).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <tuple>

#include "../pmath.h"

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;
struct uvec2;
struct uvec3;
struct uvec4;
struct ivec2;
struct LaunchXY;
struct mat4;

// read-only swizzle proxies living in the same union as the components
template <class V, class T, int N, int A, int B>
struct Sw2 {
  T d[N];
  operator V() const;
};
template <class V, class T, int N, int A, int B, int C>
struct Sw3 {
  T d[N];
  operator V() const;
};

struct vec2 {
  union {
    struct { float x, y; };
    struct { float r, g; };
  };
  vec2() : x(0), y(0) {}
  explicit vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
  explicit vec2(const uvec2& u);
  float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
  union {
    struct { float x, y, z; };
    struct { float r, g, b; };
    Sw3<vec3, float, 3, 0, 1, 2> xyz;
    Sw2<vec2, float, 3, 0, 1> xy;
  };
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
  vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
  explicit vec3(const vec4& v);
  explicit vec3(const uvec3& v);
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
  union {
    struct { float x, y, z, w; };
    struct { float r, g, b, a; };
    Sw3<vec3, float, 4, 0, 1, 2> rgb;
    Sw3<vec3, float, 4, 0, 1, 2> xyz;
    Sw2<vec2, float, 4, 0, 1> xy;
  };
  vec4() : x(0), y(0), z(0), w(0) {}
  explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
  vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
  explicit vec4(const uvec4& v);
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct uvec2 {
  uint x, y;
  uvec2() : x(0), y(0) {}
  uvec2(uint a, uint b) : x(a), y(b) {}
};
inline vec2::vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}

struct uvec3 {
  uint x, y, z;
  uvec3() : x(0), y(0), z(0) {}
  uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
inline vec3::vec3(const uvec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}

struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
  explicit ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}
  explicit ivec2(const LaunchXY& l);
};

struct uvec4 {
  union {
    struct { uint x, y, z, w; };
    Sw2<uvec2, uint, 4, 0, 1> xy;
    Sw3<uvec3, uint, 4, 0, 1, 2> xyz;
  };
  uvec4() : x(0), y(0), z(0), w(0) {}
  uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
  uvec4(const vec2& p, uint c, uint d) : x((uint)p.x), y((uint)p.y), z(c), w(d) {}
  uvec4(const uvec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
  uvec4& operator=(const uvec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
};

inline vec4::vec4(const uvec4& v) : x((float)v.x), y((float)v.y), z((float)v.z), w((float)v.w) {}

template <class V, class T, int N, int A, int B>
Sw2<V, T, N, A, B>::operator V() const { return V(d[A], d[B]); }
template <class V, class T, int N, int A, int B, int C>
Sw3<V, T, N, A, B, C>::operator V() const { return V(d[A], d[B], d[C]); }

// gl_LaunchIDEXT: .xy converts to vec2 (rng_initialize) and to ivec2 (images)
struct LaunchXY {
  uint x, y;
  operator vec2() const { return vec2((float)x, (float)y); }
};
struct LaunchID {
  union {
    struct { uint x, y, z; };
    LaunchXY xy;
  };
};
inline ivec2::ivec2(const LaunchXY& l) : x((int)l.x), y((int)l.y) {}

// ---- arithmetic
#define V3OP(op)                                                                                       \
  inline vec3 operator op(const vec3& a, const vec3& b) { return vec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
  inline vec3 operator op(const vec3& a, float s) { return vec3(a.x op s, a.y op s, a.z op s); }        \
  inline vec3 operator op(float s, const vec3& a) { return vec3(s op a.x, s op a.y, s op a.z); }
V3OP(+) V3OP(-) V3OP(*) V3OP(/)
#undef V3OP
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec3& operator-=(vec3& a, const vec3& b) { a = a - b; return a; }
inline vec3& operator*=(vec3& a, const vec3& b) { a = a * b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline vec3& operator/=(vec3& a, float s) { a = a / s; return a; }
inline vec3& operator/=(vec3& a, const vec3& b) { a = a / b; return a; }

#define V2OP(op)                                                                                 \
  inline vec2 operator op(const vec2& a, const vec2& b) { return vec2(a.x op b.x, a.y op b.y); } \
  inline vec2 operator op(const vec2& a, float s) { return vec2(a.x op s, a.y op s); }          \
  inline vec2 operator op(float s, const vec2& a) { return vec2(s op a.x, s op a.y); }
V2OP(+) V2OP(-) V2OP(*) V2OP(/)
#undef V2OP
inline vec2& operator/=(vec2& a, const vec2& b) { a = a / b; return a; }

#define V4OP(op)                                                                                           \
  inline vec4 operator op(const vec4& a, const vec4& b) { return vec4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); } \
  inline vec4 operator op(const vec4& a, float s) { return vec4(a.x op s, a.y op s, a.z op s, a.w op s); }
V4OP(+) V4OP(-) V4OP(*) V4OP(/)
#undef V4OP
inline vec2& operator*=(vec2& a, const vec2& b) { a = a * b; return a; }

inline uvec2 operator%(const uvec2& a, uint m) { return uvec2(a.x % m, a.y % m); }
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator%(const ivec2& a, int m) { return ivec2(a.x % m, a.y % m); }

inline uvec4 operator*(const uvec4& a, uint s) { return uvec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline uvec4 operator+(const uvec4& a, uint s) { return uvec4(a.x + s, a.y + s, a.z + s, a.w + s); }
inline uvec4 operator>>(const uvec4& a, uint s) { return uvec4(a.x >> s, a.y >> s, a.z >> s, a.w >> s); }
inline uvec4 operator^(const uvec4& a, const uvec4& b) { return uvec4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w); }
inline vec2 operator/(const uvec2& a, float s) { return vec2((float)a.x / s, (float)a.y / s); }
inline vec4 operator/(const uvec4& a, float s) { return vec4((float)a.x / s, (float)a.y / s, (float)a.z / s, (float)a.w / s); }

// ---- matrices (column-major like GLSL)
struct mat3 {
  vec3 c[3];
  mat3() {}
  mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
  explicit mat3(const mat4& m);
  vec3& operator[](int i) { return c[i]; }
  const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
  vec4 c[4];
};
inline mat3::mat3(const mat4& m) {
  c[0] = vec3(m.c[0].x, m.c[0].y, m.c[0].z);
  c[1] = vec3(m.c[1].x, m.c[1].y, m.c[1].z);
  c[2] = vec3(m.c[2].x, m.c[2].y, m.c[2].z);
}
inline vec3 operator*(const mat3& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline vec3 operator*(const vec3& v, const mat3& m);
inline mat3 transpose(const mat3& m) {
  return mat3(vec3(m.c[0].x, m.c[1].x, m.c[2].x), vec3(m.c[0].y, m.c[1].y, m.c[2].y),
              vec3(m.c[0].z, m.c[1].z, m.c[2].z));
}
inline mat3 inverse(const mat3& m) {  // adjugate / determinant
  auto M = [&](int r, int col) { return m.c[col][r]; };
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
  // inverse[r][c] = C[c][r] / det; columns of the result
  return mat3(vec3(C00 / det, C01 / det, C02 / det), vec3(C10 / det, C11 / det, C12 / det),
              vec3(C20 / det, C21 / det, C22 / det));
}

// ---- built-in functions
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 operator*(const vec3& v, const mat3& m) { return vec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float clamp(float x, int lo, int hi) { return clamp(x, (float)lo, (float)hi); }
inline vec3 clamp(const vec3& v, float lo, float hi) { return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline float smoothstep(float e0, float e1, float x) {
  float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }
inline vec3 refract(const vec3& i, const vec3& n, float eta) {
  float d = dot(n, i);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return vec3(0.0f);
  return eta * i - (eta * d + std::sqrt(k)) * n;
}
inline float fma(float a, float b, float c) { return std::fma(a, b, c); }
inline float sin(float x) { return pmath::sin(x); }
inline float cos(float x) { return pmath::cos(x); }
inline float tan(float x) { return pmath::tan(x); }
inline float exp(float x) { return pmath::exp(x); }
inline float log(float x) { return pmath::log(x); }
inline float pow(float x, float y) { return pmath::pow(x, y); }
inline float acos(float x) { return pmath::acos(x); }
inline float atan(float y, float x) { return pmath::atan2(y, x); }
inline vec3 exp(const vec3& v) { return vec3(exp(v.x), exp(v.y), exp(v.z)); }
inline vec3 pow(const vec3& v, const vec3& p) { return vec3(pow(v.x, p.x), pow(v.y, p.y), pow(v.z, p.z)); }

// ---- storage qualifiers and ray-tracing declarations
#define layout(...)
#define uniform
#define readonly
#define highp
#define rayPayloadEXT thread_local
#define rayPayloadInEXT extern thread_local
#define callableDataEXT thread_local
#define callableDataInEXT extern thread_local
#define hitAttributeEXT extern thread_local
#define gl_RayFlagsOpaqueEXT 1u
#define gl_RayFlagsTerminateOnFirstHitEXT 4u
#define gl_RayFlagsSkipClosestHitShaderEXT 8u

inline vec2 operator*(const vec2& a, const uvec2& b) { return vec2(a.x * (float)b.x, a.y * (float)b.y); }

// ---- resources (bound by the harness)
struct accelerationStructureEXT { int id; };
struct texture2D { int id; };
struct sampler { int id; };
struct sampler2D {
  int id;
  int kind;  // 0 environment map, 1 marginal distribution, 2 conditional distribution, 3 material texture
  sampler2D() : id(0), kind(0) {}
  sampler2D(int i, int k) : id(i), kind(k) {}
  sampler2D(const texture2D& t, const sampler&) : id(t.id), kind(t.id == 0 ? 1 : 2) {}
};
struct image2D { int id; };
vec4 texelFetch(const texture2D& t, const ivec2& p, int lod);
vec4 textureLod(const sampler2D& s, const vec2& uv, float lod);
vec4 imageLoad(const image2D& img, const ivec2& p);
void imageStore(const image2D& img, const ivec2& p, const vec4& v);
void traceRayEXT(const accelerationStructureEXT& as, uint flags, uint mask, uint sbt_offset, uint sbt_stride,
                 uint miss_index, const vec3& origin, float tmin, const vec3& direction, float tmax, int payload);
void executeCallableEXT(uint sbt_index, int callable);
bool reportIntersectionEXT(float t, uint kind);

extern thread_local LaunchID gl_LaunchIDEXT;
extern thread_local uint gl_InstanceCustomIndexEXT;
extern thread_local int gl_PrimitiveID;
extern thread_local float gl_HitTEXT;
extern thread_local uint gl_HitKindEXT;
extern thread_local vec3 gl_WorldRayOriginEXT;
extern thread_local vec3 gl_WorldRayDirectionEXT;
extern thread_local float gl_RayTminEXT;
extern thread_local float gl_RayTmaxEXT;
