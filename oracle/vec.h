// vec.h -- minimal GLSL-like float vector math for the CPU oracle.
//
// The oracle is test infrastructure: the CPU restatement of hala-pathtracer's
// integrator that the CUDA path is checked against. Nothing in the product
// library includes this file.
//
// normalize() is written as v * (1 / sqrt(dot(v, v))) with IEEE division and
// square root; the CUDA device code uses the same formula.
#pragma once
#include <cmath>
#include <cstdint>

#include "pmath.h"

namespace orc {

struct V2 {
  float x, y;
  V2() : x(0), y(0) {}
  V2(float a, float b) : x(a), y(b) {}
};

struct V3 {
  float x, y, z;
  V3() : x(0), y(0), z(0) {}
  explicit V3(float s) : x(s), y(s), z(s) {}
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct U4 {
  uint32_t x, y, z, w;
};

inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
inline V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
inline V3& operator*=(V3& a, float s) { a = a * s; return a; }
inline V3& operator/=(V3& a, float s) { a = a / s; return a; }

inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline V3 mix(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline V3 clamp(V3 v, float lo, float hi) {
  return V3(clampf(v.x, lo, hi), clampf(v.y, lo, hi), clampf(v.z, lo, hi));
}
inline V3 vexp(V3 v) { return V3(pmath::exp(v.x), pmath::exp(v.y), pmath::exp(v.z)); }
inline V3 vsqrt(V3 v) { return V3(std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z)); }
inline float max3(V3 v) { return std::fmax(std::fmax(v.x, v.y), v.z); }
inline float smoothstepf(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
// GLSL reflect(I, N) = I - 2 dot(N, I) N
inline V3 reflect(V3 i, V3 n) { return i - 2.0f * dot(n, i) * n; }
// GLSL refract(I, N, eta)
inline V3 refract(V3 i, V3 n, float eta) {
  float d = dot(n, i);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return V3(0.0f);
  return eta * i - (eta * d + std::sqrt(k)) * n;
}

}  // namespace orc
