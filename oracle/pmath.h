// pmath.h -- portable float32 transcendental functions of the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle). The CUDA library has its own
// copy of the same algorithm (pt_device.cuh, pm_*). Both evaluate the same
// IEEE operations in the same order (explicit fused multiply-adds, no other
// contraction), so the oracle and the device round every result the same way
// and per-path radiance can be compared bit for bit. The reference's GLSL
// built-ins (sin, exp, pow, ...) have implementation-defined precision, so a
// fixed portable choice is as faithful to it as glibc's or CUDA's.
//
// Method: Cody-Waite argument reduction with constants split into three
// float32 parts, then polynomial kernels whose coefficients were fitted by
// iteratively reweighted least squares (relative error, Chebyshev nodes,
// 40-digit reference values) and rounded to float32:
//   sin/cos  reduction by pi/2, sin r = r + r^3 S(r^2), cos r = 1 - r^2/2 + r^4 C(r^2)
//   exp      reduction by ln 2, exp r = 1 + r + r^2 E(r), scale by 2^k exactly
//   log      x = m 2^e, m in [sqrt(1/2), sqrt(2)), s = f / (2 + f),
//            log(1+f) = f - s (f - s^2 L(s^2))
//   acos     via asin x = x + x^3 A(x^2) on [0, 1/2] and the half-angle forms
//   atan2    atan t = t + t^3 T(t^2) on [0, tan(pi/8)], pi/4 shift above
//   pow      exp(y log x) for x > 0
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

namespace pmath {

inline float fma_(float a, float b, float c) { return std::fma(a, b, c); }
inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float nan_() { return std::numeric_limits<float>::quiet_NaN(); }

constexpr float TWO_OVER_PI = 0.6366197466850281f;
constexpr float PIO2_HI = 1.5707963705062866f, PIO2_MID = -4.371138828673793e-08f, PIO2_LO = -1.7151245100058819e-15f;
constexpr float PIO4_HI = 0.7853981852531433f, PIO4_MID = -2.1855694143368964e-08f;
constexpr float PI_HI = 3.1415927410125732f, PI_MID = -8.742277657347586e-08f;
constexpr float LOG2E = 1.4426950216293335f;
constexpr float LN2_HI = 0.6931471824645996f, LN2_MID = -1.9046542121259336e-09f;

inline void sincos(float x, float& s, float& c) {
  if (!(std::fabs(x) <= 1.0e6f)) { s = c = nan_(); return; }
  float k = std::nearbyint(x * TWO_OVER_PI);
  float r = fma_(-k, PIO2_HI, x);
  r = fma_(-k, PIO2_MID, r);
  r = fma_(-k, PIO2_LO, r);
  int q = (int)k;
  float z = r * r;
  float sp = fma_(fma_(fma_(2.7249013783148257e-06f, z, -0.00019840076856780797f), z, 0.008333331905305386f), z,
                  -0.1666666716337204f);
  float sr = fma_(r * z, sp, r);
  float cp = fma_(fma_(fma_(-2.730170649556385e-07f, z, 2.480060538800899e-05f), z, -0.00138888880610466f), z,
                  0.0416666679084301f);
  float cr = fma_(z * z, cp, fma_(-0.5f, z, 1.0f));
  switch (q & 3) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
  }
}
inline float sin(float x) { float s, c; sincos(x, s, c); return s; }
inline float cos(float x) { float s, c; sincos(x, s, c); return c; }
inline float tan(float x) { float s, c; sincos(x, s, c); return s / c; }

inline float exp(float x) {
  if (x != x) return x;
  if (x > 88.72283935546875f) return std::numeric_limits<float>::infinity();
  if (x < -103.97208404541016f) return 0.0f;
  float k = std::nearbyint(x * LOG2E);
  float r = fma_(-k, LN2_HI, x);
  r = fma_(-k, LN2_MID, r);
  float p = fma_(fma_(fma_(fma_(fma_(0.00019924867956433445f, r, 0.0013933534501120448f), r, 0.008333264850080013f), r,
                           0.041666463017463684f), r, 0.1666666716337204f), r, 0.5f);
  float er = fma_(r * r, p, r) + 1.0f;
  int ki = (int)k;
  int k1 = ki / 2, k2 = ki - k1;
  return (er * u2f((uint32_t)(k1 + 127) << 23)) * u2f((uint32_t)(k2 + 127) << 23);
}

inline float log(float x) {
  if (x != x || x < 0.0f) return nan_();
  if (x == 0.0f) return -std::numeric_limits<float>::infinity();
  if (x == std::numeric_limits<float>::infinity()) return x;
  int e = 0;
  if (x < 1.17549435e-38f) { x *= 8388608.0f; e = -23; }
  uint32_t b = f2u(x);
  e += (int)((b >> 23) & 0xffu) - 127;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m *= 0.5f; e += 1; }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float p = fma_(fma_(fma_(0.23334167897701263f, z, 0.28550657629966736f), z, 0.4000012278556824f), z,
                 0.6666666865348816f);
  float lm = fma_(-s, fma_(-z, p, f), f);
  float fe = (float)e;
  return fma_(fe, LN2_HI, fma_(fe, LN2_MID, lm));
}

inline float pow(float x, float y) {
  if (y == 0.0f || x == 1.0f) return 1.0f;
  if (x != x || y != y || x < 0.0f) return nan_();
  if (x == 0.0f) return y > 0.0f ? 0.0f : std::numeric_limits<float>::infinity();
  return exp(y * log(x));
}

inline float asin_k(float x) {  // x in [-1/2, 1/2]
  float z = x * x;
  float p = fma_(fma_(fma_(fma_(fma_(0.034081507474184036f, z, 0.01690877228975296f), z, 0.031152866780757904f), z,
                           0.044594623148441315f), z, 0.07500111311674118f), z, 0.1666666567325592f);
  return fma_(x * z, p, x);
}
inline float acos(float x) {
  if (x != x || std::fabs(x) > 1.0f) return nan_();
  if (std::fabs(x) <= 0.5f) return PIO2_HI - (asin_k(x) - PIO2_MID);
  if (x > 0.0f) return 2.0f * asin_k(std::sqrt((1.0f - x) * 0.5f));
  return PI_HI - (2.0f * asin_k(std::sqrt((1.0f + x) * 0.5f)) - PI_MID);
}

inline float atan_k(float t) {  // t in [-tan(pi/8), tan(pi/8)]
  float z = t * t;
  float p = fma_(fma_(fma_(fma_(fma_(0.05074314400553703f, z, -0.08635549992322922f), z, 0.11072912812232971f), z,
                           -0.1428423672914505f), z, 0.19999979436397552f), z, -0.3333333432674408f);
  return fma_(t * z, p, t);
}
inline float atan2(float y, float x) {
  if (x != x || y != y) return nan_();
  float ax = std::fabs(x), ay = std::fabs(y);
  float mx = std::fmax(ax, ay), mn = std::fmin(ax, ay);
  float r;
  if (mx == 0.0f) {
    r = 0.0f;
  } else {
    float t = (mx == std::numeric_limits<float>::infinity()) ? (mn == mx ? 1.0f : 0.0f) : mn / mx;
    if (t > 0.41421356f) r = PIO4_HI + (atan_k((t - 1.0f) / (t + 1.0f)) + PIO4_MID);
    else r = atan_k(t);
  }
  if (ay > ax) r = (PIO2_HI - r) + PIO2_MID;
  if (x < 0.0f) r = (PI_HI - r) + PI_MID;
  return (y < 0.0f) ? -r : r;
}

}  // namespace pmath
