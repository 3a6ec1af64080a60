// pt_shade.cuh -- device code shared by the wavefront kernels: queue
// appends, environment and light sampling, hit -> surface state, and the
// miss/emitter and material shading kernels (templates instantiated by
// pt_render.cu and pt_shade_*.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "pt_internal.h"
#include "pt_trace.cuh"

namespace hpt {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append of `val` to queue q when pred holds.
__device__ __forceinline__ void queue_push(uint32_t* q, uint32_t* counter, uint32_t val, bool pred) {
  unsigned active = __activemask();
  unsigned m = __ballot_sync(active, pred);
  if (m == 0) return;
  int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(active, base, leader);
  if (pred) q[base + __popc(m & ((1u << lane_id()) - 1u))] = val;
}

__device__ __forceinline__ void count_add(unsigned long long* c, uint32_t v) {
  unsigned active = __activemask();
  uint32_t s = __reduce_add_sync(active, v);
  if ((int)lane_id() == __ffs(active) - 1 && s) atomicAdd(c, (unsigned long long)s);
}

// ------------------------------------------------------------------ environment
__device__ __forceinline__ uint32_t env_texel_index(const DevScene& S, float u, float v) {
  float fu = u - floorf(u);
  if (!(fu >= 0.0f)) fu = 0.0f;
  float fv = v;
  if (!(fv >= 0.0f)) fv = 0.0f;
  if (fv > 1.0f) fv = 1.0f;
  uint32_t ix = (uint32_t)(fu * (float)S.env_w);
  uint32_t iy = (uint32_t)(fv * (float)S.env_h);
  if (ix > S.env_w - 1) ix = S.env_w - 1;
  if (iy > S.env_h - 1) iy = S.env_h - 1;
  return iy * S.env_w + ix;
}
__device__ __forceinline__ float3 env_texel(const DevScene& S, uint32_t idx) { return f3(__ldg(&S.env_rgba[idx])); }

// inc/env_map.glsl:43-55
__device__ __forceinline__ float env_pdf(const DevScene& S, float u, float v, float theta) {
  float st = pm_sin(theta);
  if (st > EPS) {
    float3 color = env_texel(S, env_texel_index(S, u, v)) * S.env_intensity;
    float pdf = luminance(color) / S.env_total_sum;
    if (pdf > EPS) return (pdf * (float)S.env_w * (float)S.env_h) / (TWO_PI * PI * st);
    return 0.0f;
  }
  return 0.0f;
}
// env_map_eval.rcall.glsl:14-34, env_sky_eval.rcall.glsl:12-15
__device__ __forceinline__ float3 eval_env(const DevScene& S, float3 dir, uint32_t depth, uint32_t flags,
                                           float state_pdf) {
  if (!S.env_map) {
    float a = fmaxf(dir.z, 0.0f);
    return mix(f3(S.ground), f3(S.sky), a) * S.env_intensity;
  }
  float theta = pm_acos(dir.z);
  float u = -(PI + pm_atan2(dir.y, dir.x)) * INV_TWO_PI - S.env_rotation;
  float v = theta * INV_PI;
  float mis = 1.0f;
  if (depth > 0 && (flags & RAY_FLAGS_SPECULAR) == 0) {
    float pdf = env_pdf(S, u, v, theta);
    mis = power_heuristic(state_pdf, pdf);
  }
  return mis * env_texel(S, env_texel_index(S, u, v)) * S.env_intensity;
}
__device__ __forceinline__ uint32_t alias_draw(const uint2* t, uint32_t n, float s, float& frac) {
  float x = s * (float)n;
  uint32_t k = (uint32_t)x;
  if (k > n - 1) k = n - 1;
  float r = x - (float)k;
  uint2 e = __ldg(&t[k]);
  float p = __uint_as_float(e.x);
  if (p >= 1.0f) { frac = r; return k; }
  if (r < p) { frac = r / p; return k; }
  frac = (r - p) / (1.0f - p);
  return e.y;
}
// inc/env_map.glsl:6-37, alias tables in place of the inverse-CDF textures
__device__ __forceinline__ float3 sample_env_map(const DevScene& S, uint4& rng, float3& color, float& pdf) {
  float2 s = rand2(rng);
  // v = marginal(s.x); u = conditional(s.y, v) on the row of texel v; colour
  // = nearest texel at (u, v) (inc/env_map.glsl:7-12)
  float fv, fu;
  uint32_t yr = alias_draw(S.alias_rows, S.env_h, s.x, fv);
  float v = ((float)yr + fv) / (float)S.env_h;
  uint32_t y = (uint32_t)(v * (float)S.env_h);
  if (y > S.env_h - 1) y = S.env_h - 1;
  uint32_t x = alias_draw(S.alias_cols + (size_t)y * S.env_w, S.env_w, s.y, fu);
  float u = ((float)x + fu) / (float)S.env_w;
  color = env_texel(S, env_texel_index(S, u, v)) * S.env_intensity;
  pdf = luminance(color) / S.env_total_sum;
  float phi = (u + S.env_rotation) * TWO_PI;
  float theta = v * PI;
  float st = pm_sin(theta);
  if (st <= EPS) pdf = 0.0f;
  float3 dir = normalize(make_float3(-st * pm_cos(phi), st * pm_sin(phi), pm_cos(theta)));
  pdf = (pdf * (float)S.env_w * (float)S.env_h) / (TWO_PI * PI * st);
  return dir;
}

// ------------------------------------------------------------------ light sampling
struct LightSample {
  float3 normal, emission, direction;
  float dist, pdf;
};
// inc/light/{point,distant,spot,quad,sphere}.glsl
__device__ __forceinline__ LightSample sample_light(uint4& rng, float3 fhp, const DevLight& L, uint32_t nl) {
  LightSample o;
  float fn = (float)nl;
  float3 Lpos = f3(L.position), Lu = f3(L.u), Lv = f3(L.v), LI = f3(L.intensity);
  if (L.type == PT_LIGHT_POINT || L.type == PT_LIGHT_SPOT) {
    float3 ld = Lpos - fhp;
    float d2 = dot(ld, ld);
    o.dist = sqrtf(d2);
    ld = ld / o.dist;
    o.normal = -ld;
    if (L.type == PT_LIGHT_POINT) o.emission = LI * fn / d2;
    else o.emission = smoothstepf(Lv.y, Lv.x, dot(-ld, Lu)) * LI * fn / d2;
    o.pdf = 1.0f;
    o.direction = ld;
  } else if (L.type == PT_LIGHT_DIRECTIONAL) {
    float3 dir = -Lu;
    float cos_alpha = Lv.x;
    if (cos_alpha > EPS) {
      float3 N = dir, T, B;
      onb(N, T, B);
      float r = rand1(rng);
      float phi = TWO_PI * rand1(rng);
      float z = (1.0f - r * (1.0f - cos_alpha));
      float radius = sqrtf(1.0f - z * z);
      float x = radius * pm_cos(phi);
      float y = radius * pm_sin(phi);
      dir = to_world(T, B, N, make_float3(x, y, z));
    }
    o.normal = Lu;
    o.emission = LI * fn;
    o.dist = WORLD_SIZE;
    o.pdf = 1.0f;
    o.direction = dir;
  } else if (L.type == PT_LIGHT_QUAD) {
    float r1 = rand1(rng);
    float r2 = rand1(rng);
    float3 lp = Lpos + Lu * r1 + Lv * r2;
    float3 ld = lp - fhp;
    o.normal = normalize(cross(Lv, Lu));
    float ct = dot(-ld, o.normal);
    if (ct < 0.0f) {
      o.emission = f3(0.0f);
      o.dist = 0.0f;
      o.pdf = 0.0f;
      o.direction = f3(0.0f);
    } else {
      float d2 = dot(ld, ld);
      o.dist = sqrtf(d2);
      ld /= o.dist;
      o.emission = LI * fn;
      o.pdf = d2 / (L.area * fabsf(ct));
      o.direction = ld;
    }
  } else if (L.type == PT_LIGHT_SPHERE) {
    float r1 = rand1(rng);
    float r2 = rand1(rng);
    float3 cs = fhp - Lpos;
    float dc = length(cs);
    cs /= dc;
    if (dc < L.radius) {
      o.normal = cs;
      o.emission = f3(0.0f);
      o.dist = dc;
      o.pdf = 0.0f;
      o.direction = f3(0.0f);
    } else {
      float3 sd = uniform_sample_hemisphere(r1, r2);
      float3 T, B;
      onb(cs, T, B);
      sd = T * sd.x + B * sd.y + cs * sd.z;
      float3 lp = Lpos + sd * L.radius;
      float3 ld = lp - fhp;
      float d2 = dot(ld, ld);
      o.dist = sqrtf(d2);
      ld = ld / o.dist;
      o.normal = normalize(lp - Lpos);
      o.emission = LI * fn;
      o.pdf = d2 / (L.area * 0.5f * fabsf(dot(o.normal, ld)));
      o.direction = ld;
    }
  } else {
    o.normal = o.emission = o.direction = f3(0.0f);
    o.dist = 0.0f;
    o.pdf = 0.0f;
  }
  return o;
}

// Any component non-zero (NaN counts as non-zero).
__device__ __forceinline__ bool nonzero(float3 c) { return c.x != 0.0f || c.y != 0.0f || c.z != 0.0f; }

// ------------------------------------------------------------------ hit -> state
struct SurfState {  // the State fields filled by triangles.rchit.glsl:13-76
  float3 fhp, ffnormal, normal;
  ShadeFrame fr;
  float hit_distance;
  uint32_t mat;
};
__device__ __forceinline__ float3 interp_normal(const DevScene& S, uint32_t id, float u, float v) {
  const float4* r = S.tri_shade + 6 * (size_t)id;
  float b0 = 1.0f - u - v, b1 = u, b2 = v;
  float3 n = f3(__ldg(r)) * b0 + f3(__ldg(r + 1)) * b1 + f3(__ldg(r + 2)) * b2;
  return normalize(n);
}
// Texture coordinate of a triangle hit (triangles.rchit.glsl:63).
__device__ __forceinline__ float2 hit_uv(const DevScene& S, float4 hit) {
  uint32_t id = __float_as_uint(hit.w);
  uint32_t i0 = __ldg(&S.tri_vidx[3 * id]), i1 = __ldg(&S.tri_vidx[3 * id + 1]), i2 = __ldg(&S.tri_vidx[3 * id + 2]);
  float b0 = 1.0f - hit.y - hit.z, b1 = hit.y, b2 = hit.z;
  float2 t0 = __ldg(&S.vuv[i0]), t1 = __ldg(&S.vuv[i1]), t2 = __ldg(&S.vuv[i2]);
  return make_float2(t0.x * b0 + t1.x * b1 + t2.x * b2, t0.y * b0 + t1.y * b1 + t2.y * b2);
}

__device__ __forceinline__ void fill_surface(const DevScene& S, float3 o, float3 d, float4 hit, SurfState& s) {
  uint32_t id = __float_as_uint(hit.w);
  const float4* r = S.tri_shade + 6 * (size_t)id;
  const float4 n0 = __ldg(r), n1 = __ldg(r + 1), n2 = __ldg(r + 2);
  const float4 t0 = __ldg(r + 3), t1 = __ldg(r + 4), t2 = __ldg(r + 5);
  float b0 = 1.0f - hit.y - hit.z, b1 = hit.y, b2 = hit.z;
  float3 n = f3(n0) * b0 + f3(n1) * b1 + f3(n2) * b2;
  n = normalize(n);
  float3 tg = f3(t0) * b0 + f3(t1) * b1 + f3(t2) * b2;
  tg = normalize(tg);
  s.hit_distance = hit.x;
  s.fhp = o + d * s.hit_distance;
  s.normal = n;
  s.ffnormal = dot(n, d) <= 0.0f ? n : -n;
  s.fr.tangent = tg;
  s.fr.bitangent = cross(n, tg);
  s.mat = __float_as_uint(n0.w);
}

// ------------------------------------------------------------------ material textures
// textureLod(g_textures[i], uv, 0) of pathtracer.rgen.glsl:122-145, with the
// sampler state the glTF default names: bilinear filtering, repeat wrapping,
// texel centres at half-integer coordinates, row 0 at v = 0.
__device__ __forceinline__ uint32_t wrap_texel(long long i, uint32_t n) {
  long long m = i % (long long)n;
  return (uint32_t)(m < 0 ? m + n : m);
}
__device__ __forceinline__ float4 sample_texture(const DevScene& S, uint32_t t, float u, float v) {
  const uint4 info = __ldg(&S.tex_info[t]);
  const uint32_t w = info.y, h = info.z;
  if (!(fabsf(u) < 1e6f)) u = 0.0f;
  if (!(fabsf(v) < 1e6f)) v = 0.0f;
  const float x = __fsub_rn(__fmul_rn(u, (float)w), 0.5f), y = __fsub_rn(__fmul_rn(v, (float)h), 0.5f);
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = __fsub_rn(x, x0), fy = __fsub_rn(y, y0);
  const uint32_t ix0 = wrap_texel((long long)x0, w), ix1 = wrap_texel((long long)x0 + 1, w);
  const uint32_t iy0 = wrap_texel((long long)y0, h), iy1 = wrap_texel((long long)y0 + 1, h);
  const float4* T = S.tex_texels + info.x;
  const float4 a = __ldg(&T[(size_t)iy0 * w + ix0]), b = __ldg(&T[(size_t)iy0 * w + ix1]);
  const float4 c = __ldg(&T[(size_t)iy1 * w + ix0]), e = __ldg(&T[(size_t)iy1 * w + ix1]);
  auto lerp = [](float p, float q, float f) { return __fadd_rn(p, __fmul_rn(__fsub_rn(q, p), f)); };
  return make_float4(lerp(lerp(a.x, b.x, fx), lerp(c.x, e.x, fx), fy), lerp(lerp(a.y, b.y, fx), lerp(c.y, e.y, fx), fy),
                     lerp(lerp(a.z, b.z, fx), lerp(c.z, e.z, fx), fy), lerp(lerp(a.w, b.w, fx), lerp(c.w, e.w, fx), fy));
}

// ------------------------------------------------------------------ miss / emitter / invalid
// pathtracer.rgen.glsl:70-115
template <bool MULTI>
__device__ __forceinline__ void logic_path(const DevScene& S0, const PathState& P, uint32_t p) {
  {
    const DevScene& S = MULTI ? P.jobs[P.job[p]] : S0;
    float4 h = P.hit[p];
    uint32_t id = __float_as_uint(h.w);
    float4 r4 = P.rad[p];
    float3 rad = f3(r4);
    uint32_t hash = __float_as_uint(r4.w);
    hmix(hash, id);
    float4 t4 = P.thr[p];
    float3 T = f3(t4);
    uint32_t depth = P.depth[p];
    if (id == HIT_MISS) {
      float3 d = f3(P.ray_d[p]);
      rad += T * eval_env(S, d, depth, P.flags[p] & 0xFFu, t4.w);
      if (depth == 0) {
        P.albedo[p] = make_float4(rad.x, rad.y, rad.z, 0.0f);
        P.normal[p] = make_float4(-d.x, -d.y, -d.z, 0.0f);
      }
    } else if (id & HIT_LIGHT_BIT) {
      const DevLight& L = S.lights[id & ~HIT_LIGHT_BIT];
      float w = 1.0f;
      if (depth > 0) w = power_heuristic(t4.w, h.y);
      rad += w * f3(L.intensity) * T;
    } else {
      rad = make_float3(0.7f, 0.0f, 0.7f);
    }
    P.rad[p] = make_float4(rad.x, rad.y, rad.z, __uint_as_float(hash));
  }
}

// inc/lighting.glsl:7-61 (MEDIUM && VOL_MIS): transmittance along a shadow
// ray through refractive (and, with TRANSPARENT, transparent) surfaces and
// the media behind them. Draws random numbers only with TRANSPARENT; counts
// its closest-hit rays in `nrays`.
template <bool TRANSPARENT>
__device__ __forceinline__ float3 transmittance(const DevScene& S, uint4& rng, float3 o, float3 d,
                                                unsigned long long& nrays) {
  float3 T = f3(1.0f);
  for (uint32_t depth = 0; depth < S.max_depth; ++depth) {
    ++nrays;
    HitRec h = trace_closest<false>(S, o, d, 0.0f, WORLD_SIZE);
    if (h.id == HIT_MISS || (h.id & HIT_LIGHT_BIT)) break;
    uint32_t mi = __ldg(&S.tri_mat[h.id]);
    if (mi >= S.num_mats) return f3(0.0f);
    const pt_material& m = S.mats[mi];
    bool transparent = false;
    if (TRANSPARENT) transparent = m.opacity == 0.0f || rand1(rng) > m.opacity;
    bool refractive = (1.0f - m.metallic) * m.specular_transmission > 0.0f;
    if (!(transparent || refractive)) return f3(0.0f);
    float3 nrm = interp_normal(S, h.id, h.u, h.v);
    if (dot(d, nrm) > 0.0f && m.medium.type != PT_MEDIUM_NONE) {
      float3 col = m.medium.type == PT_MEDIUM_ABSORB ? f3(1.0f) - f3(m.medium.color) : f3(1.0f);
      T *= vexp(-col * m.medium.density * h.t);
    }
    float3 fhp = o + d * h.t;
    o = fhp + d * EPS;
  }
  return T;
}

// ------------------------------------------------------------------ surface shading
template <int MAT>
struct Shader {
  const DevScene& S;
  uint4 rng;
  uint32_t hash;
  unsigned long long nshadow;

  template <bool TRANSPARENT>
  __device__ float3 eval_transmittance(float3 o, float3 d) {
    return transmittance<TRANSPARENT>(S, rng, o, d, nshadow);
  }

  // inc/lighting.glsl:69-244 with the transmittance evaluated in-thread.
  template <bool TRANSPARENT>
  __device__ float3 direct_lighting_volmis(const pt_material& mat, bool is_surface, bool ans, const SurfState& st,
                                           float3 fhp, float3 raydir, float aniso) {
    float3 Ld = f3(0.0f), Li;
    float3 scatter_pos = fhp + st.ffnormal * EPS;
    if (S.env_map) {
      float3 em;
      float light_pdf;
      float3 ldir = sample_env_map(S, rng, em, light_pdf);
      Li = em;
      if (light_pdf > 0.0f) {
        float3 T = eval_transmittance<TRANSPARENT>(scatter_pos, ldir);
        bool vis = luminance(T) > 0.0f;
        hmix(hash, 0x40000000u | (vis ? 1u : 0u));
        if (vis) {
          Li *= T;
          float pdf = 0.0f;
          float3 f = f3(0.0f);
          if (is_surface) {
            f = bsdf_eval<MAT, false>(st.fr, mat, ans, -raydir, st.ffnormal, ldir, pdf);
          } else {
            pdf = phase_hg(dot(-raydir, ldir), aniso);
            f = f3(pdf);
          }
          if (pdf > 0.0f) {
            float w = power_heuristic(light_pdf, pdf);
            if (w > 0.0f) Ld += w * Li * f / light_pdf;
          }
        }
      }
    }
    uint32_t nl = S.num_lights;
    if (nl > 0) {
      int li = (int)(rand1(rng) * (float)nl);
      DevLight L = {};
      if (li >= 0 && li < (int)nl) L = S.lights[li];
      LightSample ls = sample_light(rng, fhp, L, nl);
      float light_pdf = ls.pdf;
      Li = ls.emission;
      if (light_pdf > 0.0f && dot(ls.direction, ls.normal) < 0.0f) {
        float3 T = eval_transmittance<TRANSPARENT>(scatter_pos, ls.direction);
        bool vis = luminance(T) > 0.0f;
        hmix(hash, 0x50000000u | (vis ? 1u : 0u));
        if (vis) {
          Li *= T;
          float pdf = 0.0f;
          float3 f = f3(0.0f);
          if (is_surface) {
            f = bsdf_eval<MAT, false>(st.fr, mat, ans, -raydir, st.ffnormal, ls.direction, pdf);
          } else {
            pdf = phase_hg(dot(-raydir, ls.direction), aniso);
            f = f3(pdf);
          }
          if (pdf > 0.0f) {
            float w = 1.0f;
            if (L.area > 0.0f) w = power_heuristic(light_pdf, pdf);
            if (w > 0.0f) Ld += w * Li * f / light_pdf;
          }
        }
      }
    }
    return Ld;
  }

  // direct_lighting_volmis of a scene without transparent materials, whose
  // transmittance draws no random numbers: the light samples are drawn here
  // in the same order, and the two shadow rays with the factors of their
  // contributions are stored for k_transmit, which traces them, mixes the
  // visibility events into the hash and adds the light as the in-thread
  // form does. `T` is the throughput the contribution is scaled by. Returns
  // the pending-ray bits (PEND_ENV, PEND_LIGHT).
  __device__ uint32_t prepare_volmis(const PathState& P, uint32_t p, const pt_material& mat, bool is_surface,
                                     bool ans, const SurfState& st, float3 fhp, float3 raydir, float aniso,
                                     float3 T);
};

// Pending-event word stored with the shadow rays (applied to the hash after
// the visibility events, in the reference's order).
constexpr uint32_t PEND_ENV = 1u, PEND_LIGHT = 2u, PEND_BSDF = 4u, PEND_STOP = 8u, PEND_RR = 16u;

template <int MAT>
__device__ uint32_t Shader<MAT>::prepare_volmis(const PathState& P, uint32_t p, const pt_material& mat,
                                                bool is_surface, bool ans, const SurfState& st, float3 fhp,
                                                float3 raydir, float aniso, float3 T) {
  uint32_t pend = 0;
  const float3 scatter_pos = fhp + st.ffnormal * EPS;
  if (S.env_map) {
    float3 em;
    float light_pdf;
    float3 ldir = sample_env_map(S, rng, em, light_pdf);
    if (light_pdf > 0.0f) {
      float pdf = 0.0f;
      float3 f = f3(0.0f);
      if (is_surface) {
        f = bsdf_eval<MAT, false>(st.fr, mat, ans, -raydir, st.ffnormal, ldir, pdf);
      } else {
        pdf = phase_hg(dot(-raydir, ldir), aniso);
        f = f3(pdf);
      }
      float w = 0.0f;
      bool add = false;
      if (pdf > 0.0f) {
        w = power_heuristic(light_pdf, pdf);
        add = w > 0.0f;
      }
      pend |= PEND_ENV;
      P.sh_d0[p] = make_float4(ldir.x, ldir.y, ldir.z, w);
      P.sh_c0[p] = make_float4(em.x, em.y, em.z, light_pdf);
      P.sh_f0[p] = make_float4(f.x, f.y, f.z, add ? 1.0f : 0.0f);
    }
  }
  uint32_t nl = S.num_lights;
  if (nl > 0) {
    int li = (int)(rand1(rng) * (float)nl);
    DevLight L = {};
    if (li >= 0 && li < (int)nl) L = S.lights[li];
    LightSample ls = sample_light(rng, fhp, L, nl);
    float light_pdf = ls.pdf;
    if (light_pdf > 0.0f && dot(ls.direction, ls.normal) < 0.0f) {
      float pdf = 0.0f;
      float3 f = f3(0.0f);
      if (is_surface) {
        f = bsdf_eval<MAT, false>(st.fr, mat, ans, -raydir, st.ffnormal, ls.direction, pdf);
      } else {
        pdf = phase_hg(dot(-raydir, ls.direction), aniso);
        f = f3(pdf);
      }
      float w = 1.0f;
      bool add = false;
      if (pdf > 0.0f) {
        if (L.area > 0.0f) w = power_heuristic(light_pdf, pdf);
        add = w > 0.0f;
      }
      pend |= PEND_LIGHT;
      P.sh_d1[p] = make_float4(ls.direction.x, ls.direction.y, ls.direction.z, w);
      P.sh_c1[p] = make_float4(ls.emission.x, ls.emission.y, ls.emission.z, light_pdf);
      P.sh_f1[p] = make_float4(f.x, f.y, f.z, add ? 1.0f : 0.0f);
    }
  }
  if (pend) {
    P.sh_o[p] = make_float4(scatter_pos.x, scatter_pos.y, scatter_pos.z, 0.0f);
    P.sh_T[p] = make_float4(T.x, T.y, T.z, 0.0f);
  }
  return pend;
}

// Closest hit of path p's ray and the class of what it hit: 0 for a miss,
// an emitter or an invalid material (surface logic), else MAT_CLASS_*
// (pathtracer.rgen.glsl:56-68, triangles.rchit.glsl:13-76).
template <bool BRUTE, bool COUNT, bool MULTI>
__device__ __forceinline__ uint32_t trace_path(const DevScene& S0, const PathState& P, uint32_t p, TravCount& tc) {
  const DevScene& S = MULTI ? P.jobs[P.job[p]] : S0;
  if (P.c_train) {
    // a training path leaving the cache vertex: what it gathered so far is
    // the part of its radiance the cache does not predict
    uint32_t k = P.c_train[p];
    if (k != 0xFFFFFFFFu && P.depth[p] == P.c_depth + 1u) P.t_R[k] = P.rad[p];
  }
  float4 o4 = P.ray_o[p], d4 = P.ray_d[p];
  HitRec h = trace_closest<BRUTE, COUNT>(S, f3(o4), f3(d4), 0.0f, WORLD_SIZE, &tc);
  P.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.id));
  uint32_t cls = 0;
  if (h.id != HIT_MISS && !(h.id & HIT_LIGHT_BIT)) {
    uint32_t m = __ldg(&S.tri_mat[h.id]);
    if (m < S.num_mats) cls = __ldg(&S.mat_class[m]);
  }
  return cls;
}

// The deferred shadow rays of path p and the hash events that wait for
// them (inc/lighting.glsl:116-149 and :203-238: visibility, then
// radiance += T * Ld). Returns the number of rays traced.
template <bool BRUTE, bool MULTI>
__device__ __forceinline__ uint32_t shadow_path(const DevScene& S0, const PathState& P, uint32_t p) {
  const DevScene& S = MULTI ? P.jobs[P.job[p]] : S0;
  float4 so = P.sh_o[p];
  uint32_t pend = __float_as_uint(so.w);
  float3 o = f3(so);
  float4 r4 = P.rad[p];
  uint32_t hash = __float_as_uint(r4.w);
  float3 Ld = f3(0.0f);
  uint32_t nrays = 0;
  if (pend & PEND_ENV) {
    float4 d0 = P.sh_d0[p];
    bool occ = trace_any<BRUTE>(S, o, f3(d0), 0.0f, d0.w);
    ++nrays;
    hmix(hash, 0x40000000u | (occ ? 0u : 1u));
    if (!occ) Ld += f3(P.sh_c0[p]);
  }
  if (pend & PEND_LIGHT) {
    float4 d1 = P.sh_d1[p];
    bool occ = trace_any<BRUTE>(S, o, f3(d1), 0.0f, d1.w);
    ++nrays;
    hmix(hash, 0x50000000u | (occ ? 0u : 1u));
    if (!occ) Ld += f3(P.sh_c1[p]);
  }
  if (pend & PEND_BSDF) hmix(hash, 0x60000000u | ((pend >> 8) & 0xFFFu));
  if (pend & PEND_STOP) hmix(hash, 0x61000000u);
  if (pend & PEND_RR) hmix(hash, 0x72000000u);
  float3 rad = f3(r4) + f3(P.sh_T[p]) * Ld;
  P.rad[p] = make_float4(rad.x, rad.y, rad.z, __uint_as_float(hash));
  return nrays;
}

// The deferred next-event rays of a vertex with media (prepare_volmis):
// transmittance of each pending ray, its visibility event, and the light it
// adds, in the order and arithmetic of direct_lighting_volmis; then the
// hash events that wait for them. Returns the closest-hit rays traced.
template <bool MULTI>
__device__ __forceinline__ uint32_t transmit_path(const DevScene& S0, const PathState& P, uint32_t p) {
  const DevScene& S = MULTI ? P.jobs[P.job[p]] : S0;
  float4 so = P.sh_o[p];
  uint32_t pend = __float_as_uint(so.w);
  float3 o = f3(so);
  float4 r4 = P.rad[p];
  uint32_t hash = __float_as_uint(r4.w);
  float3 Ld = f3(0.0f);
  unsigned long long nrays = 0;
  uint4 no_rng = make_uint4(0u, 0u, 0u, 0u);  // not drawn from without transparent materials
  if (pend & PEND_ENV) {
    const float4 d0 = P.sh_d0[p], c0 = P.sh_c0[p], f0 = P.sh_f0[p];
    const float3 T = transmittance<false>(S, no_rng, o, f3(d0), nrays);
    const bool vis = luminance(T) > 0.0f;
    hmix(hash, 0x40000000u | (vis ? 1u : 0u));
    if (vis && f0.w != 0.0f) {
      float3 Li = f3(c0);
      Li *= T;
      Ld += d0.w * Li * f3(f0) / c0.w;
    }
  }
  if (pend & PEND_LIGHT) {
    const float4 d1 = P.sh_d1[p], c1 = P.sh_c1[p], f1 = P.sh_f1[p];
    const float3 T = transmittance<false>(S, no_rng, o, f3(d1), nrays);
    const bool vis = luminance(T) > 0.0f;
    hmix(hash, 0x50000000u | (vis ? 1u : 0u));
    if (vis && f1.w != 0.0f) {
      float3 Li = f3(c1);
      Li *= T;
      Ld += d1.w * Li * f3(f1) / c1.w;
    }
  }
  if (pend & PEND_BSDF) hmix(hash, 0x60000000u | ((pend >> 8) & 0xFFFu));
  if (pend & PEND_STOP) hmix(hash, 0x61000000u);
  if (pend & PEND_RR) hmix(hash, 0x72000000u);
  float3 rad = f3(r4) + f3(P.sh_T[p]) * Ld;
  P.rad[p] = make_float4(rad.x, rad.y, rad.z, __uint_as_float(hash));
  return (uint32_t)nrays;
}

// Warp-aggregated append that returns the slot index (or ~0u when !pred).
__device__ __forceinline__ uint32_t append_index(uint32_t* counter, bool pred) {
  unsigned active = __activemask();
  unsigned m = __ballot_sync(active, pred);
  if (m == 0) return 0xFFFFFFFFu;
  int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(active, base, leader);
  return pred ? base + __popc(m & ((1u << lane_id()) - 1u)) : 0xFFFFFFFFu;
}

// Material maps of pathtracer.rgen.glsl:121-145: colour, metallic/roughness
// (blue/green), emission, and the tangent-space normal map (z scaled by 5).
__device__ __forceinline__ void apply_maps(const DevScene& S, pt_material& m, SurfState& st, float3 d, float2 uv) {
  if (m.base_color_map_index < S.num_textures) {
    float4 c = sample_texture(S, m.base_color_map_index, uv.x, uv.y);
    m.base_color[0] = c.x;
    m.base_color[1] = c.y;
    m.base_color[2] = c.z;
  }
  if (m.metallic_roughness_map_index < S.num_textures) {
    float4 mr = sample_texture(S, m.metallic_roughness_map_index, uv.x, uv.y);
    m.metallic = mr.z;
    m.roughness = mr.y;
  }
  if (m.emission_map_index < S.num_textures) {
    float4 c = sample_texture(S, m.emission_map_index, uv.x, uv.y);
    m.emission[0] = c.x;
    m.emission[1] = c.y;
    m.emission[2] = c.z;
  }
  if (m.normal_map_index < S.num_textures) {
    float4 c = sample_texture(S, m.normal_map_index, uv.x, uv.y);
    float3 nts = make_float3(c.x, c.y, c.z * 5.0f);
    nts = normalize(nts * 2.0f - f3(1.0f));
    const float3 orig = st.normal;
    st.normal = normalize(st.fr.tangent * nts.x + st.fr.bitangent * nts.y + st.normal * nts.z);
    st.ffnormal = dot(orig, d) <= 0.0f ? st.normal : -st.normal;
    st.fr.bitangent = cross(st.normal, st.fr.tangent);
  }
}

// What one shading step decided for its path: the path ends (`stop`), and
// its shadow rays and pending hash events wait for k_shadow (`deferred`).
struct ShadeResult {
  bool stop, deferred;
};

// One surface (or medium) vertex of path p: pathtracer.rgen.glsl:117-256.
template <int MAT, bool MEDIUM, bool TRANSPARENT, bool MULTI, bool CACHE, bool TEXTURED>
__device__ __forceinline__ ShadeResult shade_path(const DevScene& S0, const PathState& P, uint32_t p,
                                                  unsigned long long& nshadow_total) {
  {
    const DevScene& S = MULTI ? P.jobs[P.job[p]] : S0;
    Shader<MAT> sh{S, P.rng[p], 0u, 0ull};
    float4 h = P.hit[p];
    float3 o = f3(P.ray_o[p]), d = f3(P.ray_d[p]);
    float4 t4 = P.thr[p];
    float3 T = f3(t4);
    float state_pdf = t4.w;
    float4 r4 = P.rad[p];
    float3 rad = f3(r4);
    sh.hash = __float_as_uint(r4.w);
    uint32_t depth = P.depth[p];
    uint32_t flags = P.flags[p];
    bool ans = (flags & ANS_BIT) != 0;
    bool in_medium = (flags & IN_MEDIUM_BIT) != 0;
    float4 m0 = make_float4(0, 0, 0, 0);
    float2 m1 = make_float2(1.0f, __uint_as_float(PT_MEDIUM_NONE));
    if (MEDIUM) {
      m0 = P.med0[p];
      m1 = P.med1[p];
    }
    uint32_t id = __float_as_uint(h.w);
    hmix(sh.hash, id);

    SurfState st;
    fill_surface(S, o, d, h, st);
    pt_material mtex;
    if (TEXTURED) mtex = S.mats[st.mat];
    const pt_material& mat = TEXTURED ? mtex : S.mats[st.mat];
    st.fr.eta = dot(d, st.normal) < 0.0f ? (1.0f / mat.ior) : mat.ior;
    st.fr.depth = depth;
    if (TEXTURED) apply_maps(S, mtex, st, d, hit_uv(S, h));
    // Radiance-cache vertex: its emission and direct light are computed as
    // usual; the light arriving through the BSDF continuation (indirect) is
    // either the cache's estimate -- the path ends here and the estimate is
    // added after the bounce loop -- or, for a training path, traced on.
    bool cache_query = false;
    // Only diffuse-looking vertices use the cache: at a glossy or refracting
    // vertex the light through the BSDF is a narrow, view-dependent lobe whose
    // training targets are heavy-tailed glints, so such a path goes on
    // unbiased and does not train.
    const bool cache_vertex = MAT == PT_MATERIAL_DIFFUSE ||
                              (MAT == PT_MATERIAL_DISNEY && !(mat.roughness < P.c_min_rough));
    if (CACHE && depth == P.c_depth && cache_vertex) {
      const float4 rec0 = make_float4(st.fhp.x, st.fhp.y, st.fhp.z, -d.x);
      const float4 rec1 = make_float4(-d.y, -d.z, st.ffnormal.x, st.ffnormal.y);
      const float4 rec2 = make_float4(st.ffnormal.z, mat.base_color[0], mat.base_color[1], mat.base_color[2]);
      const float4 rec3 = make_float4(mat.roughness, mat.metallic, mat.specular_transmission, 0.0f);
      const bool train = P.c_mode == 1 || P.c_shift == 0 || ((p * 2654435761u) >> (32u - P.c_shift)) == 0u;
      if (!train) {
        cache_query = true;
        P.c_rec[4 * (size_t)p] = rec0;
        P.c_rec[4 * (size_t)p + 1] = rec1;
        P.c_rec[4 * (size_t)p + 2] = rec2;
        P.c_rec[4 * (size_t)p + 3] = rec3;
        P.c_T[p] = make_float4(T.x, T.y, T.z, 0.0f);
      } else {
        const bool fresh = P.c_train[p] == 0xFFFFFFFFu;
        uint32_t k = append_index(&P.c_counts[1], fresh);
        if (fresh) {
          P.t_rec[4 * (size_t)k] = rec0;
          P.t_rec[4 * (size_t)k + 1] = rec1;
          P.t_rec[4 * (size_t)k + 2] = rec2;
          P.t_rec[4 * (size_t)k + 3] = rec3;
          P.t_T[k] = make_float4(T.x, T.y, T.z, 0.0f);
          P.t_R[k] = make_float4(__int_as_float(0x7FC00000), 0.0f, 0.0f, 0.0f);
          P.c_train[p] = k;
        }
      }
    }
    if (depth == 0) {
      P.albedo[p] = make_float4(mat.base_color[0], mat.base_color[1], mat.base_color[2], 0.0f);
      P.normal[p] = make_float4(st.normal.x, st.normal.y, st.normal.z, 0.0f);
    }
    rad += T * f3(mat.emission);

    bool stop = false;
    bool medium_sampled = false;
    float3 fhp = st.fhp;
    uint32_t pend = 0;
    if (MEDIUM && in_medium) {
      uint32_t mtype = __float_as_uint(m1.y);
      float3 mcol = f3(m0);
      float dens = m0.w;
      if (mtype == PT_MEDIUM_ABSORB) {
        T *= vexp(-(f3(1.0f) - mcol) * st.hit_distance * dens);
      } else if (mtype == PT_MEDIUM_EMISSIVE) {
        rad += mcol * st.hit_distance * dens * T;
      } else {
        float sd = fminf(-pm_log(rand1(sh.rng)) / dens, st.hit_distance);
        medium_sampled = sd < st.hit_distance;
        if (medium_sampled) {
          hmix(sh.hash, 0x70000001u);
          T *= mcol;
          o = o + d * sd;
          fhp = o;
          if (TRANSPARENT) {
            rad += sh.template direct_lighting_volmis<TRANSPARENT>(mat, false, ans, st, fhp, d, m1.x) * T;
          } else {
            pend |= sh.prepare_volmis(P, p, mat, false, ans, st, fhp, d, m1.x, T);
            if (!pend) rad += f3(0.0f) * T;  // no ray pending: Ld = 0 (NaN for a non-finite T)
          }
          float q1 = rand1(sh.rng);
          float q2 = rand1(sh.rng);
          float3 sdir = sample_hg(-d, m1.x, q1, q2);
          state_pdf = phase_hg(dot(-d, sdir), m1.x);
          d = sdir;
        }
      }
    }
    if (!medium_sampled) {
      bool skip = false;
      if (TRANSPARENT) {
        if (mat.opacity == 0.0f || rand1(sh.rng) > mat.opacity) {
          depth--;
          skip = true;
          hmix(sh.hash, 0x71000000u);
        }
      }
      if (!skip) {
        if (MEDIUM && TRANSPARENT) {
          rad += T * sh.template direct_lighting_volmis<TRANSPARENT>(mat, true, ans, st, fhp, d, m1.x);
        } else if (MEDIUM) {
          pend |= sh.prepare_volmis(P, p, mat, true, ans, st, fhp, d, m1.x, T);
          if (!pend) rad += T * f3(0.0f);
        } else {
          // Next-event estimation with deferred visibility (inc/lighting.glsl:69-244).
          float3 scatter_pos = fhp + st.ffnormal * EPS;
          float3 c0 = f3(0.0f), c1 = f3(0.0f);
          float4 d0 = make_float4(0, 0, 0, 0), d1 = make_float4(0, 0, 0, 0);
          // A shadow ray is traced only when its contribution is not zero:
          // adding a zero (visible or not) leaves the sum unchanged, so only
          // the visibility events of the hit-sequence hash depend on it (the
          // oracle hashes the same rays).
          if (S.env_map) {
            float3 em;
            float light_pdf;
            float3 ldir = sample_env_map(S, sh.rng, em, light_pdf);
            if (light_pdf > 0.0f) {
              float pdf;
              float3 f = bsdf_eval<MAT, !MEDIUM>(st.fr, mat, ans, -d, st.ffnormal, ldir, pdf);
              if (pdf > 0.0f) {
                float w = power_heuristic(light_pdf, pdf);
                if (w > 0.0f) c0 = w * em * f / light_pdf;
              }
              if (nonzero(c0)) {
                pend |= PEND_ENV;
                d0 = make_float4(ldir.x, ldir.y, ldir.z, WORLD_SIZE);
              }
            }
          }
          uint32_t nl = S.num_lights;
          if (nl > 0) {
            int li = (int)(rand1(sh.rng) * (float)nl);
            DevLight L = {};
            if (li >= 0 && li < (int)nl) L = S.lights[li];
            LightSample ls = sample_light(sh.rng, fhp, L, nl);
            if (ls.pdf > 0.0f && dot(ls.direction, ls.normal) < 0.0f) {
              float pdf;
              float3 f = bsdf_eval<MAT, !MEDIUM>(st.fr, mat, ans, -d, st.ffnormal, ls.direction, pdf);
              if (pdf > 0.0f) {
                float w = 1.0f;
                if (L.area > 0.0f) w = power_heuristic(ls.pdf, pdf);
                if (w > 0.0f) c1 = w * ls.emission * f / ls.pdf;
              }
              if (nonzero(c1)) {
                pend |= PEND_LIGHT;
                d1 = make_float4(ls.direction.x, ls.direction.y, ls.direction.z, ls.dist - 2.0f * EPS);
              }
            }
          }
          if (!pend) rad += T * f3(0.0f);  // radiance += throughput * Ld with Ld = 0 (NaN for a non-finite T)
          if (pend) {  // k_shadow reads only the records of the pending rays
            P.sh_o[p] = make_float4(scatter_pos.x, scatter_pos.y, scatter_pos.z, 0.0f);
            if (pend & PEND_ENV) {
              P.sh_d0[p] = d0;
              P.sh_c0[p] = make_float4(c0.x, c0.y, c0.z, 0.0f);
            }
            if (pend & PEND_LIGHT) {
              P.sh_d1[p] = d1;
              P.sh_c1[p] = make_float4(c1.x, c1.y, c1.z, 0.0f);
            }
            P.sh_T[p] = make_float4(T.x, T.y, T.z, 0.0f);
          }
        }
        if (CACHE && cache_query) {
          queue_push(P.c_queue, &P.c_counts[0], p, true);
          stop = true;
        }
      }
      if (!(CACHE && cache_query) && !skip) {
        float3 L;
        float pdf;
        uint32_t sflags = 0;
        float3 f = bsdf_sample<MAT, !MEDIUM>(sh.rng, ans, st.fr, mat, -d, st.ffnormal, L, pdf, sflags);
        d = L;
        state_pdf = pdf;
        flags |= sflags & 0xFFu;
        pend |= PEND_BSDF | (sflags << 8);
        if (state_pdf > 0.0f) {
          T *= f / state_pdf;
        } else {
          pend |= PEND_STOP;
          stop = true;
        }
      }
      if (!stop) {
        o = fhp + d * EPS;
        if (MEDIUM) {
          if (dot(d, st.normal) < 0.0f && mat.medium.type != PT_MEDIUM_NONE) {
            in_medium = true;
            m0 = make_float4(mat.medium.color[0], mat.medium.color[1], mat.medium.color[2], mat.medium.density);
            m1 = make_float2(mat.medium.anisotropy, __uint_as_float(mat.medium.type));
          } else {
            in_medium = false;
            m1.y = __uint_as_float(PT_MEDIUM_NONE);
          }
        }
      }
    }
    if (!stop && depth >= S.max_depth) stop = true;
    if (!stop && depth >= S.rr_depth && S.rr_depth > 0) {
      float q = fminf(fmaxf(T.x, fmaxf(T.y, T.z)) + 0.001f, 0.95f);
      if (rand1(sh.rng) > q) {
        pend |= PEND_RR;
        stop = true;
      } else {
        T /= q;
      }
    }
    // hash events of the BSDF sample / termination, unless the shadow kernel
    // has to put the visibility events first
    bool deferred = !(MEDIUM && TRANSPARENT) && (pend & (PEND_ENV | PEND_LIGHT));
    if (!deferred) {
      if (pend & PEND_BSDF) hmix(sh.hash, 0x60000000u | ((pend >> 8) & 0xFFFu));
      if (pend & PEND_STOP) hmix(sh.hash, 0x61000000u);
      if (pend & PEND_RR) hmix(sh.hash, 0x72000000u);
    }
    P.rad[p] = make_float4(rad.x, rad.y, rad.z, __uint_as_float(sh.hash));
    if (!stop) {  // a path that ends here is only read again for its radiance
      P.rng[p] = sh.rng;
      P.ray_o[p] = make_float4(o.x, o.y, o.z, 0.0f);
      P.ray_d[p] = make_float4(d.x, d.y, d.z, 0.0f);
      P.thr[p] = make_float4(T.x, T.y, T.z, state_pdf);
      P.depth[p] = depth + 1;  // loop increment of pathtracer.rgen.glsl:55
      P.flags[p] = (flags & ~(ANS_BIT | IN_MEDIUM_BIT)) | (ans ? ANS_BIT : 0u) | (in_medium ? IN_MEDIUM_BIT : 0u);
      if (MEDIUM) {
        P.med0[p] = m0;
        P.med1[p] = m1;
      }
    }
    if (deferred) {
      float4 so = P.sh_o[p];
      so.w = __uint_as_float(pend);
      P.sh_o[p] = so;
    }
    nshadow_total += sh.nshadow;
    return ShadeResult{stop, deferred};
  }
}

template <int MAT, bool MEDIUM, bool TRANSPARENT, bool MULTI, bool CACHE = false, bool TEXTURED = false>
__global__ void __launch_bounds__(256, MEDIUM ? 4 : 3) k_shade(const __grid_constant__ DevScene S0, PathState P, QueueSet Q) {
  const int slot = MAT == SHADE_DISNEY_GLASS ? Q_GLASS : (MAT == PT_MATERIAL_DISNEY ? Q_DISNEY : Q_DIFFUSE);
  const uint32_t* qin = MAT == SHADE_DISNEY_GLASS ? Q.glass : (MAT == PT_MATERIAL_DISNEY ? Q.disney : Q.diffuse);
  const uint32_t n = Q.counts[slot];
  unsigned long long nshadow_total = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t p = qin[i];
    const ShadeResult r = shade_path<MAT, MEDIUM, TRANSPARENT, MULTI, CACHE, TEXTURED>(S0, P, p, nshadow_total);
    queue_push(Q.shadow, &Q.counts[Q_SHADOW], p, r.deferred);
    queue_push(Q.next, &Q.counts[Q_NEXT], p, !r.stop);
  }
  if (MEDIUM) count_add(&Q.rays[1], (uint32_t)nshadow_total);
}

// ------------------------------------------------------------------ wave tail
// Once few paths are left in a wave, every remaining bounce of the wavefront
// loop costs about the latency of its slowest ray and its slowest shading
// call (measured on the GB300: ~140 us per bounce for 256 paths of the
// Disney grid, whatever their number), so the tail of a wave runs as one
// kernel in which each thread carries its path to the end: closest hit,
// surface logic or shading, shadow rays, again. Each step is the same device
// function the wavefront kernels call, in the same order per path, so every
// path's radiance, albedo, normal and hit-sequence hash are bit-identical to
// the wavefront's; only the schedule differs.
constexpr uint32_t TAIL_BLOCK = 64;  // small blocks spread the few paths over many SMs

template <int MAT, bool MEDIUM, bool TRANSPARENT, bool MULTI, bool TEXTURED, bool CACHE>
__device__ __noinline__ ShadeResult tail_shade(const DevScene& S0, const PathState& P, uint32_t p,
                                               unsigned long long& nshadow) {
  return shade_path<MAT, MEDIUM, TRANSPARENT, MULTI, CACHE, TEXTURED>(S0, P, p, nshadow);
}

// Paths queued in Q.in run at most `cap - done` more bounces, `done` being
// the bounces the wave already ran (*done_ptr when given, else `done`). A
// path still alive after that is appended to Q.next (the bounce cap was
// reached). The most bounces any path ran goes to *tail_bounces (atomicMax),
// the rays to Q.rays[0] / Q.rays[1].
template <bool MEDIUM, bool TRANSPARENT, bool MULTI, bool TEXTURED, bool CACHE>
__global__ void __launch_bounds__(TAIL_BLOCK) k_tail(const __grid_constant__ DevScene S0, PathState P, QueueSet Q,
                                                     const uint32_t* done_ptr, uint32_t done, uint32_t cap,
                                                     uint32_t* tail_bounces) {
  const uint32_t n = *Q.in_count;
  const uint32_t d0 = done_ptr ? *done_ptr : done;
  const uint32_t budget = cap > d0 ? cap - d0 : 0u;
  unsigned long long nclosest = 0, nshadow = 0;
  uint32_t most = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t p = Q.in[i];
    bool live = true;
    uint32_t it = 0;
    while (live && it < budget) {
      ++it;
      TravCount tc;
      const uint32_t cls = trace_path<false, false, MULTI>(S0, P, p, tc);
      ++nclosest;
      if (cls == 0) {
        logic_path<MULTI>(S0, P, p);
        live = false;
      } else {
        ShadeResult r;
        if (cls == MAT_CLASS_DIFFUSE)
          r = tail_shade<PT_MATERIAL_DIFFUSE, MEDIUM, TRANSPARENT, MULTI, TEXTURED, CACHE>(S0, P, p, nshadow);
        else if (cls == MAT_CLASS_DISNEY)
          r = tail_shade<PT_MATERIAL_DISNEY, MEDIUM, TRANSPARENT, MULTI, TEXTURED, CACHE>(S0, P, p, nshadow);
        else
          r = tail_shade<SHADE_DISNEY_GLASS, MEDIUM, TRANSPARENT, MULTI, TEXTURED, CACHE>(S0, P, p, nshadow);
        if (r.deferred) nshadow += MEDIUM ? transmit_path<MULTI>(S0, P, p) : shadow_path<false, MULTI>(S0, P, p);
        live = !r.stop;
      }
    }
    most = max(most, it);
    queue_push(Q.next, &Q.counts[Q_NEXT], p, live);
  }
  count_add(&Q.rays[0], (uint32_t)nclosest);
  count_add(&Q.rays[1], (uint32_t)nshadow);
  const unsigned active = __activemask();
  most = __reduce_max_sync(active, most);
  if ((int)lane_id() == __ffs(active) - 1 && most) atomicMax(tail_bounces, most);
}

template <bool MED, bool MULTI, bool CACHE = false>
inline void launch_tail_permutation(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                                    const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces,
                                    bool tr, bool tex, cudaStream_t st) {
  const int g = (int)std::max<uint32_t>(1u, (max_items + TAIL_BLOCK - 1) / TAIL_BLOCK);
  if (tr) {
    if (tex) k_tail<MED, true, MULTI, true, CACHE><<<g, TAIL_BLOCK, 0, st>>>(S, P, Q, done_ptr, done, cap, tail_bounces);
    else k_tail<MED, true, MULTI, false, CACHE><<<g, TAIL_BLOCK, 0, st>>>(S, P, Q, done_ptr, done, cap, tail_bounces);
  } else {
    if (tex) k_tail<MED, false, MULTI, true, CACHE><<<g, TAIL_BLOCK, 0, st>>>(S, P, Q, done_ptr, done, cap, tail_bounces);
    else k_tail<MED, false, MULTI, false, CACHE><<<g, TAIL_BLOCK, 0, st>>>(S, P, Q, done_ptr, done, cap, tail_bounces);
  }
}

// The three material kernels of one bounce (diffuse, opaque Disney, Disney
// with a glass lobe) in one feature permutation. Each pt_shade_*.cu
// instantiates the permutations of one (medium, shared-wavefront, cache)
// combination, so the variants compile in parallel.
template <bool MED, bool TR, bool MULTI, bool CACHE, bool TEX>
inline void launch_three(const DevScene& S, const PathState& P, const QueueSet& Q, int g, cudaStream_t st) {
  k_shade<PT_MATERIAL_DIFFUSE, MED, TR, MULTI, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<PT_MATERIAL_DISNEY, MED, TR, MULTI, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<SHADE_DISNEY_GLASS, MED, TR, MULTI, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
}

template <bool MED, bool MULTI, bool CACHE>
inline void launch_permutation(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                               cudaStream_t st) {
  if (tr) {
    if (tex) launch_three<MED, true, MULTI, CACHE, true>(S, P, Q, g, st);
    else launch_three<MED, true, MULTI, CACHE, false>(S, P, Q, g, st);
  } else {
    if (tex) launch_three<MED, false, MULTI, CACHE, true>(S, P, Q, g, st);
    else launch_three<MED, false, MULTI, CACHE, false>(S, P, Q, g, st);
  }
}

}  // namespace hpt
