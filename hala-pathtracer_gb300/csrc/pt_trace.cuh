// pt_trace.cuh -- ray/primitive intersection and BVH traversal (device).
//
// Replaces the RT-core traversal behind traceRayEXT
// (pathtracer.rgen.glsl:56-68, inc/lighting.glsl:119-130 / 205-216) and the
// procedural light intersection shader (lights.rint.glsl:16-37).
//
// Closest hit = lexicographic minimum of (t, global triangle id) over all
// triangles with tmin <= t <= tmax; an analytic light wins only when it is
// strictly closer. The triangle test uses explicitly rounded operations so
// it gives bit-identical t/u/v on the CPU oracle (built without FMA
// contraction), which makes BVH hits comparable bit for bit with brute force.
#pragma once
#include "pt_device.cuh"
#include "pt_types.h"

namespace hpt {

constexpr uint32_t HIT_MISS = 0xFFFFFFFFu;
constexpr uint32_t HIT_LIGHT_BIT = 0x80000000u;

__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float3 rcross(float3 a, float3 b) {
  return make_float3(rsub(rmul(a.y, b.z), rmul(a.z, b.y)), rsub(rmul(a.z, b.x), rmul(a.x, b.z)),
                     rsub(rmul(a.x, b.y), rmul(a.y, b.x)));
}
__device__ __forceinline__ float rdot(float3 a, float3 b) {
  return radd(radd(rmul(a.x, b.x), rmul(a.y, b.y)), rmul(a.z, b.z));
}

// Moller-Trumbore on (v0, e1, e2); valid when tmin <= t <= tmax.
__device__ __forceinline__ bool intersect_tri(float3 o, float3 d, float3 v0, float3 e1, float3 e2, float tmin,
                                              float tmax, float& t, float& u, float& v) {
  float3 pvec = rcross(d, e2);
  float det = rdot(e1, pvec);
  if (det == 0.0f) return false;
  float inv = __frcp_rn(det);
  float3 tvec = make_float3(rsub(o.x, v0.x), rsub(o.y, v0.y), rsub(o.z, v0.z));
  u = rmul(rdot(tvec, pvec), inv);
  if (u < 0.0f || u > 1.0f) return false;
  float3 qvec = rcross(tvec, e1);
  v = rmul(rdot(d, qvec), inv);
  if (v < 0.0f || radd(u, v) > 1.0f) return false;
  t = rmul(rdot(e2, qvec), inv);
  if (t < tmin || t > tmax) return false;
  return true;
}

// ------------------------------------------------------------------ lights
// common/intersection.glsl:31-72, inc/light/quad.glsl:42-60
__device__ __forceinline__ float quad_intersect(const DevLight& L, float3 o, float3 d, float3& normal, float& pdf) {
  float3 lu = f3(L.u), lv = f3(L.v), lp = f3(L.position);
  normal = normalize(cross(lv, lu));
  float ct = dot(-d, normal);
  if (ct < 0.0f) return INF;
  float pw = dot(normal, lp);
  float3 u = lu / dot(lu, lu);
  float3 v = lv / dot(lv, lv);
  float dt = dot(d, normal);
  float t = (pw - dot(normal, o)) / dt;
  float tr = INF;
  if (t > EPS) {
    float3 p = o + d * t;
    float3 vi = p - lp;
    float a1 = dot(u, vi);
    if (a1 >= 0.0f && a1 <= 1.0f) {
      float a2 = dot(v, vi);
      if (a2 >= 0.0f && a2 <= 1.0f) tr = t;
    }
  }
  if (tr < 0.0f) return INF;
  pdf = (tr * tr) / (L.area * ct);
  return tr;
}
// common/intersection.glsl:6-26, inc/light/sphere.glsl:50-65
__device__ __forceinline__ float sphere_light_intersect(const DevLight& L, float3 o, float3 d, float& pdf) {
  float3 lp = f3(L.position);
  float dist = length(lp - o);
  if (dist < L.radius) return INF;
  float3 op = lp - o;
  float b = dot(op, d);
  float det = b * b - dot(op, op) + L.radius * L.radius;
  float t;
  if (det < 0.0f) {
    t = INF;
  } else {
    det = sqrtf(det);
    float t1 = b - det;
    if (t1 > EPS) t = t1;
    else {
      float t2 = b + det;
      t = (t2 > EPS) ? t2 : INF;
    }
  }
  if (t < 0.0f) return INF;
  float3 hit = o + t * d;
  float ct = dot(-d, normalize(hit - lp));
  pdf = (t * t) / (L.area * ct * 0.5f);
  return t;
}
// lights.rint.glsl:16-37
__device__ __forceinline__ bool light_hit(const DevLight& L, float3 o, float3 d, float tmin, float tmax, float& t,
                                          float3& n, float& pdf) {
  t = INF;
  n = f3(0.0f);
  pdf = 1.0f;
  if (L.type == PT_LIGHT_QUAD) t = quad_intersect(L, o, d, n, pdf);
  else if (L.type == PT_LIGHT_SPHERE) t = sphere_light_intersect(L, o, d, pdf);
  else return false;
  return t >= tmin && t <= tmax;
}

// ------------------------------------------------------------------ BVH traversal
struct HitRec {
  float t, u, v;
  uint32_t id;
};

// Reciprocal direction for the slab test. A component that is exactly zero
// is replaced by +-1e-20 so fmaf(lo, inv, -o * inv) never forms inf - inf
// (which would be NaN and cull boxes the ray passes through). Only culling
// uses it; the triangle test keeps the true direction.
__device__ __forceinline__ float3 slab_inv(float3 d) {
  auto r = [](float x) { return 1.0f / (fabsf(x) < 1e-20f ? copysignf(1e-20f, x) : x); };
  return make_float3(r(d.x), r(d.y), r(d.z));
}

// Per-ray constants of the slab test: reciprocal direction, origin times it,
// and which of each axis's two planes is the near one (the child boxes are
// stored lo-then-hi per axis, so the near plane is entry 0 or 1).
struct SlabRay {
  float3 inv, oinv;
  int nx, ny, nz;
};
__device__ __forceinline__ SlabRay slab_ray(float3 o, float3 d) {
  SlabRay r;
  r.inv = slab_inv(d);
  r.oinv = make_float3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
  r.nx = r.inv.x < 0.0f ? 1 : 0;
  r.ny = r.inv.y < 0.0f ? 1 : 0;
  r.nz = r.inv.z < 0.0f ? 1 : 0;
  return r;
}

// Culling slack on the current hit distance (2^-12 relative). A triangle's
// computed t carries the rounding of the intersection test, which grows as
// the ray grazes the triangle's plane or the triangle is small against its
// distance (a shared-edge hit on the 1080p Disney grid was 21 ulps early),
// while a box's entry distance is close to exact: a box is only culled when
// it starts beyond best * (1 + 2^-12), so no triangle whose computed t beats
// the best is skipped. The oracle's BVH uses the same slack.
constexpr float TRAV_T_SLACK = 1.0f + 1.0f / 4096.0f;

// Slab test of four children of a wide node (one group of four). The
// near and far planes of each axis are picked by the ray's direction signs
// when loading, which gives exactly min/max of the two plane distances (the
// distance is monotonic in the plane coordinate, lo <= hi). The slab interval
// gets a few ulps of slack for its own rounding; `tmax` (the best hit so far)
// gets TRAV_T_SLACK.
__device__ __forceinline__ void quad_slabs(const float4* nd, const SlabRay& r, float tmin, float tmax,
                                           float (&tn)[4], bool (&hit)[4]) {
  const float4 nx = __ldg(nd + r.nx), fx = __ldg(nd + 1 - r.nx);
  const float4 ny = __ldg(nd + 2 + r.ny), fy = __ldg(nd + 3 - r.ny);
  const float4 nz = __ldg(nd + 4 + r.nz), fz = __ldg(nd + 5 - r.nz);
  const float NX[4] = {nx.x, nx.y, nx.z, nx.w}, FX[4] = {fx.x, fx.y, fx.z, fx.w};
  const float NY[4] = {ny.x, ny.y, ny.z, ny.w}, FY[4] = {fy.x, fy.y, fy.z, fy.w};
  const float NZ[4] = {nz.x, nz.y, nz.z, nz.w}, FZ[4] = {fz.x, fz.y, fz.z, fz.w};
  const float tcap = tmax * TRAV_T_SLACK;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float a0 = fmaf(NX[k], r.inv.x, -r.oinv.x), b0 = fmaf(FX[k], r.inv.x, -r.oinv.x);
    float a1 = fmaf(NY[k], r.inv.y, -r.oinv.y), b1 = fmaf(FY[k], r.inv.y, -r.oinv.y);
    float a2 = fmaf(NZ[k], r.inv.z, -r.oinv.z), b2 = fmaf(FZ[k], r.inv.z, -r.oinv.z);
    float n = fmaxf(fmaxf(a0, a1), fmaxf(a2, tmin));
    float f = fminf(fminf(b0, b1), b2) * 1.0000005f;
    tn[k] = n;
    hit[k] = n <= fminf(f, tcap);
  }
}

__device__ __forceinline__ void cswap(float& ka, int32_t& va, float& kb, int32_t& vb) {
  if (kb < ka) {
    float tk = ka;
    ka = kb;
    kb = tk;
    int32_t tv = va;
    va = vb;
    vb = tv;
  }
}

// Ascending sort of a node's (entry distance, link) pairs: the optimal
// networks of 5 (four children) and 19 (eight children) comparators.
__device__ __forceinline__ void sort_children(float (&k)[4], int32_t (&v)[4]) {
  cswap(k[0], v[0], k[1], v[1]);
  cswap(k[2], v[2], k[3], v[3]);
  cswap(k[0], v[0], k[2], v[2]);
  cswap(k[1], v[1], k[3], v[3]);
  cswap(k[1], v[1], k[2], v[2]);
}
__device__ __forceinline__ void sort_children(float (&k)[8], int32_t (&v)[8]) {
  constexpr int net[19][2] = {{0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 1}, {2, 3},
                              {4, 5}, {6, 7}, {2, 4}, {3, 5}, {1, 4}, {3, 6}, {1, 2}, {3, 4}, {5, 6}};
#pragma unroll
  for (int c = 0; c < 19; ++c) cswap(k[net[c][0]], v[net[c][0]], k[net[c][1]], v[net[c][1]]);
}

constexpr int TRAV4_STACK = 96;  // up to BVH_WIDTH - 1 entries per level of the wide tree
// Upper bound on node visits of one traversal; a well-formed tree never
// reaches it, a corrupt one ends the traversal instead of looping.
constexpr uint32_t TRAV_MAX_VISITS = 1u << 22;
// Bits of the traversal error word (DevScene::err): a push that found the
// stack full (a subtree was skipped) and a traversal that hit the visit cap.
// Either one makes the render call that saw it return PT_ERR_TRAVERSAL.
constexpr uint32_t TRAV_ERR_STACK = 1u, TRAV_ERR_VISITS = 2u;

static __device__ __noinline__ void trav_error(const DevScene& S, uint32_t bit) {
  if (S.err) atomicOr(S.err, bit);
}

// Closest hit over triangles. Returns id == HIT_MISS when nothing is hit.
struct TravCount {
  uint32_t nodes = 0, tris = 0;
};

template <bool BRUTE, bool COUNT = false>
__device__ __forceinline__ HitRec trace_tris_closest(const DevScene& S, float3 o, float3 d, float tmin, float tmax,
                                                     TravCount* tc = nullptr) {
  HitRec h;
  h.t = tmax;
  h.u = h.v = 0.0f;
  h.id = HIT_MISS;
  if (BRUTE) {
    for (uint32_t s = 0; s < S.num_tris; ++s) {
      float4 a = __ldg(&S.tri[3 * s]), b = __ldg(&S.tri[3 * s + 1]), c = __ldg(&S.tri[3 * s + 2]);
      uint32_t id = __float_as_uint(a.w);
      float t, u, v;
      if (intersect_tri(o, d, f3(a), f3(b), f3(c), tmin, h.t, t, u, v) && (t < h.t || id < h.id)) {
        h.t = t; h.u = u; h.v = v; h.id = id;
      }
    }
    return h;
  }
  if (S.num_tris == 0) return h;
  const SlabRay sr = slab_ray(o, d);
  // (entry distance, link) pairs: one 8-byte local access per push or pop
  float2 st[TRAV4_STACK];
  int sp = 0;
  const int lim = (int)min(S.trav_stack, (uint32_t)TRAV4_STACK);
  int32_t cur = 0;  // root is always internal
  uint32_t visits = 0;
  const uint32_t max_visits = S.trav_visits;
  for (;;) {
    while (cur >= 0) {
      if (++visits > max_visits || cur == EMPTY_LINK) {
        trav_error(S, TRAV_ERR_VISITS);
        return h;
      }
      if (COUNT) tc->nodes++;
      const float4* nd = S.nodes + NODE_F4 * (size_t)cur;
      // nearest first: sort (distance, link) with misses at +inf
      float k[BVH_WIDTH];
      int32_t v[BVH_WIDTH];
      int nh = 0;
#pragma unroll
      for (int g = 0; g < BVH_GROUPS; ++g) {
        float tn[4];
        bool hit[4];
        quad_slabs(nd + 6 * g, sr, tmin, h.t, tn, hit);
        const int4 l = __ldg(reinterpret_cast<const int4*>(nd + 6 * BVH_GROUPS + g));
        const int32_t L[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          k[4 * g + c] = hit[c] ? tn[c] : INF;
          v[4 * g + c] = L[c];
          nh += (int)hit[c];
        }
      }
      sort_children(k, v);
      const int32_t v0 = v[0];
      if (nh == 0) {
        cur = 0x7FFFFFFF;
        while (sp > 0) {
          --sp;
          const float2 e = st[sp];
          if (e.x <= h.t * TRAV_T_SLACK) {
            cur = __float_as_int(e.y);
            break;
          }
        }
        if (cur == 0x7FFFFFFF) return h;
        continue;
      }
      if (sp + nh - 1 > lim) trav_error(S, TRAV_ERR_STACK);  // a far child is dropped below
#pragma unroll
      for (int j = BVH_WIDTH - 1; j >= 1; --j)
        if (nh > j && sp < lim) {
          st[sp] = make_float2(k[j], __int_as_float(v[j]));
          ++sp;
        }
      cur = v0;
    }
    // leaf
    uint32_t start = (uint32_t)cur & 0x03FFFFFFu, count = ((uint32_t)cur >> 26) & 0x1Fu;
    if (COUNT) tc->tris += count;
    for (uint32_t s = start; s < start + count; ++s) {
      float4 a = __ldg(&S.tri[3 * s]), b = __ldg(&S.tri[3 * s + 1]), c = __ldg(&S.tri[3 * s + 2]);
      uint32_t id = __float_as_uint(a.w);
      float t, u, v;
      if (intersect_tri(o, d, f3(a), f3(b), f3(c), tmin, h.t, t, u, v) && (t < h.t || id < h.id)) {
        h.t = t; h.u = u; h.v = v; h.id = id;
      }
    }
    cur = 0x7FFFFFFF;
    while (sp > 0) {
      --sp;
      const float2 e = st[sp];
      if (e.x <= h.t * TRAV_T_SLACK) {
        cur = __float_as_int(e.y);
        break;
      }
    }
    if (cur == 0x7FFFFFFF) return h;
  }
}

template <bool BRUTE>
__device__ __forceinline__ bool trace_tris_any(const DevScene& S, float3 o, float3 d, float tmin, float tmax) {
  if (BRUTE) {
    for (uint32_t s = 0; s < S.num_tris; ++s) {
      float4 a = __ldg(&S.tri[3 * s]), b = __ldg(&S.tri[3 * s + 1]), c = __ldg(&S.tri[3 * s + 2]);
      float t, u, v;
      if (intersect_tri(o, d, f3(a), f3(b), f3(c), tmin, tmax, t, u, v)) return true;
    }
    return false;
  }
  if (S.num_tris == 0) return false;
  const SlabRay sr = slab_ray(o, d);
  int32_t stack[TRAV4_STACK];
  int sp = 0;
  const int lim = (int)min(S.trav_stack, (uint32_t)TRAV4_STACK);
  int32_t cur = 0;
  uint32_t visits = 0;
  const uint32_t max_visits = S.trav_visits;
  for (;;) {
    while (cur >= 0) {
      if (++visits > max_visits || cur == EMPTY_LINK) {
        trav_error(S, TRAV_ERR_VISITS);
        return false;
      }
      const float4* nd = S.nodes + NODE_F4 * (size_t)cur;
      int32_t next = 0x7FFFFFFF;
#pragma unroll
      for (int g = 0; g < BVH_GROUPS; ++g) {
        float tn[4];
        bool hit[4];
        quad_slabs(nd + 6 * g, sr, tmin, tmax, tn, hit);
        const int4 l = __ldg(reinterpret_cast<const int4*>(nd + 6 * BVH_GROUPS + g));
        const int32_t L[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (!hit[c]) continue;
          if (next == 0x7FFFFFFF) next = L[c];
          else if (sp < lim) stack[sp++] = L[c];
          else trav_error(S, TRAV_ERR_STACK);
        }
      }
      if (next == 0x7FFFFFFF) {
        if (sp == 0) return false;
        next = stack[--sp];
      }
      cur = next;
    }
    uint32_t start = (uint32_t)cur & 0x03FFFFFFu, count = ((uint32_t)cur >> 26) & 0x1Fu;
    for (uint32_t s = start; s < start + count; ++s) {
      float4 a = __ldg(&S.tri[3 * s]), b = __ldg(&S.tri[3 * s + 1]), c = __ldg(&S.tri[3 * s + 2]);
      float t, u, v;
      if (intersect_tri(o, d, f3(a), f3(b), f3(c), tmin, tmax, t, u, v)) return true;
    }
    if (sp == 0) return false;
    cur = stack[--sp];
  }
}

// Closest hit including the analytic light geometry. For a light hit,
// u = light pdf (the hit attribute of lights.rint.glsl).
template <bool BRUTE, bool COUNT = false>
__device__ __forceinline__ HitRec trace_closest(const DevScene& S, float3 o, float3 d, float tmin, float tmax,
                                                TravCount* tc = nullptr) {
  HitRec h = trace_tris_closest<BRUTE, COUNT>(S, o, d, tmin, tmax, tc);
  float lbest = (h.id != HIT_MISS) ? h.t : INF;
  for (uint32_t i = 0; i < S.num_lights; ++i) {
    float t, pdf;
    float3 n;
    if (light_hit(S.lights[i], o, d, tmin, tmax, t, n, pdf) && t < lbest) {
      lbest = t;
      h.t = t;
      h.u = pdf;
      h.v = 0.0f;
      h.id = HIT_LIGHT_BIT | i;
    }
  }
  if (h.id == HIT_MISS) h.t = INF;
  return h;
}

template <bool BRUTE>
__device__ __forceinline__ bool trace_any(const DevScene& S, float3 o, float3 d, float tmin, float tmax) {
  for (uint32_t i = 0; i < S.num_lights; ++i) {
    float t, pdf;
    float3 n;
    if (light_hit(S.lights[i], o, d, tmin, tmax, t, n, pdf)) return true;
  }
  return trace_tris_any<BRUTE>(S, o, d, tmin, tmax);
}

}  // namespace hpt
