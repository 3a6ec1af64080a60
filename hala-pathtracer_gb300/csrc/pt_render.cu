// pt_render.cu -- wavefront kernels of the GB300 path tracer.
//
// One wavefront = a contiguous range of global path indices
// g = frame_local * (W*H) + pixel. Per bounce the kernels run in this order:
//
//   k_trace        closest hit for every active path (pathtracer.rgen.glsl:56-68);
//                  a miss (environment), an emitter hit (MIS) or an invalid
//                  material (pathtracer.rgen.glsl:70-115) ends the path right
//                  there, any other hit sorts the path into the queue of its
//                  material class
//   k_shade<MAT>   one kernel per material type (diffuse / Disney): emission,
//                  media, transparency, next-event estimation, BSDF sampling,
//                  Russian roulette (pathtracer.rgen.glsl:117-256)
//   k_shadow       shadow rays of the pending next-event estimation and the
//                  radiance update it implies (inc/lighting.glsl:116-149, 203-238)
//   k_transmit     instead of k_shadow in scenes with media: the transmittance
//                  rays of next-event estimation (inc/lighting.glsl:7-61)
//
// Scenes with media use VOL_MIS like the reference host (src/bin/hala-pathtracer.rs:102-103).
// With a transparent material their transmittance loop draws from the path
// RNG between the light samples, so the shade kernel evaluates it in-thread;
// without one it draws nothing and is deferred to k_transmit.
// Once few paths of a wave are left, k_tail (pt_shade.cuh) runs their
// remaining bounces in one launch.
//
// Every kernel is a grid-stride loop over a queue whose length lives in
// device memory, so a bounce needs no host round trip.
#include <cuda_runtime.h>

#include "pt_shade.cuh"

namespace hpt {

// ------------------------------------------------------------------ camera
// perspective_ray.rcall.glsl:12-65, orthographic_ray.rcall.glsl:12-46,
// state initialisation pathtracer.rgen.glsl:23-54
__device__ __forceinline__ void init_path(const DevScene& S, const PathState& P, uint32_t i, uint64_t g) {
  const uint64_t WH = (uint64_t)S.width * S.height;
  uint32_t pix = (uint32_t)(g % WH);
  uint32_t frame = (uint32_t)(g / WH);
  uint32_t px = pix % S.width, py = pix / S.width;
  uint32_t sf = frame + S.seed;
  uint4 s0 = rng_seed_s0(px, py, sf);
  uint4 s1 = rng_seed_s1(sf);
  float4 r = rand4blue(s1, (int)px, (int)py, S.blue_noise);
  const DevCamera& cam = S.cam;
  float r1 = 2.0f * r.x, r2 = 2.0f * r.y;
  float jx = r1 < 1.0f ? sqrtf(r1) - 1.0f : 1.0f - sqrtf(2.0f - r1);
  float jy = r2 < 1.0f ? sqrtf(r2) - 1.0f : 1.0f - sqrtf(2.0f - r2);
  float W = (float)S.width, H = (float)S.height;
  jx /= (W * 0.5f);
  jy /= (H * 0.5f);
  float sx = (float)px / W, sy = (H - (float)py) / H;
  float dx = (2.0f * sx - 1.0f) + jx;
  float dy = (2.0f * sy - 1.0f) + jy;
  float3 o, d;
  if (cam.type == PT_CAMERA_ORTHOGRAPHIC) {
    d = normalize(f3(cam.forward));
    o = f3(cam.position) + f3(cam.right) * (dx * cam.fd_or_xmag) + f3(cam.up) * (dy * cam.ap_or_ymag);
  } else {
    float scale = pm_tan(cam.yfov * 0.5f);
    dx *= scale * W / H;
    dy *= scale;
    float3 rd = normalize(f3(cam.right) * dx + f3(cam.up) * dy + f3(cam.forward));
    o = f3(cam.position);
    d = rd;
    if (cam.ap_or_ymag > 0.0f) {
      float3 focal = cam.fd_or_xmag * rd;
      float c1 = r.z * TWO_PI;
      float c2 = r.w * cam.ap_or_ymag;
      float3 ap = (pm_cos(c1) * f3(cam.right) + pm_sin(c1) * f3(cam.up)) * sqrtf(c2);
      d = normalize(focal - ap);
      o = o + ap;
    }
  }
  P.rng[i] = s0;
  P.ray_o[i] = make_float4(o.x, o.y, o.z, 0.0f);
  P.ray_d[i] = make_float4(d.x, d.y, d.z, 0.0f);
  P.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  P.rad[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(HASH_INIT));
  P.depth[i] = 0;
  P.flags[i] = 0;
  P.albedo[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  P.normal[i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
  if (P.med0) {
    P.med0[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.med1[i] = make_float2(1.0f, __uint_as_float(PT_MEDIUM_NONE));
  }
  if (P.c_train) P.c_train[i] = 0xFFFFFFFFu;
}

// Queue position of path slot i: slots are read as rows of `width` (slot
// i + width is the pixel below slot i), and each band of 4 rows is queued
// tile by tile, 8 x 4 pixels per tile, so that the 32 paths of a warp start
// from a compact patch of the image instead of a 32-pixel strip. A bijection
// on [0, n): slots past the last whole band, and widths that are not a
// multiple of 8, keep their own position. Only the order in which the
// kernels visit paths changes, not any path's result.
__device__ __forceinline__ uint32_t tiled_position(uint32_t i, uint32_t n, uint32_t width) {
  if (width % 8u != 0u) return i;
  const uint64_t band = 4ull * width;
  const uint64_t b = i / band;
  if ((b + 1) * band > n) return i;
  const uint32_t r = (uint32_t)(i - b * band), ly = r / width, col = r % width;
  return (uint32_t)(b * band) + (col >> 3) * 32u + ly * 8u + (col & 7u);
}

__global__ void k_camera(const __grid_constant__ DevScene S, PathState P, uint64_t g0, uint32_t n,
                         uint32_t* q_active, uint32_t* active_count) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  init_path(S, P, i, g0 + i);
  q_active[tiled_position(i, n, S.width)] = i;
  if (i == 0) *active_count = n;
}

// Shared wavefront of several jobs: slot i belongs to the segment whose
// [start, start + count) holds it; the path is that job's index g0 + (i - start).
__global__ void k_camera_multi(PathState P, const WaveSegment* segs, uint32_t nseg, uint32_t n, uint32_t* q_active,
                               uint32_t* active_count) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t lo = 0, hi = nseg;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) / 2;
    if (segs[mid].start <= i) lo = mid;
    else hi = mid;
  }
  const WaveSegment sg = segs[lo];
  P.job[i] = sg.slot;
  init_path(P.jobs[sg.slot], P, i, sg.g0 + (i - sg.start));
  q_active[i] = i;
  if (i == 0) *active_count = n;
}

// ------------------------------------------------------------------ trace
// Traversal kernels (k_trace, k_shadow): 128-thread blocks, 9 per SM, which
// gives them 56 registers and no spills at 36 warps per SM. Measured on the
// GB300 against 256 x 5 (48 registers, spills in the node loop): k_trace
// 6.28 -> 6.04 ms per launch, Disney grid 741 -> 753 Mpaths/s, displaced
// icosphere 1228 -> 1261, media box 93.8 -> 94.2.
constexpr uint32_t TRACE_BLOCK = 128;
constexpr int TRACE_BLOCKS_PER_SM = 9;

// The surface logic of a path whose ray missed, hit an emitter or an invalid
// material, called from k_trace after its traversal (out of line, so that
// the traversal loop keeps its registers).
template <bool MULTI>
__device__ __noinline__ void logic_call(const DevScene& S0, const PathState& P, uint32_t p) {
  logic_path<MULTI>(S0, P, p);
}

template <bool BRUTE, bool COUNT, bool MULTI>
__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_BLOCKS_PER_SM)
    k_trace(const __grid_constant__ DevScene S0, PathState P, QueueSet Q) {
  const uint32_t n = *Q.in_count;
  TravCount tc;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t p = Q.in[i];
    const uint32_t cls = trace_path<BRUTE, COUNT, MULTI>(S0, P, p, tc);
    if (cls == 0) logic_call<MULTI>(S0, P, p);  // miss / emitter / invalid material: the path ends here
    queue_push(Q.diffuse, &Q.counts[Q_DIFFUSE], p, cls == MAT_CLASS_DIFFUSE);
    queue_push(Q.disney, &Q.counts[Q_DISNEY], p, cls == MAT_CLASS_DISNEY);
    queue_push(Q.glass, &Q.counts[Q_GLASS], p, cls == MAT_CLASS_GLASS);
    count_add(&Q.rays[0], 1u);
  }
  if (COUNT) {
    atomicAdd(&Q.rays[2], (unsigned long long)tc.nodes);
    atomicAdd(&Q.rays[3], (unsigned long long)tc.tris);
  }
}

// ------------------------------------------------------------------ shadow rays
template <bool BRUTE, bool MULTI>
__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_BLOCKS_PER_SM)
    k_shadow(const __grid_constant__ DevScene S0, PathState P, QueueSet Q) {
  const uint32_t n = Q.counts[Q_SHADOW];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    count_add(&Q.rays[1], shadow_path<BRUTE, MULTI>(S0, P, Q.shadow[i]));
}

// Next-event rays of vertices with media when no material is transparent
// (inc/lighting.glsl:7-61 and :69-244: transmittance, visibility, then
// radiance += T * Ld), deferred from the shading kernels like k_shadow's.
template <bool MULTI>
__global__ void __launch_bounds__(256, 4) k_transmit(const __grid_constant__ DevScene S0, PathState P, QueueSet Q) {
  const uint32_t n = Q.counts[Q_SHADOW];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    count_add(&Q.rays[1], transmit_path<MULTI>(S0, P, Q.shadow[i]));
}

// ------------------------------------------------------------------ accumulation
// pathtracer.rgen.glsl:259-278: running mean per pixel in frame order.
// Global path index g = frame * WH + pixel (frame counted from the last
// reset); the wave holds g in [g0, g0 + n), its slot is g - g0.
__global__ void k_accumulate(PathState P, uint64_t g0, uint32_t n, uint32_t WH, float4* accum, float4* albedo,
                             float4* normal, float4* keep_rad, uint32_t* keep_hash, uint64_t keep_g0,
                             uint32_t wave_off) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= WH) return;
  const uint64_t g1 = g0 + n;
  uint64_t g = g0 + (((uint64_t)pix + WH - (g0 % WH)) % WH);
  if (g >= g1) return;
  float4 a = accum[pix], b = albedo[pix], c = normal[pix];
  for (; g < g1; g += WH) {
    uint32_t i = wave_off + (uint32_t)(g - g0);
    float4 r = P.rad[i];
    float4 al = P.albedo[i];
    float4 nm = P.normal[i];
    uint64_t frame = g / WH;
    if (frame == 0) {
      a = make_float4(r.x, r.y, r.z, 1.0f);
      b = make_float4(al.x, al.y, al.z, 1.0f);
      c = make_float4(nm.x, nm.y, nm.z, 1.0f);
    } else {
      float t = 1.0f / ((float)frame + 1.0f);
      float3 na = mix(f3(a), f3(r), t), nb = mix(f3(b), f3(al), t), nc = mix(f3(c), f3(nm), t);
      a = make_float4(na.x, na.y, na.z, 1.0f);
      b = make_float4(nb.x, nb.y, nb.z, 1.0f);
      c = make_float4(nc.x, nc.y, nc.z, 1.0f);
    }
    if (keep_rad) {
      keep_rad[g - keep_g0] = make_float4(r.x, r.y, r.z, 0.0f);
      keep_hash[g - keep_g0] = __float_as_uint(r.w);
    }
  }
  accum[pix] = a;
  albedo[pix] = b;
  normal[pix] = c;
}

// Training targets of the radiance cache: what the unbiased path gathered
// after leaving the cache vertex (its indirect light there), divided by the
// throughput arriving at the vertex; zero when the path ended at the vertex.
__global__ void k_cache_targets(PathState P, uint32_t n, float4* tgt) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t k = P.c_train[i];
  if (k == 0xFFFFFFFFu) return;
  float4 r = P.rad[i], R = P.t_R[k], T = P.t_T[k];
  if (R.x != R.x) {
    tgt[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  float3 y = make_float3(T.x > 0.0f ? (r.x - R.x) / T.x : 0.0f, T.y > 0.0f ? (r.y - R.y) / T.y : 0.0f,
                         T.z > 0.0f ? (r.z - R.z) / T.z : 0.0f);
  tgt[k] = make_float4(fmaxf(y.x, 0.0f), fmaxf(y.y, 0.0f), fmaxf(y.z, 0.0f), 0.0f);
}

// pathtracer.rgen.glsl:280-304
__global__ void k_finalize(const float4* accum, uchar4* final_img, uint32_t WH, float ev, int enable, int aces,
                           int simple) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= WH) return;
  float3 c = finish_color(f3(accum[pix]), ev, enable != 0, aces != 0, simple != 0);
  final_img[pix] = make_uchar4(to_unorm8(c.x), to_unorm8(c.y), to_unorm8(c.z), 255);
}

// ------------------------------------------------------------------ geometry queries
template <bool BRUTE>
__global__ void k_trace_rays(const __grid_constant__ DevScene S, const float4* rays, uint32_t n, int any_hit,
                             uint4* hits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = rays[2 * i], b = rays[2 * i + 1];
  if (any_hit) {
    bool occ = trace_any<BRUTE>(S, f3(a), f3(b), a.w, b.w);
    hits[i] = make_uint4(__float_as_uint(occ ? 0.0f : INF), 0u, 0u, occ ? 0u : HIT_MISS);
  } else {
    HitRec h = trace_closest<BRUTE>(S, f3(a), f3(b), a.w, b.w);
    hits[i] = make_uint4(__float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v), h.id);
  }
}

__global__ void k_gather_samples(const float4* keep_rad, const uint32_t* keep_hash, const uint64_t* idx, uint32_t n,
                                 float4* out_rad, uint32_t* out_hash) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = idx[i];
  out_rad[i] = keep_rad[k];
  out_hash[i] = keep_hash[k];
}

// ------------------------------------------------------------------ launchers
// One thread per queued item (the queue length is at most max_items): the
// block scheduler then balances long and short traversals across SMs.
static inline int grid_for(uint32_t max_items, uint32_t block = 256) {
  uint32_t want = (max_items + block - 1) / block;
  return (int)(want < 1 ? 1 : want);
}

void launch_camera(const DevScene& S, const PathState& P, uint64_t g0, uint32_t n, uint32_t* q_active,
                   uint32_t* active_count, cudaStream_t st) {
  k_camera<<<(n + 255) / 256, 256, 0, st>>>(S, P, g0, n, q_active, active_count);
}

void launch_trace(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items, bool count,
                  cudaStream_t st) {
  const int g = grid_for(max_items, TRACE_BLOCK);
  const bool multi = P.job != nullptr;
  if (multi) {
    if (count) k_trace<false, true, true><<<g, TRACE_BLOCK, 0, st>>>(S, P, Q);
    else k_trace<false, false, true><<<g, TRACE_BLOCK, 0, st>>>(S, P, Q);
  } else {
    if (count) k_trace<false, true, false><<<g, TRACE_BLOCK, 0, st>>>(S, P, Q);
    else k_trace<false, false, false><<<g, TRACE_BLOCK, 0, st>>>(S, P, Q);
  }
}

void launch_shade(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items, cudaStream_t st) {
  const int g = grid_for(max_items), gs = grid_for(max_items, TRACE_BLOCK);
  const bool med = (S.features & PT_FEATURE_MEDIUM) != 0;
  const bool tr = (S.features & PT_FEATURE_TRANSPARENT) != 0;
  const bool tex = (S.features & PT_FEATURE_TEXTURED) != 0;
  if (P.job) {
    if (med) launch_materials_multi_medium(S, P, Q, g, tr, tex, st);
    else launch_materials_multi(S, P, Q, g, tr, tex, st);
    if (!med) k_shadow<false, true><<<gs, TRACE_BLOCK, 0, st>>>(S, P, Q);
    else if (!tr) k_transmit<true><<<g, 256, 0, st>>>(S, P, Q);
  } else {
    if (med) launch_materials_medium(S, P, Q, g, tr, tex, st);  // the cache is refused for scenes with media
    else if (P.c_rec != nullptr) launch_materials_cache(S, P, Q, g, tr, tex, st);
    else launch_materials_plain(S, P, Q, g, tr, tex, st);
    if (!med) k_shadow<false, false><<<gs, TRACE_BLOCK, 0, st>>>(S, P, Q);
    else if (!tr) k_transmit<false><<<g, 256, 0, st>>>(S, P, Q);
  }
}

void launch_tail(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                 const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, cudaStream_t st) {
  const bool med = (S.features & PT_FEATURE_MEDIUM) != 0;
  const bool tr = (S.features & PT_FEATURE_TRANSPARENT) != 0;
  const bool tex = (S.features & PT_FEATURE_TEXTURED) != 0;
  if (P.job) {
    if (med) launch_tail_multi_medium(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
    else launch_tail_multi(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
  } else {
    if (med) launch_tail_medium(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
    else if (P.c_rec != nullptr) launch_tail_cache(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
    else launch_tail_plain(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
  }
}

void launch_cache_targets(const PathState& P, uint32_t n, float4* tgt, cudaStream_t st) {
  k_cache_targets<<<(n + 255) / 256, 256, 0, st>>>(P, n, tgt);
}

void launch_camera_multi(const PathState& P, const WaveSegment* segs, uint32_t nseg, uint32_t n, uint32_t* q_active,
                         uint32_t* active_count, cudaStream_t st) {
  k_camera_multi<<<(n + 255) / 256, 256, 0, st>>>(P, segs, nseg, n, q_active, active_count);
}

void launch_accumulate(const PathState& P, uint64_t g0, uint32_t n, uint32_t WH, float4* accum, float4* albedo,
                       float4* normal, float4* keep_rad, uint32_t* keep_hash, uint64_t keep_g0, cudaStream_t st,
                       uint32_t wave_off) {
  k_accumulate<<<(WH + 255) / 256, 256, 0, st>>>(P, g0, n, WH, accum, albedo, normal, keep_rad, keep_hash, keep_g0,
                                                 wave_off);
}

void launch_finalize(const float4* accum, uchar4* final_img, uint32_t WH, float ev, int enable, int aces, int simple,
                     cudaStream_t st) {
  k_finalize<<<(WH + 255) / 256, 256, 0, st>>>(accum, final_img, WH, ev, enable, aces, simple);
}

void launch_gather_samples(const float4* keep_rad, const uint32_t* keep_hash, const uint64_t* idx, uint32_t n,
                           float4* out_rad, uint32_t* out_hash, cudaStream_t st) {
  k_gather_samples<<<(n + 255) / 256, 256, 0, st>>>(keep_rad, keep_hash, idx, n, out_rad, out_hash);
}

void launch_trace_rays(const DevScene& S, const float4* rays, uint32_t n, int any_hit, int brute, uint4* hits,
                       cudaStream_t st) {
  if (brute) k_trace_rays<true><<<(n + 127) / 128, 128, 0, st>>>(S, rays, n, any_hit, hits);
  else k_trace_rays<false><<<(n + 127) / 128, 128, 0, st>>>(S, rays, n, any_hit, hits);
}

}  // namespace hpt
