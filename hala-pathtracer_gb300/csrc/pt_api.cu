// pt_api.cu -- the C ABI (include/hala_pt.h): renderer lifecycle, scene
// upload, progressive rendering, image read-back.
//
// Ownership: the renderer owns every device allocation; host arrays passed
// in are copied before the call returns. Errors never abort: each call
// returns a pt_status and leaves a message in pt_renderer_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pt_cache.h"
#include "pt_impl.h"

namespace hpt {

int device_sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 132;
  }
  return sms;
}

cudaError_t WaveBuffers::ensure(uint32_t want, bool want_med, bool want_multi) {
  if (cap >= want && rng.p && (med || !want_med) && (multi || !want_multi)) return cudaSuccess;
  want = std::max(want, cap);
  want_med = want_med || (med && cap > 0);
  want_multi = want_multi || (multi && cap > 0);
  cap = 0;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  chk(rng.ensure(want));
  chk(ray_o.ensure(want));
  chk(ray_d.ensure(want));
  chk(hit.ensure(want));
  chk(thr.ensure(want));
  chk(rad.ensure(want));
  chk(albedo.ensure(want));
  chk(normal.ensure(want));
  chk(depth.ensure(want));
  chk(flags.ensure(want));
  if (want_med) {
    chk(med0.ensure(want));
    chk(med1.ensure(want));
    chk(sh_f0.ensure(want));
    chk(sh_f1.ensure(want));
  }
  if (want_multi) chk(job.ensure(want));
  chk(sh_o.ensure(want));
  chk(sh_d0.ensure(want));
  chk(sh_d1.ensure(want));
  chk(sh_c0.ensure(want));
  chk(sh_c1.ensure(want));
  chk(sh_T.ensure(want));
  chk(q_a.ensure(want));
  chk(q_b.ensure(want));
  chk(q_diff.ensure(want));
  chk(q_dis.ensure(want));
  chk(q_glass.ensure(want));
  chk(q_shadow.ensure(want));
  chk(counters.ensure(2 * Q_COUNT + G_WORDS));
  chk(rays.ensure(4));
  if (e != cudaSuccess) return e;
  cap = want;
  med = want_med;
  multi = want_multi;
  P.rng = rng.p;
  P.ray_o = ray_o.p;
  P.ray_d = ray_d.p;
  P.hit = hit.p;
  P.thr = thr.p;
  P.rad = rad.p;
  P.depth = depth.p;
  P.flags = flags.p;
  P.albedo = albedo.p;
  P.normal = normal.p;
  P.med0 = med ? med0.p : nullptr;
  P.med1 = med ? med1.p : nullptr;
  P.sh_f0 = med ? sh_f0.p : nullptr;
  P.sh_f1 = med ? sh_f1.p : nullptr;
  P.sh_o = sh_o.p;
  P.sh_d0 = sh_d0.p;
  P.sh_d1 = sh_d1.p;
  P.sh_c0 = sh_c0.p;
  P.sh_c1 = sh_c1.p;
  P.sh_T = sh_T.p;
  P.job = multi ? job.p : nullptr;
  return cudaSuccess;
}

void WaveBuffers::release() {
  graph.reset();
  Buf<uint4>* b4[] = {&rng};
  for (auto* b : b4) b->release();
  Buf<float4>* f4[] = {&ray_o, &ray_d, &hit, &thr, &rad, &albedo, &normal, &med0,
                       &sh_o, &sh_d0, &sh_d1, &sh_c0, &sh_c1, &sh_T, &sh_f0, &sh_f1};
  for (auto* b : f4) b->release();
  med1.release();
  Buf<uint32_t>* u[] = {&depth, &flags, &job, &q_a, &q_b, &q_diff, &q_dis, &q_glass, &q_shadow, &counters};
  for (auto* b : u) b->release();
  rays.release();
  cap = 0;
  med = multi = false;
  P = PathState{};
}

uint64_t WaveBuffers::bytes_per_path(bool med, bool multi) {
  // rng 16, ray_o/ray_d/hit/thr/rad/albedo/normal 7x16, depth+flags 8,
  // six NEE float4 96, six queues 24 (+ medium 24 and two NEE float4 32,
  // + job slot 4)
  return 16 + 7 * 16 + 8 + 96 + 24 + (med ? 56 : 0) + (multi ? 4 : 0);
}

cudaError_t run_bounces(const DevScene& S, WaveBuffers& W, uint32_t live, uint32_t max_depth, BounceLoop& L,
                        uint32_t* pinned, cudaStream_t st) {
  uint32_t* cnt0 = W.counters.p;
  uint32_t* cnt1 = W.counters.p + Q_COUNT;
  const uint32_t bounce_cap = 4u * max_depth + 4096u;
  // trace, 3 shades, and shadow rays (k_shadow, or k_transmit with media
  // unless a material is transparent)
  const bool med_tr = (S.features & PT_FEATURE_MEDIUM) && (S.features & PT_FEATURE_TRANSPARENT);
  const uint64_t per_bounce = med_tr ? 4 : 5;
  if (live == 0) {
    L.bounces = 0;
    L.timed_out = false;
    L.launches = 0;
    return cudaSuccess;
  }
  if (L.profiling == 0 && !L.host_loop) return run_bounces_graph(S, W, bounce_cap, L, pinned, st);
  const bool timing = (L.profiling & PT_PROFILE_TRACE_TIMING) != 0 && L.tev;
  const uint32_t tail = tail_paths(L, W);
  uint32_t* tail_word = W.counters.p + 2 * Q_COUNT + G_TAIL;
  uint32_t b = 0, tail_bounces = 0;
  for (; b < bounce_cap && live > 0; ++b) {
    uint32_t* out = (b & 1) ? cnt1 : cnt0;
    uint32_t* in_cnt = ((b & 1) ? cnt0 : cnt1) + Q_NEXT;
    uint32_t* qin = (b & 1) ? W.q_b.p : W.q_a.p;
    uint32_t* qnext = (b & 1) ? W.q_a.p : W.q_b.p;
    cudaError_t e = cudaMemsetAsync(out, 0, Q_COUNT * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    QueueSet Q{qin, in_cnt, qnext, W.q_diff.p, W.q_dis.p, W.q_glass.p, W.q_shadow.p, out,
                 W.rays.p};
    if (live <= tail) {
      // the rest of the wave in one kernel: the loop ends here
      if ((e = cudaMemsetAsync(tail_word, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      launch_tail(S, W.P, Q, live, nullptr, b, bounce_cap, tail_word, st);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if ((e = cudaMemcpyAsync(pinned, out + Q_NEXT, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
      if ((e = cudaMemcpyAsync(pinned + 1, tail_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      live = pinned[0];
      tail_bounces = pinned[1];
      b += tail_bounces;
      break;
    }
    if (timing) {
      while (L.tev->size() < 2 * (L.ntimed + 1)) {
        cudaEvent_t ev;
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return e;
        L.tev->push_back(ev);
      }
      if ((e = cudaEventRecord((*L.tev)[2 * L.ntimed], st)) != cudaSuccess) return e;
    }
    launch_trace(S, W.P, Q, live, (L.profiling & PT_PROFILE_COUNT) != 0, st);
    if (timing) {
      if ((e = cudaEventRecord((*L.tev)[2 * L.ntimed + 1], st)) != cudaSuccess) return e;
      ++L.ntimed;
    }
    launch_shade(S, W.P, Q, live, st);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(pinned, out + Q_NEXT, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    live = pinned[0];
  }
  L.bounces = b;
  L.timed_out = live > 0;
  L.launches = per_bounce * (b - tail_bounces) + (tail_bounces ? 1 : 0);
  return cudaSuccess;
}

pt_status validate_scene_desc(const pt_scene_desc* s, std::string* why) {
  auto bad = [&](pt_status st, const char* m) {
    if (why) *why = m;
    return st;
  };
  if (!s) return bad(PT_ERR_INVALID_ARG, "scene is null");
  if (s->num_cameras == 0 || !s->cameras) return bad(PT_ERR_INVALID_ARG, "scene has no camera");
  if (s->num_cameras > PT_MAX_CAMERAS) return bad(PT_ERR_INVALID_ARG, "more than 8 cameras");
  if (s->num_lights > PT_MAX_LIGHTS) return bad(PT_ERR_INVALID_ARG, "more than 16 lights");
  if (s->num_primitives && !s->primitives) return bad(PT_ERR_INVALID_ARG, "primitives is null");
  if (s->num_materials && !s->materials) return bad(PT_ERR_INVALID_ARG, "materials is null");
  if (s->num_lights && !s->lights) return bad(PT_ERR_INVALID_ARG, "lights is null");
  if (s->num_textures && !s->textures) return bad(PT_ERR_INVALID_ARG, "textures is null");
  for (uint32_t i = 0; i < s->num_textures; ++i) {
    const pt_texture& t = s->textures[i];
    if (t.width == 0 || t.height == 0 || !t.rgba) return bad(PT_ERR_INVALID_ARG, "empty texture");
    if ((uint64_t)t.width * t.height > (1ull << 28)) return bad(PT_ERR_UNSUPPORTED, "texture larger than 2^28 texels");
  }
  // Sizes first: a leaf link holds the first triangle of its leaf in 26 bits,
  // so a scene of 2^26 triangles or more cannot be traversed.
  uint64_t nv = 0, nt = 0;
  for (uint32_t i = 0; i < s->num_primitives; ++i) {
    const pt_primitive& p = s->primitives[i];
    if (p.num_indices % 3 != 0) return bad(PT_ERR_INVALID_ARG, "index count is not a multiple of 3");
    if ((p.num_vertices && !p.vertices) || (p.num_indices && !p.indices))
      return bad(PT_ERR_INVALID_ARG, "primitive arrays are null");
    nv += p.num_vertices;
    nt += p.num_indices / 3;
  }
  if (nt >= (1ull << 26) || nv >= (1ull << 31))
    return bad(PT_ERR_UNSUPPORTED, "scene exceeds 2^26 triangles or 2^31 vertices");
  for (uint32_t i = 0; i < s->num_primitives; ++i) {
    const pt_primitive& p = s->primitives[i];
    for (uint32_t k = 0; k < p.num_indices; ++k)
      if (p.indices[k] >= p.num_vertices) return bad(PT_ERR_INVALID_ARG, "index out of range");
  }
  return PT_OK;
}

pt_status validate_tracer_config(const pt_tracer_config* c, std::string* why) {
  auto bad = [&](pt_status st, const char* m) {
    if (why) *why = m;
    return st;
  };
  if (!c) return bad(PT_ERR_INVALID_ARG, "config is null");
  // src/config/window.rs:13-21 and src/config/tracer.rs:43-49
  if (c->width == 0 || c->height == 0) return bad(PT_ERR_INVALID_ARG, "width and height must be positive");
  if (c->rr_depth > c->max_depth) return bad(PT_ERR_INVALID_ARG, "rr_depth exceeds max_depth");
  if ((uint64_t)c->width * c->height > (1ull << 31)) return bad(PT_ERR_UNSUPPORTED, "more than 2^31 pixels");
  return PT_OK;
}

void renderer_drop_build_inputs(pt_renderer* r) {
  r->raw_verts.release();
  r->raw_idx.release();
  r->dprims.release();
  r->wpos.release();
  r->tri_v0.release();
  r->tri_e1.release();
  r->tri_e2.release();
}

void renderer_drop_scene(pt_renderer* r) {
  renderer_drop_build_inputs(r);
  r->vnorm.release();
  r->vtan.release();
  r->tri_shade.release();
  r->vuv.release();
  r->tri_sorted.release();
  r->nodes.release();
  r->tri_vidx.release();
  r->tri_mat.release();
  r->dmats.release();
  r->dmat_class.release();
  r->env.release();
  r->alias_rows.release();
  r->alias_cols.release();
  r->tex_texels.release();
  r->tex_info.release();
  r->committed = false;
  r->has_scene = false;
}

uint64_t renderer_estimate_bytes(const pt_scene_desc* d, uint32_t width, uint32_t height, uint32_t env_w,
                                 uint32_t env_h) {
  uint64_t nv = 0, nt = 0;
  for (uint32_t i = 0; i < d->num_primitives; ++i) {
    nv += d->primitives[i].num_vertices;
    nt += d->primitives[i].num_indices / 3;
  }
  const uint64_t V = std::max<uint64_t>(nv, 1), T = std::max<uint64_t>(nt, 1);
  // vertices: raw 44 + normal/tangent/position 48 + uv 8
  // triangles: raw indices 12 + v0/e1/e2 48 + sorted 48 + wide nodes
  // (capacity one per triangle, at most 256 B each) 256 + vertex ids 12 + material 4 + shading
  // record 96; the BVH build's scratch (binary nodes and queues) is about
  // 190 B more
  uint64_t b = V * 100 + T * (476 + 190);
  b += (uint64_t)d->num_materials * sizeof(pt_material) + 4096;
  for (uint32_t i = 0; i < d->num_textures; ++i) b += 16ull * d->textures[i].width * d->textures[i].height + 16;
  const uint64_t E = (uint64_t)env_w * env_h;
  b += E * (16 + 8 + 16 + 8) + (uint64_t)env_h * 16;
  b += (uint64_t)width * height * (3 * 16 + 4);
  return b;
}

}  // namespace hpt

using namespace hpt;

namespace {

pt_status fail(pt_renderer* r, pt_status s, const std::string& msg) {
  if (r) r->err = msg;
  return s;
}
pt_status cuda_fail(pt_renderer* r, cudaError_t e, const char* what) {
  pt_status s = (e == cudaErrorMemoryAllocation) ? PT_ERR_OOM : PT_ERR_CUDA;
  return fail(r, s, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(r, call)                                         \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail((r), e_, #call); \
  } while (0)

// Upper-left 3x3 inverse transpose by cofactors (column-major input), the
// same float operations as the oracle (this file is built without FMA
// contraction).
void normal_matrix(const float* T, float N[9]) {
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
  for (int i = 0; i < 9; ++i) N[i] = C[i] / det;
}

// Shading kernel of a material (MAT_CLASS_*). The glass lobe's weight is
// (1 - metallic) * specular_transmission, computed as the lobe probabilities
// compute it. A weight that is zero or NaN gives a zero or NaN probability,
// so the lobe is never evaluated or sampled (a negative weight can still
// give a positive probability through a negative normalisation, so only
// zero and NaN count). A metallic-roughness map replaces metallic per hit,
// so there only a zero transmission rules the lobe out.
uint32_t material_class(const pt_material& m, uint32_t num_textures) {
  if (m.type != PT_MATERIAL_DISNEY) return MAT_CLASS_DIFFUSE;
  if (m.specular_transmission == 0.0f) return MAT_CLASS_DISNEY;
  if (m.metallic_roughness_map_index < num_textures) return MAT_CLASS_GLASS;
  const float glass_wt = (1.0f - m.metallic) * m.specular_transmission;
  return (glass_wt > 0.0f || glass_wt < 0.0f) ? MAT_CLASS_GLASS : MAT_CLASS_DISNEY;
}

void fill_view(pt_renderer* r) {
  DevScene& S = r->view;
  S = DevScene{};
  S.tri = r->tri_sorted.p;
  S.nodes = r->nodes.p;
  S.tri_vidx = r->tri_vidx.p;
  S.tri_mat = r->tri_mat.p;
  S.vnorm = r->vnorm.p;
  S.vtan = r->vtan.p;
  S.tri_shade = r->tri_shade.p;
  S.vuv = r->vuv.p;
  S.mats = r->dmats.p;
  S.mat_class = r->dmat_class.p;
  S.num_mats = (uint32_t)r->mats.size();
  S.num_tris = r->ntris;
  S.num_lights = (uint32_t)r->lights.size();
  for (uint32_t i = 0; i < S.num_lights; ++i) {
    const pt_light& l = r->lights[i];
    DevLight& d = S.lights[i];
    std::memcpy(d.intensity, l.intensity, 12);
    std::memcpy(d.position, l.position, 12);
    std::memcpy(d.u, l.u, 12);
    std::memcpy(d.v, l.v, 12);
    d.radius = l.radius;
    d.area = l.area;
    d.type = l.type;
    d.pad = 0;
  }
  const pt_camera& c = r->cams[r->camera_index < r->cams.size() ? r->camera_index : 0];
  std::memcpy(S.cam.position, c.position, 12);
  std::memcpy(S.cam.right, c.right, 12);
  std::memcpy(S.cam.up, c.up, 12);
  std::memcpy(S.cam.forward, c.forward, 12);
  S.cam.yfov = c.yfov;
  S.cam.fd_or_xmag = c.focal_distance_or_xmag;
  S.cam.ap_or_ymag = c.aperture_or_ymag;
  S.cam.type = c.type;
  S.env_map = r->env_map ? 1u : 0u;
  S.env_rgba = r->env.p;
  S.alias_rows = r->alias_rows.p;
  S.alias_cols = r->alias_cols.p;
  S.env_w = r->env_w;
  S.env_h = r->env_h;
  S.env_rotation = r->env_rotation;
  S.env_intensity = r->env_intensity;
  S.env_total_sum = (float)(r->env_total * (double)r->env_intensity);
  std::memcpy(S.ground, r->ground, 12);
  std::memcpy(S.sky, r->sky, 12);
  S.width = r->cfg.width;
  S.height = r->cfg.height;
  S.max_depth = r->cfg.max_depth;
  S.rr_depth = r->cfg.rr_depth;
  S.seed = r->cfg.seed;
  S.features = r->features;
  S.tex_texels = r->tex_texels.p;
  S.tex_info = r->tex_info.p;
  S.num_textures = r->num_textures;
  S.trav_stack = r->trav_stack;
  S.trav_visits = r->trav_visits;
  S.err = r->errw.p;
  S.blue_noise = r->has_blue_noise ? r->blue_noise.p : nullptr;
}

// Reads and clears the traversal error word (stream-ordered; synchronises).
pt_status check_traversal(pt_renderer* r) {
  uint32_t* h = r->pinned + 8;
  CK(r, cudaMemcpyAsync(h, r->errw.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, r->stream));
  CK(r, cudaStreamSynchronize(r->stream));
  const uint32_t w = *h;
  if (w == 0) return PT_OK;
  CK(r, cudaMemsetAsync(r->errw.p, 0, sizeof(uint32_t), r->stream));
  std::string m = "BVH traversal exceeded its limits (";
  if (w & 1u) m += "stack of " + std::to_string(std::min<uint32_t>(r->trav_stack, 96)) + " entries full";
  if ((w & 3u) == 3u) m += ", ";
  if (w & 2u) m += std::to_string(r->trav_visits) + " node visits";
  m += "); the results of this call may be wrong";
  return fail(r, PT_ERR_TRAVERSAL, m);
}

// Default wavefront size: the paths half the free device memory holds, a
// power of two between 2^16 and 2^27.
uint32_t default_wave_paths(bool med) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return 1u << 24;
  }
  const uint64_t fit = (uint64_t)(fr / 2) / WaveBuffers::bytes_per_path(med, false);
  uint32_t w = 1u << 27;
  while (w > (1u << 16) && w > fit) w >>= 1;
  return w;
}

bool write_pfm(const char* path, const float4* px, uint32_t w, uint32_t h) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  std::fprintf(f, "PF\n%u %u\n-1.0\n", w, h);
  std::vector<float> row(3 * (size_t)w);
  for (uint32_t y = 0; y < h; ++y) {
    const float4* src = px + (size_t)(h - 1 - y) * w;  // PFM rows run bottom to top
    for (uint32_t x = 0; x < w; ++x) {
      row[3 * x] = src[x].x;
      row[3 * x + 1] = src[x].y;
      row[3 * x + 2] = src[x].z;
    }
    std::fwrite(row.data(), sizeof(float), row.size(), f);
  }
  return std::fclose(f) == 0;
}

// Creates the renderer's cache on first use (bounds from the BVH root) and
// sizes its per-path buffers for wavefronts of `cap` paths.
pt_status cache_prepare(pt_renderer* r, uint32_t cap) {
  if (r->features & PT_FEATURE_MEDIUM)
    return fail(r, PT_ERR_UNSUPPORTED, "the radiance cache does not support participating media");
  if (!r->cache) {
    pt_status cs = pt_cache_create(&r->cache_cfg, &r->cache);
    if (cs != PT_OK) return fail(r, cs, "radiance cache creation failed");
    float lo[3] = {-1, -1, -1}, hi[3] = {1, 1, 1};
    if (r->nnodes > 0) {
      // union of the root's child boxes (unused slots are +inf: skip them)
      float4 root[6];
      CK(r, cudaMemcpy(root, r->nodes.p, sizeof(root), cudaMemcpyDeviceToHost));
      float b[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY};
      for (int k = 0; k < 4; ++k) {
        const float* q[6] = {&root[0].x, &root[1].x, &root[2].x, &root[3].x, &root[4].x, &root[5].x};
        if (!(q[0][k] < INFINITY)) continue;
        for (int a = 0; a < 3; ++a) {
          b[2 * a] = std::fmin(b[2 * a], q[2 * a][k]);
          b[2 * a + 1] = std::fmax(b[2 * a + 1], q[2 * a + 1][k]);
        }
      }
      for (int i = 0; i < 3; ++i) {
        float l = b[2 * i], h = b[2 * i + 1];
        if (!(h > l)) {
          l -= 1.0f;
          h += 1.0f;
        }
        float pad = 1e-3f * (h - l);
        lo[i] = l - pad;
        hi[i] = h + pad;
      }
    }
    pt_cache_set_bounds(r->cache, lo, hi);
  }
  if (r->c_cap < cap) {
    CK(r, r->c_rec.ensure(4 * (size_t)cap));
    CK(r, r->c_T.ensure(cap));
    CK(r, r->t_rec.ensure(4 * (size_t)cap));
    CK(r, r->t_T.ensure(cap));
    CK(r, r->t_R.ensure(cap));
    CK(r, r->c_tgt.ensure(cap));
    CK(r, r->c_queue.ensure(cap));
    CK(r, r->c_train.ensure(cap));
    CK(r, r->c_counts.ensure(2));
    r->c_cap = cap;
  }
  PathState& P = r->W.P;
  P.c_rec = r->c_rec.p;
  P.c_T = r->c_T.p;
  P.c_queue = r->c_queue.p;
  P.c_counts = r->c_counts.p;
  P.c_train = r->c_train.p;
  P.t_rec = r->t_rec.p;
  P.t_T = r->t_T.p;
  P.t_R = r->t_R.p;
  P.c_depth = r->cache_cfg.query_depth;
  P.c_shift = r->cache_cfg.train_shift;
  P.c_min_rough = r->cache_cfg.min_roughness;
  P.c_mode = 2;
  return PT_OK;
}

void cache_detach(pt_renderer* r) {
  PathState& P = r->W.P;
  P.c_rec = P.c_T = P.t_rec = P.t_T = P.t_R = nullptr;
  P.c_queue = P.c_counts = P.c_train = nullptr;
}

}  // namespace

extern "C" {

uint32_t pt_abi_version(void) { return PT_ABI_VERSION; }

void pt_material_default(pt_material* m) {
  if (!m) return;
  std::memset(m, 0, sizeof(*m));
  m->base_color[0] = m->base_color[1] = m->base_color[2] = 1.0f;
  m->opacity = 1.0f;
  m->clearcoat_tint[0] = m->clearcoat_tint[1] = m->clearcoat_tint[2] = 1.0f;
  m->ior = 1.5f;
  m->medium.anisotropy = 0.0f;
  m->medium.type = PT_MEDIUM_NONE;
  m->base_color_map_index = m->normal_map_index = PT_INVALID_INDEX;
  m->metallic_roughness_map_index = m->emission_map_index = PT_INVALID_INDEX;
  m->type = PT_MATERIAL_DIFFUSE;
  pt_material_preprocess(m);
}

// Disney (inc/bxdf/disney.glsl:420): GGX alphas roughness^2 / aspect and
// roughness^2 * aspect, aspect = sqrt(1 - 0.9 anisotropic), clamped >= 0.001.
// Diffuse (inc/bxdf/oren_nayar.glsl:35-46): Oren-Nayar A, B with
// sigma = roughness * pi / 2.
void pt_material_preprocess(pt_material* m) {
  if (!m) return;
  float r = m->roughness;
  if (m->type == PT_MATERIAL_DISNEY) {
    float aspect = std::sqrt(1.0f - 0.9f * m->anisotropic);
    m->ax = std::fmax(0.001f, (r * r) / aspect);
    m->ay = std::fmax(0.001f, (r * r) * aspect);
  } else {
    float sigma = r * 1.57079637f;
    float s2 = sigma * sigma;
    m->ax = 1.0f - s2 / (2.0f * (s2 + 0.33f));
    m->ay = 0.45f * s2 / (s2 + 0.09f);
  }
}

pt_status pt_renderer_create(const pt_tracer_config* cfg, pt_renderer** out) try {
  return renderer_create_with_priority(cfg, 0, out);
} catch (...) {
  return host_exception_status(nullptr);
}

}  // extern "C"

namespace {
// The stream-ordered allocator of each device keeps freed blocks for reuse
// instead of returning them to the driver at every synchronisation, so
// renderers created one after another (jobs of a serving loop, repeated
// end-to-end renders) reuse the wavefront and scene buffers of the last one.
void keep_pool_memory(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> g(mu);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done.push_back(device);
}
}  // namespace

pt_status hpt::renderer_create_with_priority(const pt_tracer_config* cfg, int priority, pt_renderer** out) {
  if (!cfg || !out) return PT_ERR_INVALID_ARG;
  *out = nullptr;
  pt_status cs = validate_tracer_config(cfg, nullptr);
  if (cs != PT_OK) return cs;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PT_ERR_CUDA;
  int device = 0;
  cudaGetDevice(&device);
  keep_pool_memory(device);
  pt_renderer* r = new pt_renderer();
  r->cfg = *cfg;
  if (cudaStreamCreateWithPriority(&r->stream, cudaStreamNonBlocking, priority) != cudaSuccess ||
      cudaStreamCreateWithPriority(&r->side, cudaStreamNonBlocking, priority) != cudaSuccess ||
      cudaEventCreate(&r->ev0) != cudaSuccess || cudaEventCreate(&r->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&r->pinned, 64) != cudaSuccess) {
    pt_renderer_destroy(r);
    return PT_ERR_CUDA;
  }
  size_t WH = (size_t)cfg->width * cfg->height;
  AllocScope as(r->stream);
  if (r->accum.ensure(WH) || r->albedo.ensure(WH) || r->normal.ensure(WH) || r->final_img.ensure(WH) ||
      r->errw.ensure(1)) {
    pt_renderer_destroy(r);
    return PT_ERR_OOM;
  }
  cudaMemsetAsync(r->errw.p, 0, sizeof(uint32_t), r->stream);
  cudaMemsetAsync(r->accum.p, 0, WH * sizeof(float4), r->stream);
  cudaMemsetAsync(r->albedo.p, 0, WH * sizeof(float4), r->stream);
  cudaMemsetAsync(r->normal.p, 0, WH * sizeof(float4), r->stream);
  cudaMemsetAsync(r->final_img.p, 0, WH * sizeof(uchar4), r->stream);
  *out = r;
  return PT_OK;
}

extern "C" {

void pt_renderer_destroy(pt_renderer* r) {
  if (!r) return;
  if (r->stream) cudaStreamSynchronize(r->stream);
  if (r->side) cudaStreamSynchronize(r->side);
  if (r->ev0) cudaEventDestroy(r->ev0);
  if (r->ev1) cudaEventDestroy(r->ev1);
  if (r->ev_fork) cudaEventDestroy(r->ev_fork);
  if (r->ev_join) cudaEventDestroy(r->ev_join);
  if (r->pinned) cudaFreeHost(r->pinned);
  for (cudaEvent_t e : r->tev) cudaEventDestroy(e);
  if (r->cache) pt_cache_destroy(r->cache);
  cudaStream_t s = r->stream;
  delete r;
  if (s) cudaStreamDestroy(s);
}

const char* pt_renderer_last_error(const pt_renderer* r) { return r ? r->err.c_str() : "null renderer"; }

pt_status pt_renderer_set_scene(pt_renderer* r, const pt_scene_desc* s) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  {
    std::string why;
    pt_status vs = validate_scene_desc(s, &why);
    if (vs != PT_OK) return fail(r, vs, why);
  }
  std::vector<PrimUpload> prims(s->num_primitives);
  uint64_t nv = 0, nt = 0;
  for (uint32_t i = 0; i < s->num_primitives; ++i) {
    const pt_primitive& p = s->primitives[i];
    PrimUpload& u = prims[i];
    u.vbase = (uint32_t)nv;
    u.tbase = (uint32_t)nt;
    u.nverts = p.num_vertices;
    u.ntris = p.num_indices / 3;
    for (int row = 0; row < 3; ++row)
      for (int col = 0; col < 4; ++col) u.xf[row * 4 + col] = p.transform[col * 4 + row];
    normal_matrix(p.transform, u.nm);
    u.material = p.material_index;
    nv += p.num_vertices;
    nt += p.num_indices / 3;
  }
  r->committed = false;
  r->has_scene = false;
  r->nverts = (uint32_t)nv;
  r->ntris = (uint32_t)nt;
  r->mats.assign(s->materials, s->materials + s->num_materials);
  r->lights.assign(s->lights, s->lights + s->num_lights);
  r->cams.assign(s->cameras, s->cameras + s->num_cameras);
  cudaStream_t st = r->stream;
  CK(r, r->raw_verts.ensure(11 * (size_t)std::max<uint64_t>(nv, 1)));
  CK(r, r->raw_idx.ensure(3 * (size_t)std::max<uint64_t>(nt, 1)));
  CK(r, r->dprims.ensure(std::max<size_t>(prims.size(), 1)));
  {
    // every primitive's vertices and indices packed back to back on the host,
    // then one copy each: one call per primitive costs more than the bytes
    // (a copy from pageable memory has taken its source when it returns)
    std::vector<float> hv(11 * (size_t)nv);
    std::vector<uint32_t> hi(3 * (size_t)nt);
    for (uint32_t i = 0; i < s->num_primitives; ++i) {
      const pt_primitive& p = s->primitives[i];
      if (p.num_vertices)
        std::memcpy(hv.data() + 11 * (size_t)prims[i].vbase, p.vertices, 11 * sizeof(float) * (size_t)p.num_vertices);
      if (p.num_indices)
        std::memcpy(hi.data() + 3 * (size_t)prims[i].tbase, p.indices, sizeof(uint32_t) * p.num_indices);
    }
    if (nv) CK(r, cudaMemcpyAsync(r->raw_verts.p, hv.data(), hv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    if (nt) CK(r, cudaMemcpyAsync(r->raw_idx.p, hi.data(), hi.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  }
  if (!prims.empty())
    CK(r, cudaMemcpyAsync(r->dprims.p, prims.data(), prims.size() * sizeof(PrimUpload), cudaMemcpyHostToDevice, st));
  size_t V = std::max<uint64_t>(nv, 1), T = std::max<uint64_t>(nt, 1);
  CK(r, r->vnorm.ensure(V));
  CK(r, r->vtan.ensure(V));
  CK(r, r->tri_shade.ensure(6 * T));
  CK(r, r->vuv.ensure(V));
  CK(r, r->wpos.ensure(V));
  CK(r, r->tri_v0.ensure(T));
  CK(r, r->tri_e1.ensure(T));
  CK(r, r->tri_e2.ensure(T));
  CK(r, r->tri_vidx.ensure(3 * T));
  CK(r, r->tri_mat.ensure(T));
  CK(r, r->dmats.ensure(std::max<size_t>(r->mats.size(), 1)));
  {
    std::vector<uint32_t>& cls = r->mat_class;
    cls.resize(r->mats.size());
    r->has_glass = false;
    for (size_t i = 0; i < r->mats.size(); ++i) {
      cls[i] = material_class(r->mats[i], s->num_textures);
      r->has_glass = r->has_glass || cls[i] == MAT_CLASS_GLASS;
    }
    CK(r, r->dmat_class.ensure(std::max<size_t>(cls.size(), 1)));
    if (!cls.empty())
      CK(r, cudaMemcpyAsync(r->dmat_class.p, cls.data(), cls.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  }
  if (!r->mats.empty())
    CK(r, cudaMemcpyAsync(r->dmats.p, r->mats.data(), r->mats.size() * sizeof(pt_material), cudaMemcpyHostToDevice,
                          st));
  {
    // material textures, back to back (texels are RGBA32F already)
    std::vector<uint4> info(s->num_textures);
    uint64_t total = 0;
    for (uint32_t i = 0; i < s->num_textures; ++i) {
      info[i] = make_uint4((uint32_t)total, s->textures[i].width, s->textures[i].height, 0u);
      total += (uint64_t)s->textures[i].width * s->textures[i].height;
    }
    if (total >= (1ull << 32)) return fail(r, PT_ERR_UNSUPPORTED, "more than 2^32 texels in all textures");
    r->num_textures = s->num_textures;
    CK(r, r->tex_info.ensure(std::max<size_t>(info.size(), 1)));
    CK(r, r->tex_texels.ensure(std::max<uint64_t>(total, 1)));
    if (!info.empty())
      CK(r, cudaMemcpyAsync(r->tex_info.p, info.data(), info.size() * sizeof(uint4), cudaMemcpyHostToDevice, st));
    for (uint32_t i = 0; i < s->num_textures; ++i)
      CK(r, cudaMemcpyAsync(r->tex_texels.p + info[i].x, s->textures[i].rgba,
                            sizeof(float4) * (size_t)info[i].y * info[i].z, cudaMemcpyHostToDevice, st));
  }
  launch_flatten(r->raw_verts.p, r->raw_idx.p, r->dprims.p, (uint32_t)prims.size(), r->nverts, r->ntris, nullptr,
                 nullptr, r->vnorm.p, r->vtan.p, r->vuv.p, r->wpos.p, r->tri_v0.p, r->tri_e1.p, r->tri_e2.p,
                 r->tri_vidx.p, r->tri_mat.p, r->tri_shade.p, st);
  CK(r, cudaGetLastError());
  CK(r, cudaStreamSynchronize(st));
  r->has_scene = true;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_envmap(pt_renderer* r, const float* rgb, uint32_t w, uint32_t h, float rot_deg) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  r->committed = false;
  if (!rgb || w == 0 || h == 0) {
    r->env_map = false;
    return PT_OK;
  }
  // RGB as given, widened to RGBA on the device
  const size_t n = (size_t)w * h;
  Buf<float> rgb_dev;
  CK(r, rgb_dev.ensure(3 * n));
  CK(r, r->env.ensure(n));
  CK(r, cudaMemcpyAsync(rgb_dev.p, rgb, 3 * n * sizeof(float), cudaMemcpyHostToDevice, r->stream));
  launch_env_widen(rgb_dev.p, r->env.p, n, r->stream);
  CK(r, cudaGetLastError());
  CK(r, cudaStreamSynchronize(r->stream));
  r->env_map = true;
  r->env_w = w;
  r->env_h = h;
  // hdri_rotation is given in degrees (conf/*.yaml); the shaders use turns.
  r->env_rotation = rot_deg / 360.0f;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_ground_color(pt_renderer* r, const float rgba[4]) try {
  if (!r || !rgba) return PT_ERR_INVALID_ARG;
  std::memcpy(r->ground, rgba, 16);
  r->view.ground[0] = rgba[0]; r->view.ground[1] = rgba[1]; r->view.ground[2] = rgba[2];
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}
pt_status pt_renderer_set_sky_color(pt_renderer* r, const float rgba[4]) try {
  if (!r || !rgba) return PT_ERR_INVALID_ARG;
  std::memcpy(r->sky, rgba, 16);
  r->view.sky[0] = rgba[0]; r->view.sky[1] = rgba[1]; r->view.sky[2] = rgba[2];
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}
pt_status pt_renderer_set_env_intensity(pt_renderer* r, float v) try {
  if (!r) return PT_ERR_INVALID_ARG;
  r->env_intensity = v;
  r->view.env_intensity = v;
  r->view.env_total_sum = (float)(r->env_total * (double)v);
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}
pt_status pt_renderer_set_exposure_value(pt_renderer* r, float v) try {
  if (!r) return PT_ERR_INVALID_ARG;
  r->exposure = v;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}
pt_status pt_renderer_set_blue_noise(pt_renderer* r, const uint8_t* rgba8) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (!rgba8) {
    r->has_blue_noise = false;
  } else {
    AllocScope alloc_scope(r->stream);
    const size_t n = (size_t)PT_BLUE_NOISE_SIZE * PT_BLUE_NOISE_SIZE;
    CK(r, r->blue_noise.ensure(n));
    CK(r, cudaMemcpyAsync(r->blue_noise.p, rgba8, n * sizeof(uchar4), cudaMemcpyHostToDevice, r->stream));
    CK(r, cudaStreamSynchronize(r->stream));
    r->has_blue_noise = true;
  }
  if (r->committed) fill_view(r);
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_camera_index(pt_renderer* r, uint32_t i) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (r->has_scene && i >= r->cams.size()) return fail(r, PT_ERR_INVALID_ARG, "camera index out of range");
  r->camera_index = i;
  if (r->committed) fill_view(r);
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_commit(pt_renderer* r) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  if (!r->has_scene) return fail(r, PT_ERR_STATE, "set_scene must come before commit");
  // feature permutation, src/bin/hala-pathtracer.rs:101-114
  uint32_t f = 0;
  for (const pt_material& m : r->mats) {
    if (m.medium.type != PT_MEDIUM_NONE) f |= PT_FEATURE_MEDIUM | PT_FEATURE_VOL_MIS;
    if (m.opacity < 1.0f) f |= PT_FEATURE_TRANSPARENT;
    if (m.base_color_map_index < r->num_textures || m.normal_map_index < r->num_textures ||
        m.metallic_roughness_map_index < r->num_textures || m.emission_map_index < r->num_textures)
      f |= PT_FEATURE_TEXTURED;
  }
  r->features = f;
  cudaStream_t st = r->stream;
  // environment alias tables (FP64, one thread per row) on the side stream,
  // concurrently with the BVH build; joined before the commit returns
  Buf<double> q, sums, tot;
  Buf<uint32_t> stacks;
  // Declared after the scratch buffers so that on every return the main
  // stream waits for the side stream before their stream-ordered frees.
  struct Join {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    ~Join() {
      if (st) cudaStreamWaitEvent(st, ev, 0);
    }
  } join;
  if (r->env_map) {
    const size_t WH = (size_t)r->env_w * r->env_h;
    CK(r, q.ensure(2 * WH));
    CK(r, sums.ensure(r->env_h));
    CK(r, tot.ensure(1));
    CK(r, stacks.ensure(2 * WH));
    CK(r, r->alias_rows.ensure(r->env_h));
    CK(r, r->alias_cols.ensure(WH));
    CK(r, cudaEventRecord(r->ev_fork, st));
    CK(r, cudaStreamWaitEvent(r->side, r->ev_fork, 0));
    launch_env_tables(r->env.p, r->env_w, r->env_h, r->alias_rows.p, r->alias_cols.p, q.p, stacks.p, sums.p, tot.p,
                      r->side);
    const cudaError_t le = cudaGetLastError();
    CK(r, cudaEventRecord(r->ev_join, r->side));
    join.st = st;
    join.ev = r->ev_join;
    CK(r, le);
  }
  CK(r, r->tri_sorted.ensure(3 * (size_t)std::max<uint32_t>(r->ntris, 1)));
  CK(r, cudaEventRecord(r->ev0, st));
  if (r->ntris > 0) {
    // binary SAH tree first (scratch), then its wide collapse for traversal
    Buf<float4> bin;
    const uint32_t cap = 2 * r->ntris;
    CK(r, bin.ensure(4 * (size_t)cap));
    BvhBuffers bb{bin.p, r->tri_sorted.p, cap};
    uint32_t nn = 0, nn4 = 0;
    int rc = r->bvh_build == PT_BVH_BUILD_FAST ? build_bvh_fast(r->tri_v0.p, r->tri_e1.p, r->tri_e2.p, r->ntris, bb, &nn, st)
                                               : build_bvh(r->tri_v0.p, r->tri_e1.p, r->tri_e2.p, r->ntris, bb, &nn, st);
    if (rc == 2) return fail(r, PT_ERR_OOM, "BVH build: out of device memory");
    if (rc != 0) return fail(r, PT_ERR_CUDA, "BVH build failed (code " + std::to_string(rc) + ")");
    // every wide node starts from a distinct internal binary node, and a
    // binary tree of nn nodes has fewer than nn / 2 + 1 of them
    const uint32_t cap_wide = nn / 2 + 1;
    CK(r, r->nodes.ensure(NODE_F4 * (size_t)cap_wide));
    uint32_t leaves = 0;
    rc = collapse_wide(bin.p, nn, r->nodes.p, cap_wide, &nn4, st, &leaves);
    if (rc == 2) return fail(r, PT_ERR_OOM, "BVH collapse: out of device memory");
    if (rc != 0) return fail(r, PT_ERR_CUDA, "BVH collapse failed (code " + std::to_string(rc) + ")");
    r->nnodes = nn4;
    r->stats.bvh_binary_nodes = 2ull * leaves - 1;  // reachable from the root (the build reserves more slots)
  } else {
    r->stats.bvh_binary_nodes = 0;
    CK(r, r->nodes.ensure(NODE_F4));
    r->nnodes = 0;
  }
  CK(r, cudaEventRecord(r->ev1, st));
  CK(r, cudaEventSynchronize(r->ev1));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, r->ev0, r->ev1);
  r->stats.bvh_build_ms = ms;
  r->stats.bvh_nodes = r->nnodes;
  r->stats.triangles = r->ntris;
  if (r->env_map) {
    CK(r, cudaStreamWaitEvent(st, r->ev_join, 0));
    CK(r, cudaMemcpyAsync(&r->env_total, tot.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(r, cudaStreamSynchronize(st));
  }
  fill_view(r);
  r->stats.features = f;
  r->committed = true;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_render(pt_renderer* r, uint32_t frames) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  if (!r->committed) return fail(r, PT_ERR_STATE, "commit must come before render");
  uint64_t nf = frames;
  if (r->cfg.max_samples > 0) {
    if (r->frame_index >= r->cfg.max_samples) nf = 0;
    else nf = std::min<uint64_t>(nf, r->cfg.max_samples - r->frame_index);
  }
  const uint32_t WH = r->cfg.width * r->cfg.height;
  const uint64_t total = nf * WH;
  r->stats.paths = 0;
  r->stats.closest_rays = r->stats.shadow_rays = 0;
  r->stats.render_ms = 0.0;
  if (total == 0) return PT_OK;
  const bool med = (r->features & PT_FEATURE_MEDIUM) != 0;
  const bool auto_wave = r->cfg.wave_paths == 0;
  if (auto_wave && r->auto_wave_paths == 0) r->auto_wave_paths = default_wave_paths(med);
  uint64_t want = auto_wave ? r->auto_wave_paths : r->cfg.wave_paths;
  if (r->cache_on) want = std::min<uint64_t>(want, r->cache_cfg.paths_per_pass);
  uint32_t cap = (uint32_t)std::min<uint64_t>(want, total);
  for (;;) {
    cudaError_t we = r->W.ensure(cap, med, false);
    if (we == cudaSuccess) break;
    // the default size steps down while the device cannot hold it
    if (we != cudaErrorMemoryAllocation || !auto_wave || cap <= (1u << 16)) {
      r->W.release();
      return cuda_fail(r, we, "wavefront buffers");
    }
    cudaGetLastError();
    r->W.release();
    cap >>= 1;
    r->auto_wave_paths = cap;
  }
  if (!r->cache_on) cap = r->W.cap;  // a larger wavefront already allocated costs nothing more
  cudaStream_t st = r->stream;
  const uint64_t g_start = r->frame_index * WH;
  if (r->cfg.keep_samples) {
    CK(r, r->keep_rad.ensure(total));
    CK(r, r->keep_hash.ensure(total));
    r->keep_count = total;
  }
  CK(r, cudaMemsetAsync(r->W.rays.p, 0, 4 * sizeof(unsigned long long), st));
  CK(r, cudaMemsetAsync(r->errw.p, 0, sizeof(uint32_t), st));
  CK(r, cudaEventRecord(r->ev0, st));
  uint32_t max_bounces = 0;
  uint64_t launches = 0;
  BounceLoop L;
  L.profiling = r->profiling;
  L.tail_paths = r->tail_paths;
  if (L.tail_paths == PT_TAIL_PATHS_AUTO) {
    // Paths that refract through glass or scatter in media run long chains
    // of bounces, and the tail kernel lasts as long as its longest path: a
    // wave of such paths goes on in per-bounce launches down to 16384 paths
    // (measured on the GB300: Disney grid 1080p one sample per call 4.87 ms
    // at 16384 against 5.63 at 65536, media box 7.2 against 9.9), one of
    // diffuse and opaque surfaces down to 65536 (displaced icosphere 4.24
    // against 4.86 ms).
    L.tail_paths = (r->has_glass || (r->features & PT_FEATURE_MEDIUM)) ? 16384u : 65536u;
  }
  // With a radiance cache, the paths that go on past the cache vertex are
  // the 1 in 2^train_shift that train it: the tail takes over once only
  // they are left.
  if (r->cache_on && L.tail_paths > 0)
    L.tail_paths = std::max<uint32_t>(L.tail_paths, (uint32_t)(r->cache_cfg.paths_per_pass >> r->cache_cfg.train_shift));
  L.tev = &r->tev;
  const bool use_cache = r->cache_on;
  if (use_cache) {
    pt_status cs = cache_prepare(r, cap);
    if (cs != PT_OK) return cs;
  }
  uint64_t c_queries = 0, c_samples = 0, c_steps = 0;
  for (uint64_t off = 0; off < total;) {
    uint32_t n = (uint32_t)std::min<uint64_t>(cap, total - off);
    PathState P = r->W.P;
    if (use_cache) {
      // warm-up: the first frames after the cache is attached train only
      const uint64_t warm = (uint64_t)r->cache_cfg.warmup_frames * WH;
      P.c_mode = r->cache_paths_seen < warm ? 1u : 2u;
      if (P.c_mode == 1) n = (uint32_t)std::min<uint64_t>(n, warm - r->cache_paths_seen);
      CK(r, cudaMemsetAsync(r->c_counts.p, 0, 2 * sizeof(uint32_t), st));
    }
    uint64_t g0 = g_start + off;
    launch_camera(r->view, P, g0, n, r->W.q_a.p, r->W.counters.p + Q_COUNT + Q_NEXT, st);
    {
      WaveBuffers& W = r->W;
      PathState keep = W.P;
      W.P = P;
      cudaError_t be = run_bounces(r->view, W, n, r->cfg.max_depth, L, r->pinned, st);
      W.P = keep;
      CK(r, be);
    }
    if (L.timed_out) return fail(r, PT_ERR_TIMEOUT, "paths still alive after the bounce cap");
    max_bounces = std::max(max_bounces, L.bounces);
    launches += 2 + L.launches;  // camera + accumulate + bounces
    if (use_cache && P.c_mode == 2) {
      launch_cache_infer(cache_view(r->cache), P.c_rec, P.c_queue, P.c_counts, n, P.rad, P.c_T, st);
      ++launches;
    }
    launch_accumulate(P, g0, n, WH, r->accum.p, r->albedo.p, r->normal.p,
                      r->cfg.keep_samples ? r->keep_rad.p : nullptr, r->cfg.keep_samples ? r->keep_hash.p : nullptr,
                      g_start, st);
    CK(r, cudaGetLastError());
    if (use_cache) {
      launch_cache_targets(P, n, r->c_tgt.p, st);
      CK(r, cudaMemcpyAsync(r->pinned + 4, r->c_counts.p, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      CK(r, cudaStreamSynchronize(st));
      const uint32_t nq = r->pinned[4], ns = r->pinned[5];
      uint32_t steps = 0;
      CK(r, cache_train_device(r->cache, r->t_rec.p, r->c_tgt.p, ns, st, &steps));
      c_queries += P.c_mode == 2 ? nq : 0;
      c_samples += ns;
      c_steps += steps;
      launches += 1 + 4ull * steps;  // targets + per step: forward/backward, dW, two Adam kernels
      r->cache_paths_seen += n;
    }
    off += n;
  }
  const size_t ntimed = L.ntimed;
  launch_finalize(r->accum.p, r->final_img.p, WH, r->exposure, r->cfg.enable_tonemap, r->cfg.enable_aces,
                  r->cfg.use_simple_aces, st);
  CK(r, cudaGetLastError());
  CK(r, cudaEventRecord(r->ev1, st));
  unsigned long long rays[4] = {0, 0, 0, 0};
  CK(r, cudaMemcpyAsync(rays, r->W.rays.p, sizeof(rays), cudaMemcpyDeviceToHost, st));
  CK(r, cudaStreamSynchronize(st));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, r->ev0, r->ev1);
  r->frame_index += nf;
  r->stats.frame_index = r->frame_index;
  r->stats.paths = total;
  r->stats.closest_rays = rays[0];
  r->stats.shadow_rays = rays[1];
  r->stats.render_ms = ms;
  r->stats.max_bounces_seen = max_bounces;
  r->stats.trav_nodes = rays[2];
  r->stats.trav_tris = rays[3];
  r->stats.trace_launches = ntimed;
  r->stats.kernel_launches = launches + 1;  // + finalize
  r->stats.wave_paths = cap;
  r->stats.cache_queries = c_queries;
  r->stats.cache_train_samples = c_samples;
  r->stats.cache_train_steps = c_steps;
  if (use_cache) {
    float lossv = 0.0f;
    cache_last_loss(r->cache, &lossv);
    r->stats.cache_loss = lossv;
  }
  double tms = 0.0;
  for (size_t k = 0; k < ntimed; ++k) {
    float e = 0.0f;
    cudaEventElapsedTime(&e, r->tev[2 * k], r->tev[2 * k + 1]);
    tms += e;
  }
  r->stats.trace_ms = tms;
  return check_traversal(r);
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_radiance_cache(pt_renderer* r, const pt_cache_config* cfg) try {
  if (!r) return PT_ERR_INVALID_ARG;
  CK(r, cudaStreamSynchronize(r->stream));
  if (r->cache) pt_cache_destroy(r->cache);
  r->cache = nullptr;
  r->cache_paths_seen = 0;
  cache_detach(r);
  if (!cfg) {
    r->cache_on = false;
    return PT_OK;
  }
  pt_cache_config c;
  pt_cache_config_default(&c);
  c.query_depth = cfg->query_depth;
  c.train_shift = cfg->train_shift;
  c.warmup_frames = cfg->warmup_frames;
  if (cfg->batch_size) c.batch_size = cfg->batch_size;
  if (cfg->log2_table_size) c.log2_table_size = cfg->log2_table_size;
  if (cfg->learning_rate > 0.0f) c.learning_rate = cfg->learning_rate;
  if (cfg->min_resolution) c.min_resolution = cfg->min_resolution;
  if (cfg->max_resolution) c.max_resolution = cfg->max_resolution;
  if (cfg->paths_per_pass) c.paths_per_pass = cfg->paths_per_pass;
  c.steps_per_pass = cfg->steps_per_pass;
  c.weight_grad_kernel = cfg->weight_grad_kernel;
  c.min_roughness = cfg->min_roughness;
  c.seed = cfg->seed;
  if (c.query_depth == 0) return fail(r, PT_ERR_INVALID_ARG, "query_depth must be at least 1");
  if (c.train_shift > 16) return fail(r, PT_ERR_INVALID_ARG, "train_shift must be at most 16");
  if (r->committed && (r->features & PT_FEATURE_MEDIUM))
    return fail(r, PT_ERR_UNSUPPORTED, "the radiance cache does not support participating media");
  r->cache_cfg = c;
  r->cache_on = true;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_profiling(pt_renderer* r, uint32_t flags) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (flags & ~(PT_PROFILE_TRACE_TIMING | PT_PROFILE_COUNT | PT_PROFILE_HOST_LOOP))
    return fail(r, PT_ERR_INVALID_ARG, "unknown profiling flag");
  r->profiling = flags;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_reset(pt_renderer* r) try {
  if (!r) return PT_ERR_INVALID_ARG;
  size_t WH = (size_t)r->cfg.width * r->cfg.height;
  CK(r, cudaMemsetAsync(r->accum.p, 0, WH * sizeof(float4), r->stream));
  CK(r, cudaMemsetAsync(r->albedo.p, 0, WH * sizeof(float4), r->stream));
  CK(r, cudaMemsetAsync(r->normal.p, 0, WH * sizeof(float4), r->stream));
  CK(r, cudaMemsetAsync(r->final_img.p, 0, WH * sizeof(uchar4), r->stream));
  CK(r, cudaStreamSynchronize(r->stream));
  r->frame_index = 0;
  r->stats.frame_index = 0;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_load_accumulation(pt_renderer* r, const float* accum, const float* albedo, const float* normal,
                                        uint64_t frame_index) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (!accum || !albedo || !normal) return fail(r, PT_ERR_INVALID_ARG, "image pointer is null");
  if (r->cfg.max_samples > 0 && frame_index > r->cfg.max_samples)
    return fail(r, PT_ERR_INVALID_ARG, "frame_index exceeds max_samples");
  const size_t WH = (size_t)r->cfg.width * r->cfg.height;
  CK(r, cudaMemcpyAsync(r->accum.p, accum, WH * sizeof(float4), cudaMemcpyDefault, r->stream));
  CK(r, cudaMemcpyAsync(r->albedo.p, albedo, WH * sizeof(float4), cudaMemcpyDefault, r->stream));
  CK(r, cudaMemcpyAsync(r->normal.p, normal, WH * sizeof(float4), cudaMemcpyDefault, r->stream));
  launch_finalize(r->accum.p, r->final_img.p, (uint32_t)WH, r->exposure, r->cfg.enable_tonemap, r->cfg.enable_aces,
                  r->cfg.use_simple_aces, r->stream);
  CK(r, cudaGetLastError());
  CK(r, cudaStreamSynchronize(r->stream));
  r->frame_index = frame_index;
  r->stats.frame_index = frame_index;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_read_image(pt_renderer* r, pt_image which, void* host, size_t bytes) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (!host) return fail(r, PT_ERR_INVALID_ARG, "host pointer is null");
  const size_t WH = (size_t)r->cfg.width * r->cfg.height;
  CK(r, cudaStreamSynchronize(r->stream));
  switch (which) {
    case PT_IMAGE_ACCUM:
    case PT_IMAGE_ALBEDO:
    case PT_IMAGE_NORMAL: {
      if (bytes != WH * sizeof(float4)) return fail(r, PT_ERR_INVALID_ARG, "image size mismatch");
      const float4* src = which == PT_IMAGE_ACCUM ? r->accum.p : (which == PT_IMAGE_ALBEDO ? r->albedo.p : r->normal.p);
      CK(r, cudaMemcpy(host, src, bytes, cudaMemcpyDefault));
      return PT_OK;
    }
    case PT_IMAGE_FINAL:
      if (bytes != WH * 4) return fail(r, PT_ERR_INVALID_ARG, "image size mismatch");
      CK(r, cudaMemcpy(host, r->final_img.p, bytes, cudaMemcpyDefault));
      return PT_OK;
    case PT_IMAGE_SAMPLE_RADIANCE: {
      if (!r->cfg.keep_samples) return fail(r, PT_ERR_STATE, "keep_samples is off");
      if (bytes != r->keep_count * 12) return fail(r, PT_ERR_INVALID_ARG, "sample buffer size mismatch");
      std::vector<float4> tmp(r->keep_count);
      CK(r, cudaMemcpy(tmp.data(), r->keep_rad.p, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      float* o = (float*)host;
      for (size_t i = 0; i < tmp.size(); ++i) {
        o[3 * i] = tmp[i].x;
        o[3 * i + 1] = tmp[i].y;
        o[3 * i + 2] = tmp[i].z;
      }
      return PT_OK;
    }
    case PT_IMAGE_SAMPLE_HASH:
      if (!r->cfg.keep_samples) return fail(r, PT_ERR_STATE, "keep_samples is off");
      if (bytes != r->keep_count * 4) return fail(r, PT_ERR_INVALID_ARG, "sample buffer size mismatch");
      CK(r, cudaMemcpy(host, r->keep_hash.p, bytes, cudaMemcpyDeviceToHost));
      return PT_OK;
  }
  return fail(r, PT_ERR_INVALID_ARG, "unknown image");
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_save_images(pt_renderer* r, const char* prefix) try {
  if (!r || !prefix) return PT_ERR_INVALID_ARG;
  const uint32_t W = r->cfg.width, H = r->cfg.height;
  const size_t WH = (size_t)W * H;
  std::vector<float4> img(WH);
  std::string p(prefix);
  const pt_image kinds[3] = {PT_IMAGE_ACCUM, PT_IMAGE_ALBEDO, PT_IMAGE_NORMAL};
  const char* names[3] = {"_color.pfm", "_albedo.pfm", "_normal.pfm"};
  for (int k = 0; k < 3; ++k) {
    pt_status s = pt_renderer_read_image(r, kinds[k], img.data(), WH * sizeof(float4));
    if (s != PT_OK) return s;
    if (!write_pfm((p + names[k]).c_str(), img.data(), W, H))
      return fail(r, PT_ERR_INVALID_ARG, "cannot write " + p + names[k]);
  }
  std::vector<unsigned char> rgba(WH * 4);
  pt_status s = pt_renderer_read_image(r, PT_IMAGE_FINAL, rgba.data(), rgba.size());
  if (s != PT_OK) return s;
  FILE* f = std::fopen((p + "_final.ppm").c_str(), "wb");
  if (!f) return fail(r, PT_ERR_INVALID_ARG, "cannot write " + p + "_final.ppm");
  std::fprintf(f, "P6\n%u %u\n255\n", W, H);
  for (size_t i = 0; i < WH; ++i) std::fwrite(&rgba[4 * i], 1, 3, f);
  std::fclose(f);
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_wait_idle(pt_renderer* r) try {
  if (!r) return PT_ERR_INVALID_ARG;
  CK(r, cudaStreamSynchronize(r->stream));
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_get_stats(const pt_renderer* r, pt_stats* out) try {
  if (!r || !out) return PT_ERR_INVALID_ARG;
  *out = r->stats;
  return PT_OK;
} catch (...) {
  return host_exception_status(nullptr);
}

pt_status pt_renderer_get_stream(const pt_renderer* r, void** stream) try {
  if (!r || !stream) return PT_ERR_INVALID_ARG;
  *stream = (void*)r->stream;
  return PT_OK;
} catch (...) {
  return host_exception_status(nullptr);
}

pt_status pt_renderer_trace_rays(pt_renderer* r, const float* rays, uint32_t n, int32_t any_hit, int32_t brute,
                                 uint32_t* hits) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  if (!r->committed) return fail(r, PT_ERR_STATE, "commit must come before trace_rays");
  if (n == 0) return PT_OK;
  if (!rays || !hits) return fail(r, PT_ERR_INVALID_ARG, "null ray or hit buffer");
  Buf<float4> dr;
  Buf<uint4> dh;
  CK(r, dr.ensure(2 * (size_t)n));
  CK(r, dh.ensure(n));
  CK(r, cudaMemcpyAsync(dr.p, rays, 32 * (size_t)n, cudaMemcpyHostToDevice, r->stream));
  CK(r, cudaMemsetAsync(r->errw.p, 0, sizeof(uint32_t), r->stream));
  launch_trace_rays(r->view, dr.p, n, any_hit, brute, dh.p, r->stream);
  CK(r, cudaGetLastError());
  CK(r, cudaMemcpyAsync(hits, dh.p, 16 * (size_t)n, cudaMemcpyDeviceToHost, r->stream));
  CK(r, cudaStreamSynchronize(r->stream));
  return check_traversal(r);
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_bvh_build(pt_renderer* r, uint32_t mode) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (mode != PT_BVH_BUILD_SAH && mode != PT_BVH_BUILD_FAST) return fail(r, PT_ERR_INVALID_ARG, "unknown BVH build");
  r->bvh_build = mode;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_tail_paths(pt_renderer* r, uint32_t paths) try {
  if (!r) return PT_ERR_INVALID_ARG;
  r->tail_paths = paths;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_set_traversal_limits(pt_renderer* r, uint32_t stack_entries, uint32_t max_visits) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (stack_entries > 96) return fail(r, PT_ERR_INVALID_ARG, "the traversal stack holds at most 96 entries");
  r->trav_stack = stack_entries ? stack_entries : 96;
  r->trav_visits = max_visits ? max_visits : (1u << 22);
  r->view.trav_stack = r->trav_stack;
  r->view.trav_visits = r->trav_visits;
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

pt_status pt_renderer_read_samples(pt_renderer* r, const uint64_t* paths, uint32_t n, float* radiance,
                                   uint32_t* hash) try {
  if (!r) return PT_ERR_INVALID_ARG;
  AllocScope alloc_scope(r->stream);
  if (!r->cfg.keep_samples) return fail(r, PT_ERR_STATE, "keep_samples is off");
  if (n == 0) return PT_OK;
  if (!paths) return fail(r, PT_ERR_INVALID_ARG, "path index array is null");
  for (uint32_t i = 0; i < n; ++i)
    if (paths[i] >= r->keep_count) return fail(r, PT_ERR_INVALID_ARG, "path index beyond the last render call");
  Buf<uint64_t> di;
  Buf<float4> dr;
  Buf<uint32_t> dh;
  CK(r, di.ensure(n));
  CK(r, dr.ensure(n));
  CK(r, dh.ensure(n));
  CK(r, cudaMemcpyAsync(di.p, paths, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, r->stream));
  launch_gather_samples(r->keep_rad.p, r->keep_hash.p, di.p, n, dr.p, dh.p, r->stream);
  CK(r, cudaGetLastError());
  std::vector<float4> tmp(n);
  CK(r, cudaMemcpyAsync(tmp.data(), dr.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, r->stream));
  if (hash) CK(r, cudaMemcpyAsync(hash, dh.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, r->stream));
  CK(r, cudaStreamSynchronize(r->stream));
  if (radiance)
    for (uint32_t i = 0; i < n; ++i) {
      radiance[3 * i] = tmp[i].x;
      radiance[3 * i + 1] = tmp[i].y;
      radiance[3 * i + 2] = tmp[i].z;
    }
  return PT_OK;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

}  // extern "C"
