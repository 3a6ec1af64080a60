// pt_impl.h -- host-side objects shared by the single-scene renderer
// (pt_api.cu) and the job server (pt_serve.cu): device buffers, the
// wavefront path state and the bounce loop that drives one wave.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "pt_internal.h"

namespace hpt {

// Stream on which Buf allocates and frees (stream-ordered allocator) on
// this host thread; null = plain cudaMalloc/cudaFree. cudaFree waits for the
// whole device, so a thread that uploads a scene while another thread's
// wavefronts run allocates through a scope on its own stream instead.
inline thread_local cudaStream_t tl_alloc_stream = nullptr;
struct AllocScope {
  cudaStream_t prev;
  explicit AllocScope(cudaStream_t s) : prev(tl_alloc_stream) { tl_alloc_stream = s; }
  ~AllocScope() { tl_alloc_stream = prev; }
  AllocScope(const AllocScope&) = delete;
  AllocScope& operator=(const AllocScope&) = delete;
};

template <class T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // stream of a stream-ordered allocation
  bool pooled = false;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() { release(); }
  void release() {
    if (p) {
      if (pooled) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    pooled = false;
  }
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e;
    if (tl_alloc_stream) {
      e = cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), tl_alloc_stream);
      pooled = e == cudaSuccess;
      s = tl_alloc_stream;
    } else {
      e = cudaMalloc(&p, count * sizeof(T));
    }
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
};

// The bounce loop of one wave as a single CUDA graph launch: a while node
// whose body is two bounces (even, then odd queue parity). Each bounce is a
// switch node over grid sizes (4096 x 4^k paths, the last one the wavefront
// capacity) whose case the previous one-thread control kernel picks from the
// live-path count, so tail bounces launch small grids without a host round
// trip. Kernel parameters are captured by value: the graph is rebuilt when
// the bytes it captured (scene record, path state, queues) change.
struct BounceGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<unsigned char> key;
  uint32_t builds = 0;  // graphs captured (instantiated or updated) so far
  BounceGraph() = default;
  BounceGraph(const BounceGraph&) = delete;
  BounceGraph& operator=(const BounceGraph&) = delete;
  ~BounceGraph() { reset(); }
  void reset();
};

// Structure-of-arrays state and queues of one wavefront of `cap` paths.
// `med` adds the medium fields, `multi` the per-path job slot of a shared
// wavefront.
struct WaveBuffers {
  uint32_t cap = 0;
  bool med = false, multi = false;
  Buf<uint4> rng;
  Buf<float4> ray_o, ray_d, hit, thr, rad, albedo, normal, med0;
  Buf<float2> med1;
  Buf<float4> sh_o, sh_d0, sh_d1, sh_c0, sh_c1, sh_T, sh_f0, sh_f1;
  Buf<uint32_t> depth, flags, job;
  Buf<uint32_t> q_a, q_b, q_diff, q_dis, q_glass, q_shadow, counters;
  Buf<unsigned long long> rays;
  PathState P{};
  BounceGraph graph;
  cudaError_t ensure(uint32_t cap, bool med, bool multi);
  // Frees every buffer and the bounce graph (cap back to 0).
  void release();
  // Bytes one path slot occupies (state + queues), for memory budgets.
  static uint64_t bytes_per_path(bool med, bool multi);
};

// Options and results of the bounce loop of one wave.
struct BounceLoop {
  uint32_t profiling = 0;            // PT_PROFILE_* flags (any flag selects the host-driven loop)
  bool host_loop = false;            // one host round trip per bounce instead of the bounce graph
  std::vector<cudaEvent_t>* tev = nullptr;  // start/stop pairs around closest-hit launches
  size_t ntimed = 0;
  uint32_t bounces = 0;              // bounces run by the last wave
  bool timed_out = false;            // paths still alive after the bounce cap
  uint64_t launches = 0;             // kernels launched by the last wave's bounces
  uint32_t tail_paths = 16384;       // live paths at or below which the rest of a wave is one k_tail launch
};

// Runs bounce after bounce of the `live` paths queued in W.q_a (the camera
// kernel wrote their count to counters[Q_COUNT + Q_NEXT]) until no path
// continues, at most 4 * max_depth + 4096 bounces. Without profiling flags
// the loop is one launch of W.graph and one read-back of (bounces, live);
// otherwise the host reads the continuing-path count after every bounce.
// `pinned` is at least two uint32_t of pinned host memory.
cudaError_t run_bounces(const DevScene& S, WaveBuffers& W, uint32_t live, uint32_t max_depth, BounceLoop& L,
                        uint32_t* pinned, cudaStream_t st);

// The graph form of run_bounces (pt_graph.cu). Control words live after the
// two counter sets: counters[2 * Q_COUNT + G_*].
// G_TAIL: the most bounces a path ran in the wave's k_tail launch (0 before it).
enum GraphWord : uint32_t { G_DONE = 0, G_LIVE = 1, G_GO = 2, G_TAIL = 3, G_WORDS = 4 };

// The wave-tail threshold in effect: none under the traversal-timing or
// counting instrumentation (which instruments the wavefront's closest-hit
// launches).
inline uint32_t tail_paths(const BounceLoop& L, const WaveBuffers&) {
  if ((L.profiling & (PT_PROFILE_TRACE_TIMING | PT_PROFILE_COUNT)) != 0) return 0;
  return L.tail_paths;
}
cudaError_t run_bounces_graph(const DevScene& S, WaveBuffers& W, uint32_t bounce_cap, BounceLoop& L,
                              uint32_t* pinned, cudaStream_t st);

}  // namespace hpt

struct pt_renderer {
  pt_tracer_config cfg{};
  cudaStream_t stream = nullptr;
  std::string err;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // second stream of the commit: the environment's alias tables are built on
  // it while the BVH builds on `stream`
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  uint32_t* pinned = nullptr;

  // scene
  std::vector<pt_material> mats;
  std::vector<pt_light> lights;
  std::vector<pt_camera> cams;
  uint32_t camera_index = 0;
  uint32_t nverts = 0, ntris = 0, nnodes = 0;
  bool has_scene = false, committed = false;
  hpt::Buf<float> raw_verts;
  hpt::Buf<uint32_t> raw_idx;
  hpt::Buf<hpt::PrimUpload> dprims;
  hpt::Buf<float4> vnorm, vtan, tri_shade, wpos, tri_v0, tri_e1, tri_e2, tri_sorted, nodes;
  hpt::Buf<float2> vuv;
  hpt::Buf<uint32_t> tri_vidx, tri_mat;
  hpt::Buf<pt_material> dmats;
  hpt::Buf<uint32_t> dmat_class;
  std::vector<uint32_t> mat_class;  // host copy (kept alive for the asynchronous upload)
  hpt::Buf<float4> tex_texels;
  hpt::Buf<uint4> tex_info;
  uint32_t num_textures = 0;

  // environment
  bool env_map = false;
  uint32_t env_w = 0, env_h = 0;
  float env_rotation = 0.0f, env_intensity = 1.0f;
  float ground[4] = {0, 0, 0, 1}, sky[4] = {0, 0, 0, 1};
  float exposure = 0.0f;
  double env_total = 1.0;
  hpt::Buf<float4> env;
  hpt::Buf<uint2> alias_rows, alias_cols;
  // loaded blue-noise texture (load_blue_noise_texture), else the substitute
  hpt::Buf<uchar4> blue_noise;
  bool has_blue_noise = false;

  hpt::DevScene view{};
  uint32_t features = 0;

  // wavefront
  hpt::WaveBuffers W;
  uint32_t auto_wave_paths = 0;  // default wavefront size, chosen at the first render (wave_paths = 0)

  // images
  hpt::Buf<float4> accum, albedo, normal;
  hpt::Buf<uchar4> final_img;
  hpt::Buf<float4> keep_rad;
  hpt::Buf<uint32_t> keep_hash;
  uint64_t keep_count = 0;
  uint64_t frame_index = 0;
  pt_stats stats{};
  uint32_t profiling = 0;
  std::vector<cudaEvent_t> tev;  // start/stop pairs around closest-hit launches
  uint32_t bvh_build = PT_BVH_BUILD_SAH;  // pt_renderer_set_bvh_build
  uint32_t tail_paths = PT_TAIL_PATHS_AUTO; // pt_renderer_set_tail_paths
  bool has_glass = false;                  // some material can sample the glass lobe
  // traversal limits and the device word their violations set (TRAV_ERR_*)
  uint32_t trav_stack = 96, trav_visits = 1u << 22;
  hpt::Buf<uint32_t> errw;

  // radiance cache (pt_renderer_set_radiance_cache)
  bool cache_on = false;
  pt_cache_config cache_cfg{};
  pt_cache* cache = nullptr;
  uint64_t cache_paths_seen = 0;  // paths rendered since the cache was attached
  uint32_t c_cap = 0;
  hpt::Buf<float4> c_rec, c_T, t_rec, t_T, t_R, c_tgt;
  hpt::Buf<uint32_t> c_queue, c_train, c_counts;
};

namespace hpt {
// Frees the build-time inputs of a committed scene (raw vertices, indices,
// unsorted triangles): rendering needs only the flattened attributes, the
// BVH and the sorted triangles.
void renderer_drop_build_inputs(pt_renderer* r);
// Frees everything of a finished render but its four images.
void renderer_drop_scene(pt_renderer* r);
// pt_renderer_create with a stream priority (cudaStreamCreateWithPriority;
// lower numbers run first).
pt_status renderer_create_with_priority(const pt_tracer_config* cfg, int priority, pt_renderer** out);
// Checks of set_scene / HalaRenderer::new; `why` receives the reason.
pt_status validate_scene_desc(const pt_scene_desc* desc, std::string* why);
pt_status validate_tracer_config(const pt_tracer_config* config, std::string* why);
// Device bytes a renderer for `desc` at width x height would hold after
// commit (scene, BVH, environment tables, images), without wave buffers.
uint64_t renderer_estimate_bytes(const pt_scene_desc* desc, uint32_t width, uint32_t height, uint32_t env_w,
                                 uint32_t env_h);
}  // namespace hpt

// The C entry points are function-try-blocks whose handler returns this:
// PT_ERR_OOM for a host allocation failure (std::bad_alloc), otherwise
// PT_ERR_INVALID_ARG, with the exception's text left in *err (the handle's
// last-error string) when there is one. No C++ exception unwinds into a C
// caller. Call it only from a catch handler.
inline pt_status host_exception_status(std::string* err) noexcept {
  auto note = [err](const char* m) noexcept {
    if (!err) return;
    try {
      *err = m;
    } catch (...) {
    }
  };
  try {
    throw;
  } catch (const std::bad_alloc&) {
    note("out of host memory");
    return PT_ERR_OOM;
  } catch (const std::exception& e) {
    note(e.what());
    return PT_ERR_INVALID_ARG;
  } catch (...) {
    note("unexpected C++ exception");
    return PT_ERR_INVALID_ARG;
  }
}

