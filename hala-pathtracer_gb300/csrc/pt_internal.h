// pt_internal.h -- host-side interface between the C ABI and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "pt_types.h"

namespace hpt {

// Queues of one bounce (all device pointers).
struct QueueSet {
  const uint32_t* in;        // active paths of this bounce
  const uint32_t* in_count;  // their number
  uint32_t* next;            // paths continuing to the next bounce
  uint32_t* diffuse;
  uint32_t* disney;
  uint32_t* glass;
  uint32_t* shadow;
  uint32_t* counts;            // [Q_COUNT], zeroed at the start of the bounce
  unsigned long long* rays;    // [0] closest rays, [1] shadow rays, [2] nodes, [3] triangle tests
};

int device_sm_count();

// pt_exr.cu: a zlib stream (RFC 1950/1951) into `out`, at most `limit`
// bytes; false on any format error (also used for PNG image data).
bool inflate_zlib(const uint8_t* data, size_t size, std::vector<uint8_t>& out, size_t limit);
// pt_png.cu: a PNG file's bytes as float RGBA in [0, 1] (every colour type
// and bit depth) or as RGBA8 (8-bit and palette images); "" on success,
// otherwise the reason.
std::string png_decode_float(const uint8_t* data, size_t size, uint32_t& w, uint32_t& h, std::vector<float>& rgba);
std::string png_decode_rgba8(const uint8_t* data, size_t size, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba);

// pt_render.cu
void launch_camera(const DevScene& S, const PathState& P, uint64_t g0, uint32_t n, uint32_t* q_active,
                   uint32_t* active_count, cudaStream_t st);
void launch_trace(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items, bool count,
                  cudaStream_t st);
void launch_shade(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items, cudaStream_t st);
// pt_shade_*.cu: the three material kernels of one bounce (diffuse, opaque
// Disney, glass Disney) for single-scene wavefronts without media
// (plain), with media (medium), with a radiance cache (cache), and for
// shared multi-job wavefronts without and with media.
void launch_materials_plain(const DevScene& S, const PathState& P, const QueueSet& Q, int grid, bool tr, bool tex,
                            cudaStream_t st);
void launch_materials_medium(const DevScene& S, const PathState& P, const QueueSet& Q, int grid, bool tr, bool tex,
                             cudaStream_t st);
void launch_materials_cache(const DevScene& S, const PathState& P, const QueueSet& Q, int grid, bool tr, bool tex,
                            cudaStream_t st);
void launch_materials_multi(const DevScene& S, const PathState& P, const QueueSet& Q, int grid, bool tr, bool tex,
                            cudaStream_t st);
void launch_materials_multi_medium(const DevScene& S, const PathState& P, const QueueSet& Q, int grid, bool tr,
                                   bool tex, cudaStream_t st);
// The tail of a wave: every remaining bounce of the paths queued in Q.in,
// one thread per path (k_tail in pt_shade.cuh), at most `cap` bounces in
// the wave counting the `done` (or *done_ptr) already run; the most bounces
// a path ran goes to *tail_bounces (atomicMax).
void launch_tail(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                 const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, cudaStream_t st);
void launch_tail_plain(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                       const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr, bool tex,
                       cudaStream_t st);
void launch_tail_medium(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                        const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr, bool tex,
                        cudaStream_t st);
void launch_tail_cache(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                       const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr, bool tex,
                       cudaStream_t st);
void launch_tail_multi(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                       const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr, bool tex,
                       cudaStream_t st);
void launch_tail_multi_medium(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                              const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr,
                              bool tex, cudaStream_t st);
void launch_camera_multi(const PathState& P, const WaveSegment* segs, uint32_t nseg, uint32_t n, uint32_t* q_active,
                         uint32_t* active_count, cudaStream_t st);
void launch_accumulate(const PathState& P, uint64_t g0, uint32_t n, uint32_t WH, float4* accum, float4* albedo,
                       float4* normal, float4* keep_rad, uint32_t* keep_hash, uint64_t keep_g0, cudaStream_t st,
                       uint32_t wave_off = 0);
void launch_cache_targets(const PathState& P, uint32_t n, float4* tgt, cudaStream_t st);
void launch_finalize(const float4* accum, uchar4* final_img, uint32_t WH, float ev, int enable, int aces, int simple,
                     cudaStream_t st);
// out_rad[i] / out_hash[i] = keep_rad / keep_hash at idx[i] (indices checked by the caller).
void launch_gather_samples(const float4* keep_rad, const uint32_t* keep_hash, const uint64_t* idx, uint32_t n,
                           float4* out_rad, uint32_t* out_hash, cudaStream_t st);
void launch_trace_rays(const DevScene& S, const float4* rays, uint32_t n, int any_hit, int brute, uint4* hits,
                       cudaStream_t st);

// pt_scene.cu: geometry flattening and environment tables
struct PrimUpload {
  uint32_t vbase;       // first global vertex
  uint32_t tbase;       // first global triangle
  uint32_t nverts, ntris;
  float xf[12];         // rows of the 3x4 object-to-world matrix
  float nm[9];          // inverse-transpose of the upper 3x3 (row-major)
  uint32_t material;
};
// Transforms raw vertices (11 floats each) and triangles into world space.
void launch_flatten(const float* raw_verts, const uint32_t* raw_idx, const PrimUpload* prims, uint32_t nprims,
                    uint32_t total_verts, uint32_t total_tris, const uint32_t* vert_prim, const uint32_t* tri_prim,
                    float4* vnorm, float4* vtan, float2* vuv, float4* wpos, float4* tri_v0, float4* tri_e1,
                    float4* tri_e2, uint32_t* tri_vidx, uint32_t* tri_mat, float4* tri_shade, cudaStream_t st);
// FP64 alias tables of the environment map; returns the FP64 luminance sum
// through *total_out (device pointer to one double).
// RGB float triples -> RGBA (alpha 0) environment texels.
void launch_env_widen(const float* rgb, float4* env, size_t n, cudaStream_t st);
void launch_env_tables(const float4* env, uint32_t w, uint32_t h, uint2* rows, uint2* cols, double* scratch_q,
                       uint32_t* scratch_stack, double* row_sums, double* total_out, cudaStream_t st);

// pt_bvh.cu: device BVH build over world-space triangles.
struct BvhBuffers {
  float4* nodes;        // output traversal nodes (4 float4 each)
  float4* tri_sorted;   // output triangles in leaf order (3 float4 each)
  uint32_t node_capacity;
};
// Returns 0 on success; *num_nodes receives the number of nodes used.
int build_bvh(const float4* tri_v0, const float4* tri_e1, const float4* tri_e2, uint32_t ntris, BvhBuffers& out,
              uint32_t* num_nodes, cudaStream_t st);
// pt_bvh_fast.cu: the same output layout from a linear BVH over Morton codes
// (fewer passes, no host round trip per level, a tree of lower quality).
int build_bvh_fast(const float4* tri_v0, const float4* tri_e1, const float4* tri_e2, uint32_t ntris,
                   BvhBuffers& out, uint32_t* num_nodes, cudaStream_t st);
// Collapses the binary tree (64-B nodes) into BVH_WIDTH-wide nodes (NODE_F4
// float4 each, at most cap4 of them); *num_leaves (optional) receives the
// tree's leaf count. Returns 0 on success.
int collapse_wide(const float4* bin, uint32_t nn_bin, float4* out4, uint32_t cap4, uint32_t* num4, cudaStream_t st,
                  uint32_t* num_leaves = nullptr);

}  // namespace hpt
