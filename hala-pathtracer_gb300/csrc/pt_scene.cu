// pt_scene.cu -- scene preparation kernels: world-space flattening of the
// mesh primitives and the FP64 alias tables of the environment map.
#include <cuda_runtime.h>

#include "pt_internal.h"

namespace hpt {

namespace {

__device__ __forceinline__ uint32_t find_prim(const PrimUpload* prims, uint32_t nprims, uint32_t idx, bool by_tri) {
  uint32_t lo = 0, hi = nprims;  // last prim with base <= idx
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) / 2;
    uint32_t b = by_tri ? prims[mid].tbase : prims[mid].vbase;
    if (b <= idx) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Object-to-world transform of the positions (rows of the 3x4 matrix) and
// of normals/tangents by the inverse transpose, with the operation order of
// the oracle and without FMA contraction, so world positions are bit-exact.
__global__ void k_flatten_verts(const float* raw, const PrimUpload* prims, uint32_t nprims, uint32_t nverts,
                                float4* vnorm, float4* vtan, float2* vuv, float4* wpos) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nverts) return;
  const PrimUpload& P = prims[find_prim(prims, nprims, v, false)];
  const float* q = raw + 11 * (size_t)v;
  float x = q[0], y = q[1], z = q[2];
  const float* T = P.xf;
  float px = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[0], x), __fmul_rn(T[1], y)), __fmul_rn(T[2], z)), T[3]);
  float py = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[4], x), __fmul_rn(T[5], y)), __fmul_rn(T[6], z)), T[7]);
  float pz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[8], x), __fmul_rn(T[9], y)), __fmul_rn(T[10], z)), T[11]);
  wpos[v] = make_float4(px, py, pz, 0.0f);
  const float* N = P.nm;
  auto xd = [&](float a, float b, float c) {
    return make_float4(__fadd_rn(__fadd_rn(__fmul_rn(N[0], a), __fmul_rn(N[1], b)), __fmul_rn(N[2], c)),
                       __fadd_rn(__fadd_rn(__fmul_rn(N[3], a), __fmul_rn(N[4], b)), __fmul_rn(N[5], c)),
                       __fadd_rn(__fadd_rn(__fmul_rn(N[6], a), __fmul_rn(N[7], b)), __fmul_rn(N[8], c)), 0.0f);
  };
  vnorm[v] = xd(q[3], q[4], q[5]);
  vtan[v] = xd(q[6], q[7], q[8]);
  vuv[v] = make_float2(q[9], q[10]);
}

__global__ void k_flatten_tris(const uint32_t* raw_idx, const PrimUpload* prims, uint32_t nprims, uint32_t ntris,
                               const float4* wpos, float4* tv0, float4* te1, float4* te2, uint32_t* tvidx,
                               uint32_t* tmat) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntris) return;
  const PrimUpload& P = prims[find_prim(prims, nprims, t, true)];
  uint32_t a = P.vbase + raw_idx[3 * (size_t)t], b = P.vbase + raw_idx[3 * (size_t)t + 1],
           c = P.vbase + raw_idx[3 * (size_t)t + 2];
  float4 pa = wpos[a], pb = wpos[b], pc = wpos[c];
  tv0[t] = pa;
  te1[t] = make_float4(__fsub_rn(pb.x, pa.x), __fsub_rn(pb.y, pa.y), __fsub_rn(pb.z, pa.z), 0.0f);
  te2[t] = make_float4(__fsub_rn(pc.x, pa.x), __fsub_rn(pc.y, pa.y), __fsub_rn(pc.z, pa.z), 0.0f);
  tvidx[3 * (size_t)t] = a;
  tvidx[3 * (size_t)t + 1] = b;
  tvidx[3 * (size_t)t + 2] = c;
  tmat[t] = P.material;
}

// BT.709 luminance in FP64, rounded like the oracle (no contraction).
__device__ __forceinline__ double lum64(float4 p) {
  double l = __dadd_rn(__dadd_rn(__dmul_rn(0.212671, (double)p.x), __dmul_rn(0.715160, (double)p.y)),
                       __dmul_rn(0.072169, (double)p.z));
  return (l > 0.0) ? l : 0.0;
}

// Vose's alias method, sequential in one thread; small/large lists are stacks.
__device__ void vose(const double* w, uint32_t n, double* q, uint32_t* small, uint32_t* large, uint2* out) {
  double total = 0.0;
  for (uint32_t i = 0; i < n; ++i) total = __dadd_rn(total, w[i]);
  if (!(total > 0.0)) {
    for (uint32_t i = 0; i < n; ++i) out[i] = make_uint2(__float_as_uint(1.0f), i);
    return;
  }
  uint32_t ns = 0, nl = 0;
  for (uint32_t i = 0; i < n; ++i) {
    q[i] = __ddiv_rn(__dmul_rn(w[i], (double)n), total);
    if (q[i] < 1.0) small[ns++] = i;
    else large[nl++] = i;
  }
  while (ns > 0 && nl > 0) {
    uint32_t s = small[--ns];
    uint32_t l = large[--nl];
    out[s] = make_uint2(__float_as_uint((float)q[s]), l);
    q[l] = __dsub_rn(__dadd_rn(q[l], q[s]), 1.0);
    if (q[l] < 1.0) small[ns++] = l;
    else large[nl++] = l;
  }
  while (nl > 0) { uint32_t l = large[--nl]; out[l] = make_uint2(__float_as_uint(1.0f), l); }
  while (ns > 0) { uint32_t s = small[--ns]; out[s] = make_uint2(__float_as_uint(1.0f), s); }
}

// One thread per row: texel weights, the row sum, and the row's alias table.
__global__ void k_env_rows(const float4* env, uint32_t w, uint32_t h, double* weights, double* q, uint32_t* stacks,
                           double* row_sums, uint2* cols) {
  uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= h) return;
  double* wr = weights + (size_t)y * w;
  double rs = 0.0;
  for (uint32_t x = 0; x < w; ++x) {
    double l = lum64(env[(size_t)y * w + x]);
    wr[x] = l;
    rs = __dadd_rn(rs, l);
  }
  row_sums[y] = rs;
  vose(wr, w, q + (size_t)y * w, stacks + (size_t)y * 2 * w, stacks + (size_t)y * 2 * w + w, cols + (size_t)y * w);
}

// Single thread: marginal alias table over the row sums and the total.
__global__ void k_env_marginal(const double* row_sums, uint32_t h, double* q, uint32_t* stacks, uint2* rows,
                               double* total_out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double total = 0.0;
  for (uint32_t y = 0; y < h; ++y) total = __dadd_rn(total, row_sums[y]);
  *total_out = total;
  vose(row_sums, h, q, stacks, stacks + h, rows);
}

}  // namespace

void launch_flatten(const float* raw_verts, const uint32_t* raw_idx, const PrimUpload* prims, uint32_t nprims,
                    uint32_t total_verts, uint32_t total_tris, const uint32_t*, const uint32_t*, float4* vnorm,
                    float4* vtan, float2* vuv, float4* wpos, float4* tri_v0, float4* tri_e1, float4* tri_e2,
                    uint32_t* tri_vidx, uint32_t* tri_mat, cudaStream_t st) {
  if (total_verts)
    k_flatten_verts<<<(total_verts + 255) / 256, 256, 0, st>>>(raw_verts, prims, nprims, total_verts, vnorm, vtan,
                                                                vuv, wpos);
  if (total_tris)
    k_flatten_tris<<<(total_tris + 255) / 256, 256, 0, st>>>(raw_idx, prims, nprims, total_tris, wpos, tri_v0,
                                                              tri_e1, tri_e2, tri_vidx, tri_mat);
}

void launch_env_tables(const float4* env, uint32_t w, uint32_t h, uint2* rows, uint2* cols, double* scratch_q,
                       uint32_t* scratch_stack, double* row_sums, double* total_out, cudaStream_t st) {
  // scratch_q holds w*h weights followed by w*h working q values
  double* weights = scratch_q;
  double* q = scratch_q + (size_t)w * h;
  k_env_rows<<<(h + 63) / 64, 64, 0, st>>>(env, w, h, weights, q, scratch_stack, row_sums, cols);
  k_env_marginal<<<1, 1, 0, st>>>(row_sums, h, q, scratch_stack, rows, total_out);
}

}  // namespace hpt
