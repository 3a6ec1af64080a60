// pt_scene.cu -- scene preparation kernels: world-space flattening of the
// mesh primitives and the FP64 alias tables of the environment map.
#include <cuda_runtime.h>

#include <algorithm>

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
                               const float4* wpos, const float4* vnorm, const float4* vtan, float4* tv0, float4* te1,
                               float4* te2, uint32_t* tvidx, uint32_t* tmat, float4* tshade) {
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
  float4* r = tshade + 6 * (size_t)t;
  const float4 n0 = vnorm[a];
  r[0] = make_float4(n0.x, n0.y, n0.z, __uint_as_float(P.material));
  r[1] = vnorm[b];
  r[2] = vnorm[c];
  r[3] = vtan[a];
  r[4] = vtan[b];
  r[5] = vtan[c];
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

// The same tables with one warp per row and the row in shared memory: lane 0
// performs every order-dependent step (the sums and Vose's pairing loop) in
// the order the sequential version does, the warp does the per-element steps
// (luminance, q = w * n / total, the stable split into the small and large
// lists, the final writes), so the tables are bit-identical and the
// sequential part runs at shared-memory instead of L2 latency.
__device__ void vose_warp(double* q, uint32_t n, double total, uint32_t* small, uint32_t* large, uint2* out) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u;
  if (!(total > 0.0)) {
    for (uint32_t i = lane; i < n; i += 32) out[i] = make_uint2(__float_as_uint(1.0f), i);
    return;
  }
  const unsigned lt = (1u << lane) - 1u;
  uint32_t ns = 0, nl = 0;
  for (uint32_t base = 0; base < n; base += 32) {
    const uint32_t i = base + lane;
    const bool v = i < n;
    bool sm = false;
    if (v) {
      const double qi = __ddiv_rn(__dmul_rn(q[i], (double)n), total);
      q[i] = qi;
      sm = qi < 1.0;
    }
    const unsigned ms = __ballot_sync(FULL, v && sm), ml = __ballot_sync(FULL, v && !sm);
    if (v) {
      if (sm) small[ns + __popc(ms & lt)] = i;
      else large[nl + __popc(ml & lt)] = i;
    }
    ns += __popc(ms);
    nl += __popc(ml);
  }
  __syncwarp();
  if (lane == 0) {
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
  __syncwarp();
}

// Shared memory of a row of n texels: q (n doubles), then the two stacks.
__host__ __device__ inline size_t vose_smem(uint32_t n) { return (size_t)n * (sizeof(double) + 2 * sizeof(uint32_t)); }

__global__ void __launch_bounds__(32) k_env_rows_warp(const float4* env, uint32_t w, double* row_sums, uint2* cols) {
  extern __shared__ double sq[];
  uint32_t* small = reinterpret_cast<uint32_t*>(sq + w);
  uint32_t* large = small + w;
  const uint32_t y = blockIdx.x, lane = threadIdx.x;
  for (uint32_t x = lane; x < w; x += 32) sq[x] = lum64(env[(size_t)y * w + x]);
  __syncwarp();
  double rs = 0.0;
  if (lane == 0) {
    for (uint32_t x = 0; x < w; ++x) rs = __dadd_rn(rs, sq[x]);
    row_sums[y] = rs;
  }
  rs = __shfl_sync(0xffffffffu, rs, 0);
  vose_warp(sq, w, rs, small, large, cols + (size_t)y * w);
}

__global__ void __launch_bounds__(32) k_env_marginal_warp(const double* row_sums, uint32_t h, uint2* rows,
                                                          double* total_out) {
  extern __shared__ double sq[];
  uint32_t* small = reinterpret_cast<uint32_t*>(sq + h);
  uint32_t* large = small + h;
  const uint32_t lane = threadIdx.x;
  for (uint32_t y = lane; y < h; y += 32) sq[y] = row_sums[y];
  __syncwarp();
  double total = 0.0;
  if (lane == 0) {
    for (uint32_t y = 0; y < h; ++y) total = __dadd_rn(total, sq[y]);
    *total_out = total;
  }
  total = __shfl_sync(0xffffffffu, total, 0);
  vose_warp(sq, h, total, small, large, rows);
}

}  // namespace

void launch_flatten(const float* raw_verts, const uint32_t* raw_idx, const PrimUpload* prims, uint32_t nprims,
                    uint32_t total_verts, uint32_t total_tris, const uint32_t*, const uint32_t*, float4* vnorm,
                    float4* vtan, float2* vuv, float4* wpos, float4* tri_v0, float4* tri_e1, float4* tri_e2,
                    uint32_t* tri_vidx, uint32_t* tri_mat, float4* tri_shade, cudaStream_t st) {
  if (total_verts)
    k_flatten_verts<<<(total_verts + 255) / 256, 256, 0, st>>>(raw_verts, prims, nprims, total_verts, vnorm, vtan,
                                                                vuv, wpos);
  if (total_tris)
    k_flatten_tris<<<(total_tris + 255) / 256, 256, 0, st>>>(raw_idx, prims, nprims, total_tris, wpos, vnorm, vtan,
                                                              tri_v0, tri_e1, tri_e2, tri_vidx, tri_mat, tri_shade);
}

__global__ void k_env_widen(const float* __restrict__ rgb, float4* __restrict__ env, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    env[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
}

void launch_env_widen(const float* rgb, float4* env, size_t n, cudaStream_t st) {
  const size_t blocks = std::min<size_t>((n + 255) / 256, 65535);
  k_env_widen<<<(unsigned)std::max<size_t>(blocks, 1), 256, 0, st>>>(rgb, env, n);
}

void launch_env_tables(const float4* env, uint32_t w, uint32_t h, uint2* rows, uint2* cols, double* scratch_q,
                       uint32_t* scratch_stack, double* row_sums, double* total_out, cudaStream_t st) {
  // scratch_q holds w*h weights followed by w*h working q values
  double* weights = scratch_q;
  double* q = scratch_q + (size_t)w * h;
  int dev = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t row_smem = vose_smem(w), marg_smem = vose_smem(h);
  if (row_smem <= (size_t)smem_max &&
      cudaFuncSetAttribute(k_env_rows_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem) ==
          cudaSuccess) {
    k_env_rows_warp<<<h, 32, row_smem, st>>>(env, w, row_sums, cols);
  } else {
    cudaGetLastError();
    k_env_rows<<<(h + 63) / 64, 64, 0, st>>>(env, w, h, weights, q, scratch_stack, row_sums, cols);
  }
  if (marg_smem <= (size_t)smem_max &&
      cudaFuncSetAttribute(k_env_marginal_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)marg_smem) ==
          cudaSuccess) {
    k_env_marginal_warp<<<1, 32, marg_smem, st>>>(row_sums, h, rows, total_out);
  } else {
    cudaGetLastError();
    k_env_marginal<<<1, 1, 0, st>>>(row_sums, h, q, scratch_stack, rows, total_out);
  }
}

}  // namespace hpt
