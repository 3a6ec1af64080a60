// pt_cache.cu -- online radiance cache: multiresolution hash-grid encoding
// (16 levels x 2 fp16 features) feeding a 64-wide MLP with 5 hidden ReLU
// layers, BF16 weights and activations, FP32 accumulation on the tensor
// cores (mma.sync m16n8k16), trained with Adam.
//
// Kernels
//   k_cache_infer     encode + forward, one warp per 16 records; the
//                     activations never leave registers: the accumulator
//                     fragment of two adjacent 8-column tiles is the operand
//                     fragment of the next layer's 16-wide k slice.
//   k_cache_train_fb  forward as above keeping every layer's input fragments,
//                     relative-L2 loss, backward through the layers
//                     (dX = dZ W^T on the tensor cores, ReLU masks from the
//                     kept fragments), scatter of the encoding gradient into
//                     the hash table (fp32 float2 atomics); stores each
//                     layer's input X and output gradient dZ (bf16) for:
//   k_cache_dw        dW = X^T dZ per layer, one partial per block
//                     (deterministic, no atomics), on the tensor cores;
//   k_cache_adam_mlp  sums the partials in a fixed order, Adam on the FP32
//                     master weights, re-quantises both BF16 weight layouts;
//   k_cache_adam_grid Adam on the hash-table entries that received gradient.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pt_cache.h"
#include "pt_impl.h"

namespace hpt {
namespace {

constexpr int WSTRIDE = 72;   // smem row stride (bf16) of 64-wide rows: conflict-free fragment loads
constexpr int WSTRIDE5 = 24;  // smem row stride of the 16-wide backward rows of the output layer
constexpr int SMEM_WN = 5 * 64 * WSTRIDE + NC_OUT * WSTRIDE;   // forward weights (bf16 elements)
constexpr int SMEM_WK = 5 * 64 * WSTRIDE + 64 * WSTRIDE5;      // backward weights
constexpr int TILE = 16 * WSTRIDE;                               // one warp's 16-row staging tile
constexpr int CACHE_WARPS = 4;  // training kernels (255 registers per thread)
constexpr int INFER_WARPS = 8;  // more warps hide the latency of the hash-table gathers
constexpr uint32_t HASH_P1 = 2654435761u, HASH_P2 = 805459861u;

__device__ __forceinline__ int wn_smem_off(int l) { return l * 64 * WSTRIDE; }
__device__ __forceinline__ int wk_smem_off(int l) { return l * 64 * WSTRIDE; }

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_u16(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ bool bf16_positive(uint32_t word, int half) {
  uint32_t b = (word >> (16 * half)) & 0xFFFFu;
  return b != 0u && (b & 0x8000u) == 0u;
}

// Trilinear corners of one level: global table index and weight.
// (`N` = V.res[l], passed in so that V.res is only indexed by constants and
// the view stays in the parameter bank.)
__device__ __forceinline__ void level_corners(const CacheView& V, int l, uint32_t N, float px, float py, float pz,
                                              uint32_t (&idx)[8], float (&w)[8]) {
  const uint32_t T = 1u << V.log2_table;
  float x = px * (float)N, y = py * (float)N, z = pz * (float)N;
  uint32_t x0 = min((uint32_t)x, N - 1u), y0 = min((uint32_t)y, N - 1u), z0 = min((uint32_t)z, N - 1u);
  float fx = x - (float)x0, fy = y - (float)y0, fz = z - (float)z0;
  const uint64_t side = (uint64_t)N + 1u;
  const bool dense = side * side * side <= (uint64_t)T;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    uint32_t cx = x0 + (c & 1), cy = y0 + ((c >> 1) & 1), cz = z0 + (c >> 2);
    uint32_t i = dense ? (uint32_t)(cx + side * (cy + side * cz)) : ((cx ^ (cy * HASH_P1) ^ (cz * HASH_P2)) & (T - 1u));
    idx[c] = (uint32_t)l * T + i;
    w[c] = ((c & 1) ? fx : 1.0f - fx) * ((c & 2) ? fy : 1.0f - fy) * ((c & 4) ? fz : 1.0f - fz);
  }
}

__device__ __forceinline__ void unit_position(const CacheView& V, float4 r0, float& px, float& py, float& pz) {
  px = fminf(fmaxf((r0.x - V.lo[0]) * V.inv_ext[0], 0.0f), 1.0f);
  py = fminf(fmaxf((r0.y - V.lo[1]) * V.inv_ext[1], 0.0f), 1.0f);
  pz = fminf(fmaxf((r0.z - V.lo[2]) * V.inv_ext[2], 0.0f), 1.0f);
}

// Fills one row of the staging tile: lanes 0-15 encode levels 0-7 and the raw
// inputs, lanes 16-31 levels 8-15 and the zero padding.
__device__ __forceinline__ void encode_row(const CacheView& V, const float4* rec, bool valid, int half,
                                          __nv_bfloat16* row) {
  float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0, r3 = r0;
  if (valid) {
    r0 = rec[0];
    r1 = rec[1];
    r2 = rec[2];
    r3 = rec[3];
  }
  float px, py, pz;
  unit_position(V, r0, px, py, pz);
  uint32_t* w32 = reinterpret_cast<uint32_t*>(row);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int l = half * 8 + k;
    const uint32_t N = half ? V.res[8 + k] : V.res[k];
    uint32_t idx[8];
    float w[8];
    level_corners(V, l, N, px, py, pz, idx, w);
    float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float2 v = __half22float2(V.grid[idx[c]]);
      f0 += w[c] * v.x;
      f1 += w[c] * v.y;
    }
    w32[l] = pack_bf16(f0, f1);  // columns 2l, 2l+1
  }
  if (half == 0) {
    // columns 32..47: direction, normal (mapped to [0,1]), colour, roughness,
    // metallic, transmission, constant 1, zeros
    float v[16] = {r0.w * 0.5f + 0.5f, r1.x * 0.5f + 0.5f, r1.y * 0.5f + 0.5f,
                   r1.z * 0.5f + 0.5f, r1.w * 0.5f + 0.5f, r2.x * 0.5f + 0.5f,
                   r2.y, r2.z, r2.w, r3.x, r3.y, r3.z, 1.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 8; ++k) w32[16 + k] = pack_bf16(v[2 * k], v[2 * k + 1]);
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) w32[24 + k] = 0u;
  }
}

// Forward of one layer: acc (16 x 8*NT) = A (16 x 64) x W^T, W in smem as
// [n][k] rows of stride WSTRIDE.
template <int NT>
__device__ __forceinline__ void layer_fwd(const uint32_t (&a)[4][4], const __nv_bfloat16* W, float (&acc)[NT][4],
                                          int g, int t) {
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const uint32_t* row = reinterpret_cast<const uint32_t*>(W + (8 * nt + g) * WSTRIDE);
      mma16816(acc[nt], a[s], row[8 * s + t], row[8 * s + 4 + t]);
    }
  }
}

// Accumulator fragments of 8 n-tiles -> operand fragments of 4 k-slices.
__device__ __forceinline__ void c_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4], bool relu) {
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    float v[8];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      v[e] = acc[2 * s][e];
      v[4 + e] = acc[2 * s + 1][e];
    }
    if (relu) {
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = fmaxf(v[e], 0.0f);
    }
    a[s][0] = pack_bf16(v[0], v[1]);  // row g,   k 16s+2t
    a[s][1] = pack_bf16(v[2], v[3]);  // row g+8, k 16s+2t
    a[s][2] = pack_bf16(v[4], v[5]);  // row g,   k 16s+8+2t
    a[s][3] = pack_bf16(v[6], v[7]);  // row g+8, k 16s+8+2t
  }
}

__device__ __forceinline__ void load_a_from_tile(const __nv_bfloat16* X, uint32_t (&a)[4][4], int g, int t) {
  const uint32_t* r0 = reinterpret_cast<const uint32_t*>(X + g * WSTRIDE);
  const uint32_t* r8 = reinterpret_cast<const uint32_t*>(X + (g + 8) * WSTRIDE);
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    a[s][0] = r0[8 * s + t];
    a[s][1] = r8[8 * s + t];
    a[s][2] = r0[8 * s + 4 + t];
    a[s][3] = r8[8 * s + 4 + t];
  }
}

// Copies the compact global weights into padded smem rows.
__device__ void load_wn(const CacheView& V, __nv_bfloat16* sm) {
  for (int i = threadIdx.x; i < NC_PARAMS / 2; i += blockDim.x) {
    int e = 2 * i;
    int l = e / 4096, loc = e - l * 4096;
    if (l >= NC_LAYERS) break;
    int n = loc / 64, k = loc - n * 64;
    *reinterpret_cast<uint32_t*>(sm + wn_smem_off(l) + n * WSTRIDE + k) =
        *reinterpret_cast<const uint32_t*>(V.wn + e);
  }
}
__device__ void load_wk(const CacheView& V, __nv_bfloat16* sm) {
  for (int i = threadIdx.x; i < NC_PARAMS / 2; i += blockDim.x) {
    int e = 2 * i;
    int l = e / 4096, loc = e - l * 4096;
    if (l >= NC_LAYERS) break;
    const int N = nc_layer_n(l);
    const int stride = l == NC_LAYERS - 1 ? WSTRIDE5 : WSTRIDE;
    int k = loc / N, n = loc - k * N;
    *reinterpret_cast<uint32_t*>(sm + wk_smem_off(l) + k * stride + n) =
        *reinterpret_cast<const uint32_t*>(V.wk + e);
  }
}

// Forward through all layers; returns the output fragments (2 n-tiles).
// With `keep`, the operand fragments of the inputs of layers 1..5 are kept
// (for the ReLU masks) and every layer input is stored to X (row-major bf16,
// 64 columns per layer, rows >= n skipped).
template <bool KEEP>
__device__ __forceinline__ void mlp_forward(const __nv_bfloat16* wn_sm, uint32_t (&a)[4][4], float (&out)[2][4],
                                            uint32_t (*keep)[4][4], __nv_bfloat16* X, size_t layer_stride,
                                            uint32_t row0, uint32_t n, int g, int t) {
  float acc[8][4];
#pragma unroll
  for (int l = 0; l < NC_LAYERS - 1; ++l) {
    if (KEEP) {
      __nv_bfloat16* Xl = X + l * layer_stride;
      uint32_t ra = row0 + g, rb = row0 + g + 8;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        if (ra < n) {
          uint32_t* w = reinterpret_cast<uint32_t*>(Xl + (size_t)ra * 64);
          w[8 * s + t] = a[s][0];
          w[8 * s + 4 + t] = a[s][2];
        }
        if (rb < n) {
          uint32_t* w = reinterpret_cast<uint32_t*>(Xl + (size_t)rb * 64);
          w[8 * s + t] = a[s][1];
          w[8 * s + 4 + t] = a[s][3];
        }
      }
    }
    layer_fwd<8>(a, wn_sm + wn_smem_off(l), acc, g, t);
    c_to_a(acc, a, true);
    if (KEEP) {
#pragma unroll
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int r = 0; r < 4; ++r) keep[l][s][r] = a[s][r];
    }
  }
  if (KEEP) {
    __nv_bfloat16* Xl = X + (NC_LAYERS - 1) * layer_stride;
    uint32_t ra = row0 + g, rb = row0 + g + 8;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (ra < n) {
        uint32_t* w = reinterpret_cast<uint32_t*>(Xl + (size_t)ra * 64);
        w[8 * s + t] = a[s][0];
        w[8 * s + 4 + t] = a[s][2];
      }
      if (rb < n) {
        uint32_t* w = reinterpret_cast<uint32_t*>(Xl + (size_t)rb * 64);
        w[8 * s + t] = a[s][1];
        w[8 * s + 4 + t] = a[s][3];
      }
    }
  }
  layer_fwd<2>(a, wn_sm + wn_smem_off(NC_LAYERS - 1), out, g, t);
}

__global__ void __launch_bounds__(INFER_WARPS * 32) k_cache_infer(CacheView V, const float4* rec, const uint32_t* idx,
                                                                 const uint32_t* count_dev, uint32_t n_max,
                                                                 float4* out, const float4* scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* wn_sm = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  __nv_bfloat16* tiles = wn_sm + SMEM_WN;
  const uint32_t n = count_dev ? min(*count_dev, n_max) : n_max;
  if ((uint32_t)blockIdx.x * INFER_WARPS * 16 >= n) return;
  load_wn(V, wn_sm);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  __nv_bfloat16* X = tiles + warp * TILE;
  for (uint32_t tile = blockIdx.x * INFER_WARPS + warp; tile * 16 < n; tile += gridDim.x * INFER_WARPS) {
    const uint32_t row0 = tile * 16;
    {
      uint32_t r = row0 + (lane & 15);
      bool valid = r < n;
      uint32_t slot = valid ? (idx ? idx[r] : r) : 0u;
      encode_row(V, rec + (size_t)slot * 4, valid, lane >> 4, X + (lane & 15) * WSTRIDE);
    }
    __syncwarp();
    uint32_t a[4][4];
    load_a_from_tile(X, a, g, t);
    float o[2][4];
    mlp_forward<false>(wn_sm, a, o, nullptr, nullptr, 0, row0, n, g, t);
    // rgb of row g: columns 0,1 (lane t=0) and 2 (lane t=1)
    float c2a = __shfl_down_sync(0xFFFFFFFFu, o[0][0], 1);
    float c2b = __shfl_down_sync(0xFFFFFFFFu, o[0][2], 1);
    if (t == 0) {
      uint32_t ra = row0 + g, rb = row0 + g + 8;
      float3 pa = make_float3(o[0][0], o[0][1], c2a), pb = make_float3(o[0][2], o[0][3], c2b);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t r = h ? rb : ra;
        float3 pr = h ? pb : pa;
        if (r >= n) continue;
        uint32_t slot = idx ? idx[r] : r;
        if (scale) {
          float4 s4 = scale[slot];
          float4 o4 = out[slot];
          o4.x += s4.x * fmaxf(pr.x, 0.0f);
          o4.y += s4.y * fmaxf(pr.y, 0.0f);
          o4.z += s4.z * fmaxf(pr.z, 0.0f);
          out[slot] = o4;
        } else {
          out[slot] = make_float4(pr.x, pr.y, pr.z, 0.0f);
        }
      }
    }
    __syncwarp();
  }
}

// Forward + loss + backward-data for one batch. X/D: per-layer row-major
// bf16 inputs and output gradients, `cap` rows per layer.
__global__ void __launch_bounds__(CACHE_WARPS * 32) k_cache_train_fb(CacheView V, const float4* rec,
                                                                    const float4* tgt, uint32_t n, float inv_n,
                                                                    __nv_bfloat16* X, __nv_bfloat16* D, size_t cap,
                                                                    float* loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* wn_sm = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  __nv_bfloat16* wk_sm = wn_sm + SMEM_WN;
  __nv_bfloat16* tiles = wk_sm + SMEM_WK;
  if ((uint32_t)blockIdx.x * CACHE_WARPS * 16 >= n) return;
  load_wn(V, wn_sm);
  load_wk(V, wk_sm);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  __nv_bfloat16* Xt = tiles + warp * TILE;
  const size_t ls = cap * 64;  // layer stride of X and D
  float lsum = 0.0f;
  for (uint32_t tile = blockIdx.x * CACHE_WARPS + warp; tile * 16 < n; tile += gridDim.x * CACHE_WARPS) {
    const uint32_t row0 = tile * 16;
    {
      uint32_t r = row0 + (lane & 15);
      encode_row(V, rec + (size_t)(r < n ? r : 0u) * 4, r < n, lane >> 4, Xt + (lane & 15) * WSTRIDE);
    }
    __syncwarp();
    uint32_t a[4][4];
    load_a_from_tile(Xt, a, g, t);
    uint32_t keep[NC_LAYERS - 1][4][4];
    float o[2][4];
    mlp_forward<true>(wn_sm, a, o, keep, X, ls, row0, n, g, t);

    // relative L2 loss, d/dpred = 2 (pred - y) / (pred^2 + 0.01)
    const uint32_t ra = row0 + g, rb = row0 + g + 8;
    float4 ya = ra < n ? tgt[ra] : make_float4(0, 0, 0, 0);
    float4 yb = rb < n ? tgt[rb] : make_float4(0, 0, 0, 0);
    float dz5[2][4];
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int col = 8 * nt + 2 * t + (e & 1);
        const uint32_t r = e < 2 ? ra : rb;
        const float4 y4 = e < 2 ? ya : yb;
        float d = 0.0f;
        if (r < n && col < 3) {
          float y = col == 0 ? y4.x : (col == 1 ? y4.y : y4.z);
          float p = o[nt][e];
          float den = p * p + 0.01f;
          float diff = p - y;
          lsum += diff * diff / den;
          d = 2.0f * diff / den * inv_n;
        }
        dz5[nt][e] = d;
      }
    uint32_t ad[4];  // dZ5 as one 16-wide k slice
    ad[0] = pack_bf16(dz5[0][0], dz5[0][1]);
    ad[1] = pack_bf16(dz5[0][2], dz5[0][3]);
    ad[2] = pack_bf16(dz5[1][0], dz5[1][1]);
    ad[3] = pack_bf16(dz5[1][2], dz5[1][3]);
    {
      __nv_bfloat16* D5 = D + (NC_LAYERS - 1) * ls;
      if (ra < n) {
        uint32_t* w = reinterpret_cast<uint32_t*>(D5 + (size_t)ra * NC_OUT);
        w[t] = ad[0];
        w[4 + t] = ad[2];
      }
      if (rb < n) {
        uint32_t* w = reinterpret_cast<uint32_t*>(D5 + (size_t)rb * NC_OUT);
        w[t] = ad[1];
        w[4 + t] = ad[3];
      }
    }
    // dX5 = dZ5 W5^T (K = 16)
    float acc[8][4];
    {
      const __nv_bfloat16* W = wk_sm + wk_smem_off(NC_LAYERS - 1);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
        const uint32_t* row = reinterpret_cast<const uint32_t*>(W + (8 * nt + g) * WSTRIDE5);
        mma16816(acc[nt], ad, row[t], row[4 + t]);
      }
    }
    uint32_t da[4][4];
#pragma unroll
    for (int l = NC_LAYERS - 2; l >= 0; --l) {
      // dZ_l = dX_{l+1} * [X_{l+1} > 0]; X_{l+1} fragments are keep[l]
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int s = nt >> 1, reg = ((nt & 1) ? 2 : 0) + (e >> 1);
          if (!bf16_positive(keep[l][s][reg], e & 1)) acc[nt][e] = 0.0f;
        }
      c_to_a(acc, da, false);
      {
        __nv_bfloat16* Dl = D + l * ls;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          if (ra < n) {
            uint32_t* w = reinterpret_cast<uint32_t*>(Dl + (size_t)ra * 64);
            w[8 * s + t] = da[s][0];
            w[8 * s + 4 + t] = da[s][2];
          }
          if (rb < n) {
            uint32_t* w = reinterpret_cast<uint32_t*>(Dl + (size_t)rb * 64);
            w[8 * s + t] = da[s][1];
            w[8 * s + 4 + t] = da[s][3];
          }
        }
      }
      // dX_l = dZ_l W_l^T; for l = 0 only the 32 encoded columns are needed
      const __nv_bfloat16* W = wk_sm + wk_smem_off(l);
      const int NTo = l == 0 ? 4 : 8;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          if (nt >= NTo) continue;
          const uint32_t* row = reinterpret_cast<const uint32_t*>(W + (8 * nt + g) * WSTRIDE);
          mma16816(acc[nt], da[s], row[8 * s + t], row[8 * s + 4 + t]);
        }
    }
    // encoding gradient: lane holds levels 4nt+t (nt 0..3) for rows g, g+8
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t r = h ? rb : ra;
      if (r >= n) continue;
      float px, py, pz;
      unit_position(V, rec[(size_t)r * 4], px, py, pz);
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int l = 4 * nt + t;
        const uint32_t N = t == 0 ? V.res[4 * nt] : t == 1 ? V.res[4 * nt + 1] : t == 2 ? V.res[4 * nt + 2]
                                                                                       : V.res[4 * nt + 3];
        const float d0 = acc[nt][2 * h], d1 = acc[nt][2 * h + 1];
        if (d0 == 0.0f && d1 == 0.0f) continue;
        uint32_t idx[8];
        float w[8];
        level_corners(V, l, N, px, py, pz, idx, w);
#pragma unroll
        for (int c = 0; c < 8; ++c) atomicAdd(&V.grid_grad[idx[c]], make_float2(w[c] * d0, w[c] * d1));
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, off);
  if (lane == 0 && lsum != 0.0f) atomicAdd(loss, lsum * inv_n);
}

// dW_l partial over rows [blockIdx.x * rows_per_block, ...): warp w owns the
// 16 input features 16w..16w+15 and all output columns.
constexpr int DW_CHUNK = 64;
__global__ void __launch_bounds__(CACHE_WARPS * 32) k_cache_dw(const __nv_bfloat16* X, const __nv_bfloat16* D,
                                                              size_t cap, uint32_t n, uint32_t rows_per_block,
                                                              float* partials, uint32_t nblocks) {
  __shared__ __align__(16) uint16_t xs[DW_CHUNK * WSTRIDE];
  __shared__ __align__(16) uint16_t ds[DW_CHUNK * WSTRIDE];
  const int l = blockIdx.y;
  const int N = nc_layer_n(l);
  const int NT = N / 8;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const __nv_bfloat16* Xl = X + (size_t)l * cap * 64;
  const __nv_bfloat16* Dl = D + (size_t)l * cap * 64;
  const uint32_t r_begin = blockIdx.x * rows_per_block;
  const uint32_t r_end = min(n, r_begin + rows_per_block);
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
  for (uint32_t c0 = r_begin; c0 < r_end; c0 += DW_CHUNK) {
    __syncthreads();
    for (int i = threadIdx.x; i < DW_CHUNK * 32; i += blockDim.x) {
      int r = i >> 5, w = i & 31;
      uint32_t gr = c0 + r;
      uint32_t v = gr < r_end ? reinterpret_cast<const uint32_t*>(Xl + (size_t)gr * 64)[w] : 0u;
      reinterpret_cast<uint32_t*>(xs + r * WSTRIDE)[w] = v;
    }
    const int wpr = N / 2;  // words per gradient row
    for (int i = threadIdx.x; i < DW_CHUNK * wpr; i += blockDim.x) {
      int r = i / wpr, w = i - r * wpr;
      uint32_t gr = c0 + r;
      uint32_t v = gr < r_end ? reinterpret_cast<const uint32_t*>(Dl + (size_t)gr * N)[w] : 0u;
      reinterpret_cast<uint32_t*>(ds + r * WSTRIDE)[w] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < DW_CHUNK / 16; ++kk) {
      const int r0 = 16 * kk;
      const int i0 = 16 * warp;
      uint32_t a[4];
      a[0] = pack_u16(xs[(r0 + 2 * t) * WSTRIDE + i0 + g], xs[(r0 + 2 * t + 1) * WSTRIDE + i0 + g]);
      a[1] = pack_u16(xs[(r0 + 2 * t) * WSTRIDE + i0 + g + 8], xs[(r0 + 2 * t + 1) * WSTRIDE + i0 + g + 8]);
      a[2] = pack_u16(xs[(r0 + 2 * t + 8) * WSTRIDE + i0 + g], xs[(r0 + 2 * t + 9) * WSTRIDE + i0 + g]);
      a[3] = pack_u16(xs[(r0 + 2 * t + 8) * WSTRIDE + i0 + g + 8], xs[(r0 + 2 * t + 9) * WSTRIDE + i0 + g + 8]);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        if (nt >= NT) continue;
        uint32_t b0 = pack_u16(ds[(r0 + 2 * t) * WSTRIDE + 8 * nt + g], ds[(r0 + 2 * t + 1) * WSTRIDE + 8 * nt + g]);
        uint32_t b1 =
            pack_u16(ds[(r0 + 2 * t + 8) * WSTRIDE + 8 * nt + g], ds[(r0 + 2 * t + 9) * WSTRIDE + 8 * nt + g]);
        mma16816(acc[nt], a, b0, b1);
      }
    }
  }
  // partial[l][block][k][n], k = input feature, n = output column
  float* P = partials + ((size_t)l * nblocks + blockIdx.x) * 4096;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    if (nt >= NT) continue;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      int k = 16 * warp + g + (e >= 2 ? 8 : 0);
      int col = 8 * nt + 2 * t + (e & 1);
      P[k * N + col] = acc[nt][e];
    }
  }
}

struct AdamArgs {
  float lr, b1, b2, eps, c1, c2;  // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
};

__device__ __forceinline__ float adam_step(float& w, float& m, float& v, float gr, const AdamArgs& A) {
  m = A.b1 * m + (1.0f - A.b1) * gr;
  v = A.b2 * v + (1.0f - A.b2) * gr * gr;
  float mh = m * A.c1, vh = v * A.c2;
  w -= A.lr * mh / (sqrtf(vh) + A.eps);
  return w;
}

// Sums the per-block partials (fixed order). With `grad_out` the sum is only
// written out (gradient check); otherwise Adam updates the weights.
__global__ void k_cache_adam_mlp(const float* partials, uint32_t nblocks, float* w, float* m, float* v,
                                 __nv_bfloat16* wn, __nv_bfloat16* wk, AdamArgs A, float* grad_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NC_PARAMS) return;
  const int l = p / 4096, loc = p - l * 4096;
  const int N = nc_layer_n(l);
  float gsum = 0.0f;
  for (uint32_t b = 0; b < nblocks; ++b) gsum += partials[((size_t)l * nblocks + b) * 4096 + loc];
  if (grad_out) {
    grad_out[p] = gsum;
    return;
  }
  float wi = w[p], mi = m[p], vi = v[p];
  adam_step(wi, mi, vi, gsum, A);
  w[p] = wi;
  m[p] = mi;
  v[p] = vi;
  const int k = loc / N, n = loc - k * N;
  wn[nc_layer_off(l) + n * 64 + k] = __float2bfloat16_rn(wi);
  wk[p] = __float2bfloat16_rn(wi);
}

__global__ void k_cache_adam_grid(float* grad, float* w, float* m, float* v, __half* wh, uint64_t count, AdamArgs A) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gr = grad[i];
  if (gr == 0.0f) return;
  float wi = w[i], mi = m[i], vi = v[i];
  adam_step(wi, mi, vi, gr, A);
  w[i] = wi;
  m[i] = mi;
  v[i] = vi;
  wh[i] = __float2half_rn(wi);
  grad[i] = 0.0f;
}

__global__ void k_cache_set_weights(const float* w, __nv_bfloat16* wn, __nv_bfloat16* wk) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NC_PARAMS) return;
  const int l = p / 4096, loc = p - l * 4096;
  const int N = nc_layer_n(l);
  const int k = loc / N, n = loc - k * N;
  wn[nc_layer_off(l) + n * 64 + k] = __float2bfloat16_rn(w[p]);
  wk[p] = __float2bfloat16_rn(w[p]);
}

__global__ void k_cache_set_grid(const float* w, __half* wh, uint64_t count) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) wh[i] = __float2half_rn(w[i]);
}

// splitmix64-based uniform initialisation (seeded, deterministic)
__host__ __device__ inline float init_uniform(uint64_t seed, uint64_t i) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f) * 2.0f - 1.0f;
}

__global__ void k_cache_init_grid(float* w, uint64_t count, uint64_t seed, float scale) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) w[i] = scale * init_uniform(seed, i);
}

// Seeded query records inside the unit box (for the device-timed benchmark).
__global__ void k_cache_bench_records(float4* rec, float4* tgt, uint32_t n, uint64_t seed) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float u[16];
  for (int k = 0; k < 16; ++k) u[k] = 0.5f + 0.5f * init_uniform(seed, 16ull * i + k);
  rec[4 * (size_t)i] = make_float4(u[0], u[1], u[2], u[3] * 2.0f - 1.0f);
  rec[4 * (size_t)i + 1] = make_float4(u[4] * 2.0f - 1.0f, u[5] * 2.0f - 1.0f, u[6] * 2.0f - 1.0f, u[7] * 2.0f - 1.0f);
  rec[4 * (size_t)i + 2] = make_float4(u[8] * 2.0f - 1.0f, u[9], u[10], u[11]);
  rec[4 * (size_t)i + 3] = make_float4(u[12], u[13], u[14], 0.0f);
  tgt[i] = make_float4(u[0] + u[9], u[1] + u[10], u[2] + u[11], 0.0f);
}

constexpr size_t SMEM_INFER = (size_t)(SMEM_WN + INFER_WARPS * TILE) * 2;
constexpr size_t SMEM_TRAIN = (size_t)(SMEM_WN + SMEM_WK + CACHE_WARPS * TILE) * 2;
constexpr uint32_t DW_ROWS_PER_BLOCK = 512;
constexpr uint32_t DW_TC_ROWS_PER_BLOCK = 1024;  // 16 chunks of 64 rows per tensor-core CTA

}  // namespace

void launch_cache_infer(const CacheView& V, const float4* rec, const uint32_t* idx, const uint32_t* count_dev,
                        uint32_t n_max, float4* out, const float4* scale, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_cache_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_INFER);
    attr = true;
  }
  if (n_max == 0) return;
  uint32_t tiles = (n_max + 15) / 16;
  uint32_t blocks = std::min<uint32_t>((tiles + INFER_WARPS - 1) / INFER_WARPS, (uint32_t)device_sm_count() * 2);
  k_cache_infer<<<blocks, INFER_WARPS * 32, SMEM_INFER, st>>>(V, rec, idx, count_dev, n_max, out, scale);
}

}  // namespace hpt

using namespace hpt;

struct pt_cache {
  pt_cache_config cfg{};
  std::string err;
  CacheView V{};
  uint64_t grid_count = 0;  // floats in the table (levels x entries x 2)
  Buf<float> w, wm, wv;
  Buf<__nv_bfloat16> wn, wk;
  Buf<float> gw, gm, gv, ggrad;
  Buf<__half> gh;
  Buf<__nv_bfloat16> X, D;
  size_t cap = 0;
  Buf<float> partials, loss, gradbuf;
  Buf<float4> rec, tgt;
  Buf<uint32_t> tc_err;            // wait-limit flag of the tensor-core kernel
  uint32_t* tc_err_host = nullptr;  // pinned copy, refreshed after every training pass
  uint32_t step = 0;
  float last_loss = 0.0f;
  cudaStream_t stream = nullptr;
};

namespace hpt {

CacheView cache_view(const pt_cache* c) { return c->V; }

cudaError_t cache_last_loss(pt_cache* c, float* loss) {
  return cudaMemcpy(loss, c->loss.p, sizeof(float), cudaMemcpyDeviceToHost);
}

static cudaError_t ensure_train(pt_cache* c, size_t rows) {
  if (rows <= c->cap && c->X.p) return cudaSuccess;
  size_t cap = std::max<size_t>(rows, 1024);
  cudaError_t e;
  if ((e = c->X.ensure(cap * 64 * NC_LAYERS)) != cudaSuccess) return e;
  if ((e = c->D.ensure(cap * 64 * NC_LAYERS)) != cudaSuccess) return e;
  const size_t nb = (cap + DW_ROWS_PER_BLOCK - 1) / DW_ROWS_PER_BLOCK;
  if ((e = c->partials.ensure(nb * NC_LAYERS * 4096)) != cudaSuccess) return e;
  c->cap = cap;
  return cudaSuccess;
}

// One forward/backward pass over rows [0, n) of rec/tgt; leaves the MLP
// gradient partials and the table gradient in place.
static cudaError_t forward_backward(pt_cache* c, const float4* rec, const float4* tgt, uint32_t n, cudaStream_t st,
                                    uint32_t* nblocks_out) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_cache_train_fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TRAIN);
    attr = true;
  }
  cudaError_t e;
  if ((e = ensure_train(c, n)) != cudaSuccess) return e;
  uint32_t tiles = (n + 15) / 16;
  uint32_t blocks = std::min<uint32_t>((tiles + CACHE_WARPS - 1) / CACHE_WARPS, (uint32_t)device_sm_count() * 2);
  k_cache_train_fb<<<blocks, CACHE_WARPS * 32, SMEM_TRAIN, st>>>(c->V, rec, tgt, n, 1.0f / (float)n, c->X.p, c->D.p,
                                                                 c->cap, c->loss.p);
  if (c->cfg.weight_grad_kernel == 0) {
    const uint32_t nb = (n + DW_TC_ROWS_PER_BLOCK - 1) / DW_TC_ROWS_PER_BLOCK;
    launch_cache_dw_tc(c->X.p, c->D.p, c->cap, n, DW_TC_ROWS_PER_BLOCK, c->partials.p, nb, c->tc_err.p, st);
    *nblocks_out = nb;
  } else {
    const uint32_t nb = (n + DW_ROWS_PER_BLOCK - 1) / DW_ROWS_PER_BLOCK;
    k_cache_dw<<<dim3(nb, NC_LAYERS), CACHE_WARPS * 32, 0, st>>>(c->X.p, c->D.p, c->cap, n, DW_ROWS_PER_BLOCK,
                                                                 c->partials.p, nb);
    *nblocks_out = nb;
  }
  return cudaGetLastError();
}

static AdamArgs adam_args(pt_cache* c) {
  AdamArgs A;
  A.lr = c->cfg.learning_rate;
  A.b1 = 0.9f;
  A.b2 = 0.99f;
  A.eps = 1e-15f;
  ++c->step;
  A.c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)c->step)));
  A.c2 = (float)(1.0 / (1.0 - std::pow(0.99, (double)c->step)));
  return A;
}

static cudaError_t train_step(pt_cache* c, const float4* rec, const float4* tgt, uint32_t n, cudaStream_t st) {
  uint32_t nb = 0;
  cudaError_t e = cudaMemsetAsync(c->loss.p, 0, sizeof(float), st);
  if (e != cudaSuccess) return e;
  e = forward_backward(c, rec, tgt, n, st, &nb);
  if (e != cudaSuccess) return e;
  AdamArgs A = adam_args(c);
  k_cache_adam_mlp<<<(NC_PARAMS + 255) / 256, 256, 0, st>>>(c->partials.p, nb, c->w.p, c->wm.p, c->wv.p, c->wn.p,
                                                            c->wk.p, A, nullptr);
  k_cache_adam_grid<<<(unsigned)((c->grid_count + 255) / 256), 256, 0, st>>>(c->ggrad.p, c->gw.p, c->gm.p, c->gv.p,
                                                                              c->gh.p, c->grid_count, A);
  return cudaGetLastError();
}

// The tensor-core kernel's wait-limit flag as of the last completed pass
// (the pinned copy is refreshed at the end of every pass, in stream order).
static cudaError_t tc_status(const pt_cache* c) {
  return (c->tc_err_host && *c->tc_err_host) ? cudaErrorLaunchTimeout : cudaSuccess;
}

cudaError_t cache_train_device(pt_cache* c, const float4* rec, const float4* tgt, uint32_t n, cudaStream_t st,
                               uint32_t* steps_done) {
  if (tc_status(c) != cudaSuccess) return cudaErrorLaunchTimeout;
  uint32_t steps = 0;
  if (n > 0) {
    const uint32_t B = c->cfg.batch_size;
    const uint32_t batches = (n + B - 1) / B;
    const uint32_t total = std::max(batches, c->cfg.steps_per_pass);
    for (uint32_t k = 0; k < total; ++k) {
      const uint32_t off = (k % batches) * B;
      const uint32_t m = std::min(B, n - off);
      cudaError_t e = train_step(c, rec + (size_t)off * 4, tgt + off, m, st);
      if (e != cudaSuccess) return e;
      ++steps;
    }
    cudaError_t e = cudaMemcpyAsync(c->tc_err_host, c->tc_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
  }
  if (steps_done) *steps_done = steps;
  return cudaSuccess;
}

}  // namespace hpt

namespace {
pt_status cfail(pt_cache* c, pt_status s, const std::string& m) {
  if (c) c->err = m;
  return s;
}
#define CCK(c, call)                                                                             \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return cfail((c), e_ == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA,              \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                          \
  } while (0)
}  // namespace

extern "C" {

void pt_cache_config_default(pt_cache_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->query_depth = 1;
  c->train_shift = 5;
  c->weight_grad_kernel = 0;
  c->batch_size = 1u << 16;
  c->log2_table_size = 19;
  c->learning_rate = 1e-2f;
  c->min_resolution = 16;
  c->max_resolution = 2048;
  c->seed = 1;
  c->warmup_frames = 1;
  c->paths_per_pass = 1u << 21;
  c->steps_per_pass = 1;
  c->min_roughness = 0.3f;
}

pt_status pt_cache_create(const pt_cache_config* cfg, pt_cache** out) try {
  if (!out) return PT_ERR_INVALID_ARG;
  *out = nullptr;
  pt_cache_config c;
  pt_cache_config_default(&c);
  if (cfg) {
    c = *cfg;
    pt_cache_config d;
    pt_cache_config_default(&d);
    if (!c.batch_size) c.batch_size = d.batch_size;
    if (!c.log2_table_size) c.log2_table_size = d.log2_table_size;
    if (c.learning_rate <= 0.0f) c.learning_rate = d.learning_rate;
    if (!c.min_resolution) c.min_resolution = d.min_resolution;
    if (!c.max_resolution) c.max_resolution = d.max_resolution;
  }
  if (c.log2_table_size < 8 || c.log2_table_size > 24 || c.min_resolution < 2 ||
      c.max_resolution < c.min_resolution || c.max_resolution > (1u << 20) || c.batch_size > (1u << 24) ||
      c.batch_size % 16 != 0 || c.train_shift > 16 || c.weight_grad_kernel > 1)
    return PT_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PT_ERR_CUDA;
  pt_cache* k = new pt_cache();
  k->cfg = c;
  const double b = std::exp((std::log((double)c.max_resolution) - std::log((double)c.min_resolution)) / (NC_LEVELS - 1));
  for (int l = 0; l < NC_LEVELS; ++l)
    k->V.res[l] = std::max<uint32_t>(2u, (uint32_t)std::floor((double)c.min_resolution * std::pow(b, (double)l)));
  k->V.log2_table = c.log2_table_size;
  for (int i = 0; i < 3; ++i) {
    k->V.lo[i] = 0.0f;
    k->V.inv_ext[i] = 1.0f;
  }
  k->grid_count = (uint64_t)NC_LEVELS * (1ull << c.log2_table_size) * 2;
  if (cudaStreamCreateWithFlags(&k->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete k;
    return PT_ERR_CUDA;
  }
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  chk(k->w.ensure(NC_PARAMS));
  chk(k->wm.ensure(NC_PARAMS));
  chk(k->wv.ensure(NC_PARAMS));
  chk(k->wn.ensure(NC_PARAMS));
  chk(k->wk.ensure(NC_PARAMS));
  chk(k->gw.ensure(k->grid_count));
  chk(k->gm.ensure(k->grid_count));
  chk(k->gv.ensure(k->grid_count));
  chk(k->ggrad.ensure(k->grid_count));
  chk(k->gh.ensure(k->grid_count));
  chk(k->loss.ensure(1));
  chk(k->tc_err.ensure(1));
  chk(cudaMallocHost(&k->tc_err_host, sizeof(uint32_t)));
  if (k->tc_err_host) *k->tc_err_host = 0;
  if (e != cudaSuccess) {
    pt_cache_destroy(k);
    return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
  }
  // Xavier-uniform MLP weights from a seeded generator; small uniform table
  std::vector<float> hw(NC_PARAMS);
  for (int l = 0; l < NC_LAYERS; ++l) {
    const int N = nc_layer_n(l);
    const float lim = std::sqrt(6.0f / (64.0f + (float)N));
    for (int i = 0; i < 64 * N; ++i)
      hw[nc_layer_off(l) + i] = lim * init_uniform(c.seed, (uint64_t)nc_layer_off(l) + i);
  }
  cudaStream_t st = k->stream;
  chk(cudaMemcpyAsync(k->w.p, hw.data(), NC_PARAMS * sizeof(float), cudaMemcpyHostToDevice, st));
  chk(cudaMemsetAsync(k->wm.p, 0, NC_PARAMS * sizeof(float), st));
  chk(cudaMemsetAsync(k->wv.p, 0, NC_PARAMS * sizeof(float), st));
  chk(cudaMemsetAsync(k->gm.p, 0, k->grid_count * sizeof(float), st));
  chk(cudaMemsetAsync(k->gv.p, 0, k->grid_count * sizeof(float), st));
  chk(cudaMemsetAsync(k->ggrad.p, 0, k->grid_count * sizeof(float), st));
  chk(cudaMemsetAsync(k->tc_err.p, 0, sizeof(uint32_t), st));
  k_cache_set_weights<<<(NC_PARAMS + 255) / 256, 256, 0, st>>>(k->w.p, k->wn.p, k->wk.p);
  const unsigned gb = (unsigned)((k->grid_count + 255) / 256);
  k_cache_init_grid<<<gb, 256, 0, st>>>(k->gw.p, k->grid_count, (uint64_t)c.seed * 7919u + 17u, 1e-4f);
  k_cache_set_grid<<<gb, 256, 0, st>>>(k->gw.p, k->gh.p, k->grid_count);
  chk(cudaGetLastError());
  chk(cudaStreamSynchronize(st));
  if (e != cudaSuccess) {
    pt_cache_destroy(k);
    return PT_ERR_CUDA;
  }
  k->V.wn = k->wn.p;
  k->V.wk = k->wk.p;
  k->V.grid = reinterpret_cast<const __half2*>(k->gh.p);
  k->V.grid_grad = reinterpret_cast<float2*>(k->ggrad.p);
  *out = k;
  return PT_OK;
} catch (...) {
  return host_exception_status(nullptr);
}

void pt_cache_destroy(pt_cache* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->tc_err_host) cudaFreeHost(c->tc_err_host);
  cudaStream_t s = c->stream;
  delete c;
  if (s) cudaStreamDestroy(s);
}

const char* pt_cache_last_error(const pt_cache* c) { return c ? c->err.c_str() : "null cache"; }

pt_status pt_cache_set_bounds(pt_cache* c, const float lo[3], const float hi[3]) try {
  if (!c || !lo || !hi) return PT_ERR_INVALID_ARG;
  for (int i = 0; i < 3; ++i) {
    if (!(hi[i] > lo[i])) return cfail(c, PT_ERR_INVALID_ARG, "bounds must have positive extent");
    c->V.lo[i] = lo[i];
    c->V.inv_ext[i] = 1.0f / (hi[i] - lo[i]);
  }
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

pt_status pt_cache_num_params(const pt_cache* c, uint64_t* mlp, uint64_t* grid) try {
  if (!c) return PT_ERR_INVALID_ARG;
  if (mlp) *mlp = NC_PARAMS;
  if (grid) *grid = c->grid_count;
  return PT_OK;
} catch (...) {
  return host_exception_status(nullptr);
}

pt_status pt_cache_get_params(pt_cache* c, float* mlp, float* grid) try {
  if (!c) return PT_ERR_INVALID_ARG;
  CCK(c, cudaStreamSynchronize(c->stream));
  if (mlp) CCK(c, cudaMemcpy(mlp, c->w.p, NC_PARAMS * sizeof(float), cudaMemcpyDeviceToHost));
  if (grid) CCK(c, cudaMemcpy(grid, c->gw.p, c->grid_count * sizeof(float), cudaMemcpyDeviceToHost));
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

pt_status pt_cache_set_params(pt_cache* c, const float* mlp, const float* grid) try {
  if (!c) return PT_ERR_INVALID_ARG;
  cudaStream_t st = c->stream;
  if (mlp) {
    CCK(c, cudaMemcpyAsync(c->w.p, mlp, NC_PARAMS * sizeof(float), cudaMemcpyHostToDevice, st));
    k_cache_set_weights<<<(NC_PARAMS + 255) / 256, 256, 0, st>>>(c->w.p, c->wn.p, c->wk.p);
  }
  if (grid) {
    CCK(c, cudaMemcpyAsync(c->gw.p, grid, c->grid_count * sizeof(float), cudaMemcpyHostToDevice, st));
    k_cache_set_grid<<<(unsigned)((c->grid_count + 255) / 256), 256, 0, st>>>(c->gw.p, c->gh.p, c->grid_count);
  }
  CCK(c, cudaGetLastError());
  CCK(c, cudaStreamSynchronize(st));
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

static pt_status upload_rows(pt_cache* c, const float* records, const float* targets, uint32_t n) {
  std::vector<float4> tg;
  CCK(c, c->rec.ensure((size_t)n * 4));
  CCK(c, cudaMemcpyAsync(c->rec.p, records, (size_t)n * NC_REC * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  if (targets) {
    tg.resize(n);
    for (uint32_t i = 0; i < n; ++i) tg[i] = make_float4(targets[3 * i], targets[3 * i + 1], targets[3 * i + 2], 0.0f);
    CCK(c, c->tgt.ensure(n));
    CCK(c, cudaMemcpyAsync(c->tgt.p, tg.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    CCK(c, cudaStreamSynchronize(c->stream));
  }
  return PT_OK;
}

pt_status pt_cache_infer(pt_cache* c, const float* records, uint32_t n, float* out_rgb) try {
  if (!c) return PT_ERR_INVALID_ARG;
  if (n == 0) return PT_OK;
  if (!records || !out_rgb) return cfail(c, PT_ERR_INVALID_ARG, "null buffer");
  pt_status s = upload_rows(c, records, nullptr, n);
  if (s != PT_OK) return s;
  Buf<float4> o;
  CCK(c, o.ensure(n));
  launch_cache_infer(c->V, c->rec.p, nullptr, nullptr, n, o.p, nullptr, c->stream);
  CCK(c, cudaGetLastError());
  std::vector<float4> h(n);
  CCK(c, cudaMemcpyAsync(h.data(), o.p, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
  CCK(c, cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < n; ++i) {
    out_rgb[3 * i] = h[i].x;
    out_rgb[3 * i + 1] = h[i].y;
    out_rgb[3 * i + 2] = h[i].z;
  }
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

pt_status pt_cache_gradients(pt_cache* c, const float* records, const float* targets, uint32_t n, float* mlp_grad,
                             float* grid_grad, float* loss) try {
  if (!c) return PT_ERR_INVALID_ARG;
  if (n == 0 || !records || !targets) return cfail(c, PT_ERR_INVALID_ARG, "empty batch or null buffer");
  pt_status s = upload_rows(c, records, targets, n);
  if (s != PT_OK) return s;
  cudaStream_t st = c->stream;
  CCK(c, cudaMemsetAsync(c->loss.p, 0, sizeof(float), st));
  uint32_t nb = 0;
  CCK(c, forward_backward(c, c->rec.p, c->tgt.p, n, st, &nb));
  CCK(c, c->gradbuf.ensure(NC_PARAMS));
  AdamArgs A{};
  k_cache_adam_mlp<<<(NC_PARAMS + 255) / 256, 256, 0, st>>>(c->partials.p, nb, c->w.p, c->wm.p, c->wv.p, c->wn.p,
                                                            c->wk.p, A, c->gradbuf.p);
  CCK(c, cudaGetLastError());
  if (mlp_grad)
    CCK(c, cudaMemcpyAsync(mlp_grad, c->gradbuf.p, NC_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (grid_grad)
    CCK(c, cudaMemcpyAsync(grid_grad, c->ggrad.p, c->grid_count * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (loss) CCK(c, cudaMemcpyAsync(loss, c->loss.p, sizeof(float), cudaMemcpyDeviceToHost, st));
  CCK(c, cudaMemsetAsync(c->ggrad.p, 0, c->grid_count * sizeof(float), st));
  CCK(c, cudaMemcpyAsync(c->tc_err_host, c->tc_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CCK(c, cudaStreamSynchronize(st));
  CCK(c, tc_status(c));
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}


pt_status pt_cache_benchmark(pt_cache* c, uint32_t n, uint32_t iterations, double* infer_ms, double* train_ms) try {
  if (!c || n == 0 || iterations == 0) return PT_ERR_INVALID_ARG;
  cudaStream_t st = c->stream;
  Buf<float4> rec, tgt, out;
  CCK(c, rec.ensure(4 * (size_t)n));
  CCK(c, tgt.ensure(n));
  CCK(c, out.ensure(n));
  k_cache_bench_records<<<(n + 255) / 256, 256, 0, st>>>(rec.p, tgt.p, n, 0x5EEDull);
  cudaEvent_t e0, e1;
  CCK(c, cudaEventCreate(&e0));
  CCK(c, cudaEventCreate(&e1));
  // warm-up, then timed inference
  launch_cache_infer(c->V, rec.p, nullptr, nullptr, n, out.p, nullptr, st);
  CCK(c, cudaEventRecord(e0, st));
  for (uint32_t k = 0; k < iterations; ++k) launch_cache_infer(c->V, rec.p, nullptr, nullptr, n, out.p, nullptr, st);
  CCK(c, cudaEventRecord(e1, st));
  CCK(c, cudaEventSynchronize(e1));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (infer_ms) *infer_ms = ms / iterations;
  // training steps over the same samples (one pass of batch_size batches each)
  const uint32_t keep = c->cfg.steps_per_pass;
  c->cfg.steps_per_pass = 0;
  uint32_t steps = 0;
  CCK(c, cudaEventRecord(e0, st));
  for (uint32_t k = 0; k < iterations; ++k) {
    uint32_t done = 0;
    cudaError_t e = cache_train_device(c, rec.p, tgt.p, n, st, &done);
    if (e != cudaSuccess) {
      c->cfg.steps_per_pass = keep;
      CCK(c, e);
    }
    steps += done;
  }
  CCK(c, cudaEventRecord(e1, st));
  CCK(c, cudaEventSynchronize(e1));
  c->cfg.steps_per_pass = keep;
  cudaEventElapsedTime(&ms, e0, e1);
  if (train_ms) *train_ms = ms / iterations;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CCK(c, cudaGetLastError());
  CCK(c, tc_status(c));
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

pt_status pt_cache_train(pt_cache* c, const float* records, const float* targets, uint32_t n, uint32_t steps,
                         float* last_loss) try {
  if (!c) return PT_ERR_INVALID_ARG;
  if (n == 0 || !records || !targets) return cfail(c, PT_ERR_INVALID_ARG, "empty batch or null buffer");
  pt_status s = upload_rows(c, records, targets, n);
  if (s != PT_OK) return s;
  cudaStream_t st = c->stream;
  const uint32_t keep = c->cfg.steps_per_pass;
  c->cfg.steps_per_pass = 0;
  for (uint32_t k = 0; k < steps; ++k) {
    uint32_t done = 0;
    cudaError_t e = cache_train_device(c, c->rec.p, c->tgt.p, n, st, &done);
    if (e != cudaSuccess) {
      c->cfg.steps_per_pass = keep;
      CCK(c, e);
    }
  }
  c->cfg.steps_per_pass = keep;
  if (last_loss) CCK(c, cudaMemcpyAsync(last_loss, c->loss.p, sizeof(float), cudaMemcpyDeviceToHost, st));
  CCK(c, cudaStreamSynchronize(st));
  CCK(c, tc_status(c));
  return PT_OK;
} catch (...) {
  return host_exception_status(c ? &c->err : nullptr);
}

}  // extern "C"
