// pt_cache.h -- device view of the radiance cache (multiresolution hash-grid
// encoding + 6-layer MLP) shared by the cache kernels and the renderer.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/hala_pt.h"

namespace hpt {

constexpr int NC_LEVELS = 16;      // hash-grid levels, 2 features each -> 32 inputs
constexpr int NC_IN = 64;          // MLP input width (32 encoded + 13 raw + padding)
constexpr int NC_LAYERS = 6;       // 5 hidden layers of 64 + the output layer
constexpr int NC_OUT = 16;         // output width (RGB in 0..2, the rest padding)
constexpr int NC_PARAMS = 5 * 64 * 64 + 64 * NC_OUT;  // 21504
constexpr int NC_REC = 16;         // floats per query record

__host__ __device__ constexpr int nc_layer_n(int l) { return l == NC_LAYERS - 1 ? NC_OUT : 64; }
__host__ __device__ constexpr int nc_layer_off(int l) { return l * 64 * 64; }

// Query record (16 floats): position xyz, outgoing direction xyz, shading
// normal xyz, base colour rgb, roughness, metallic, specular transmission, 0.
struct CacheView {
  const __nv_bfloat16* wn;  // weights [layer][out n][in k] (forward operand)
  const __nv_bfloat16* wk;  // weights [layer][in k][out n] (backward operand)
  const __half2* grid;      // [level][table] two fp16 features
  float2* grid_grad;        // [level][table] fp32 gradient (training)
  float lo[3], inv_ext[3];  // scene bounds -> unit cube
  uint32_t res[NC_LEVELS];  // grid resolution per level
  uint32_t log2_table;
};

// Evaluates the cache for `n` records (n read from *count_dev when it is not
// null). Record slot of row r: idx ? idx[r] : r. With `scale`, out[slot].xyz
// += scale[slot].xyz * max(prediction, 0) (w kept); without, out[slot] =
// (prediction, 0).
void launch_cache_infer(const CacheView& V, const float4* rec, const uint32_t* idx, const uint32_t* count_dev,
                        uint32_t n_max, float4* out, const float4* scale, cudaStream_t st);

}  // namespace hpt

struct pt_cache;

namespace hpt {
// Renderer-side training interface: one optimisation pass over `n` samples
// already on the device (records + targets as float4 rgb), in batches.
cudaError_t cache_train_device(pt_cache* c, const float4* rec, const float4* tgt, uint32_t n, cudaStream_t st,
                               uint32_t* steps_done);
CacheView cache_view(const pt_cache* c);
// pt_cache_tc.cu: dW of every layer on the tensor cores (tcgen05, TMEM
// accumulators) into per-block partials [layer][block][k][n]; *err gets bit 0
// if a wait for the tensor cores ran out of its iteration limit.
size_t cache_dw_tc_smem();
void launch_cache_dw_tc(const __nv_bfloat16* X, const __nv_bfloat16* D, size_t cap, uint32_t n,
                        uint32_t rows_per_block, float* partials, uint32_t nblocks, uint32_t* err, cudaStream_t st);
// Loss of the last training batch (synchronous read).
cudaError_t cache_last_loss(pt_cache* c, float* loss);
}  // namespace hpt
