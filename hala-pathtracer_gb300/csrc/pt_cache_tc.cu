// pt_cache_tc.cu -- weight gradients of the radiance-cache MLP on the
// Blackwell tensor cores: tcgen05.mma with the accumulator in tensor memory.
//
// dW_l = X_l^T dZ_l for every layer l, X_l the layer's input rows (batch x 64,
// bf16) and dZ_l its output gradient rows (batch x N_l, bf16), summed over the
// batch: a contraction with M = 64 input features, N = N_l outputs and the
// batch as K. Two layers share one 128 x 128 MMA tile: A stacks X_a^T over
// X_b^T (128 rows), B stacks dZ_a^T over dZ_b^T (128 columns), so the tile's
// two diagonal 64 x 64 blocks are dW_a and dW_b (the off-diagonal blocks are
// computed and dropped: the MMAs are not what this kernel waits on). Layer
// pairs (0,1), (2,3), (4,5); layer 5 has 16 outputs, zero-padded to 64.
//
// One CTA of four warps per (pair, run of rows). Per chunk of 64 rows the
// warps stage A and B into shared memory transposed to K-major order in the
// 128-byte swizzled layout (8 rows of 128 B per 1024-B atom, 16-B chunk c of
// row m at c ^ (m & 7)); one thread issues four tcgen05.mma (K = 16 each)
// into the 128 x 128 fp32 accumulator in TMEM (128 columns) and commits them
// to an mbarrier that every thread waits on, with an iteration limit, before
// the buffers are reused. The epilogue reads the diagonal blocks from TMEM
// (tcgen05.ld, warp w owns lanes 32w..32w+31) into the per-block partials
// that the Adam kernel sums in a fixed order, the layout of k_cache_dw.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pt_cache.h"

namespace hpt {
namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_KC = 64;                       // rows (K) per staged chunk: one 128-B swizzle row
constexpr int TC_TILE_BYTES = 128 * TC_KC * 2;  // 128 rows x 64 bf16 = 16 KB per operand
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;    // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): K-major, 128-byte swizzle,
// 1024 B between 8-row groups, descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);            // start address
  d |= (uint64_t)(16u >> 4) << 16;                    // leading byte offset (unused with swizzling)
  d |= (uint64_t)(1024u >> 4) << 32;                  // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                             // version
  d |= (uint64_t)2 << 61;                             // layout: 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// Byte offset of element (row m, column k) of a K-major 128-row x 64-column
// bf16 tile in the 128-byte swizzled layout.
__device__ __forceinline__ uint32_t sw128_off(uint32_t m, uint32_t k) {
  return m * 128u + ((((k >> 3) ^ (m & 7u)) & 7u) << 4) + ((k & 7u) << 1);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (uint32_t it = 0; it < TC_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__global__ void __launch_bounds__(TC_THREADS) k_cache_dw_tc(const __nv_bfloat16* X, const __nv_bfloat16* D,
                                                            size_t cap, uint32_t n, uint32_t rows_per_block,
                                                            float* partials, uint32_t nblocks, uint32_t* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // 1024-byte alignment of the swizzled tiles
  const uint32_t base = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (base & 1023u)) & 1023u;
  unsigned char* tiles = smem_raw + pad;
  unsigned char* tileA = tiles;
  unsigned char* tileB = tiles + TC_TILE_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tiles + 2 * TC_TILE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tiles + 2 * TC_TILE_BYTES + 8);

  const int pair = blockIdx.y;
  const int la = 2 * pair, lb = 2 * pair + 1;
  const int Nb = nc_layer_n(lb);  // 64, or 16 for the output layer
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t ls = cap * 64;
  const __nv_bfloat16* Xa = X + (size_t)la * ls;
  const __nv_bfloat16* Xb = X + (size_t)lb * ls;
  const __nv_bfloat16* Da = D + (size_t)la * ls;
  const __nv_bfloat16* Db = D + (size_t)lb * ls;
  const uint32_t r_begin = blockIdx.x * rows_per_block;
  const uint32_t r_end = min(n, r_begin + rows_per_block);

  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {  // 128 TMEM columns: the 128 x 128 fp32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;\n" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const uint32_t idesc = mma_idesc(128, 128);
  const uint32_t a_addr = smem_u32(tileA), b_addr = smem_u32(tileB);
  uint32_t phase = 0;
  bool ok = true;
  bool first = true;
  for (uint32_t c0 = r_begin; c0 < r_end && ok; c0 += TC_KC) {
    // stage: item = (operand half h: 0 = layer a, 1 = layer b; row pair rp;
    // group of 8 columns g); two rows r, r+1 of 8 columns become eight
    // (column, k-pair) words of the K-major tile
    for (int item = threadIdx.x; item < 2 * 2 * 32 * 8; item += TC_THREADS) {
      const int which = item >> 9;          // 0 = A (inputs), 1 = B (gradients)
      const int h = (item >> 8) & 1;
      const int rp = (item >> 3) & 31;
      const int g = item & 7;
      const uint32_t k = 2u * rp;
      const uint32_t r0 = c0 + k, r1 = r0 + 1;
      uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0;
      if (which == 0) {
        const __nv_bfloat16* src = h ? Xb : Xa;
        if (r0 < r_end) v0 = *reinterpret_cast<const uint4*>(src + (size_t)r0 * 64 + 8 * g);
        if (r1 < r_end) v1 = *reinterpret_cast<const uint4*>(src + (size_t)r1 * 64 + 8 * g);
      } else {
        const int N = h ? Nb : 64;
        const __nv_bfloat16* src = h ? Db : Da;
        if (8 * g < N) {
          if (r0 < r_end) v0 = *reinterpret_cast<const uint4*>(src + (size_t)r0 * N + 8 * g);
          if (r1 < r_end) v1 = *reinterpret_cast<const uint4*>(src + (size_t)r1 * N + 8 * g);
        }
      }
      unsigned char* tile = which ? tileB : tileA;
      const uint32_t w0[4] = {v0.x, v0.y, v0.z, v0.w}, w1[4] = {v1.x, v1.y, v1.z, v1.w};
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t lo = (w0[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
        const uint32_t hi = (w1[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
        const uint32_t m = 64u * h + 8u * g + j;
        *reinterpret_cast<uint32_t*>(tile + sw128_off(m, k)) = lo | (hi << 16);
      }
    }
    // the generic-proxy stores must be visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < TC_KC / 16; ++ks) {
        const uint64_t ad = sw128_desc(a_addr + 32u * ks), bd = sw128_desc(b_addr + 32u * ks);
        const uint32_t acc = first && ks == 0 ? 0u : 1u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(mbar))
                   : "memory");
    }
    first = false;
    // every thread waits for the MMAs before the tiles are overwritten
    if (!mbar_wait(smem_u32(mbar), phase)) {
      ok = false;
      if (threadIdx.x == 0) atomicOr(err, 1u);
    }
    phase ^= 1u;
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

  // epilogue: lanes 0-63 are dW_a rows (input feature k), columns 0-63 its
  // outputs; lanes 64-127 are dW_b rows, columns 64.. its outputs
  if (ok && !first) {
    const int row = 32 * warp + lane;
    const bool is_b = warp >= 2;
    const int l = is_b ? lb : la;
    const int N = is_b ? Nb : 64;
    const int k = is_b ? row - 64 : row;
    float* P = partials + ((size_t)l * nblocks + blockIdx.x) * 4096 + (size_t)k * N;
    for (int cb = 0; cb < N; cb += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)((is_b ? 64 : 0) + cb);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
          "[%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) P[cb + j] = __uint_as_float(v[j]);
    }
  } else if (first) {
    // no rows in this block: zero partials
    const int row = 32 * warp + lane;
    const bool is_b = warp >= 2;
    const int l = is_b ? lb : la;
    const int N = is_b ? Nb : 64;
    const int k = is_b ? row - 64 : row;
    float* P = partials + ((size_t)l * nblocks + blockIdx.x) * 4096 + (size_t)k * N;
    for (int j = 0; j < N; ++j) P[j] = 0.0f;
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;\n" ::"r"(tmem) : "memory");
  }
}

}  // namespace

// 1 KB alignment slack + two 16 KB tiles + the mbarrier and TMEM address,
// rounded up to 64 KB so that at most three CTAs share an SM: 3 x 128 TMEM
// columns fit the SM's 512, and no tcgen05.alloc waits for another CTA.
size_t cache_dw_tc_smem() { return 64 * 1024; }
static_assert(1024 + 2 * TC_TILE_BYTES + 16 <= 64 * 1024, "tiles exceed the shared-memory request");

void launch_cache_dw_tc(const __nv_bfloat16* X, const __nv_bfloat16* D, size_t cap, uint32_t n,
                        uint32_t rows_per_block, float* partials, uint32_t nblocks, uint32_t* err, cudaStream_t st) {
  static bool attr = false;
  const size_t smem = cache_dw_tc_smem();
  if (!attr) {
    cudaFuncSetAttribute(k_cache_dw_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_cache_dw_tc<<<dim3(nblocks, NC_LAYERS / 2), TC_THREADS, smem, st>>>(X, D, cap, n, rows_per_block, partials,
                                                                        nblocks, err);
}

}  // namespace hpt
