// pt_bvh_fast.cu -- the fast BVH build of pt_renderer_set_bvh_build(r,
// PT_BVH_BUILD_FAST): a linear BVH over Morton codes, for geometry rebuilt
// every frame.
//
// The default build (pt_bvh.cu) prices 45 SAH planes at every node, level by
// level, with a host round trip per level. This one does a fixed number of
// passes over the triangles instead:
//   1. widened triangle boxes and centroids, block-reduced scene bounds;
//   2. 30-bit Morton codes of the centroids in the centroid bounds, with
//      bit 30 set for triangles much larger than the scene (a ground quad),
//      so that they form their own subtree under the root instead of
//      inflating the boxes along the path to wherever their centroid falls;
//   3. a stable least-significant-digit radix sort of the 31-bit keys
//      (4 passes of 8 bits; per tile of 1024 keys a digit histogram, one
//      exclusive scan of all tiles' histograms, then a stable scatter that
//      ranks equal digits by tile position through warp match masks);
//   4. the binary hierarchy of the sorted keys, every internal node at once
//      (Karras 2012: each node finds the direction and extent of its key
//      range from the common prefix lengths of neighbouring keys, ties broken
//      by index, then its split by binary search); a child whose range holds
//      at most 4 triangles becomes a leaf;
//   5. boxes bottom-up: a node with two leaf children starts a thread, which
//      climbs while it is the last of a parent's internal children to arrive
//      (an atomic counter per node);
//   6. the triangles in key order.
// The output is the binary traversal layout of pt_bvh.cu (node 0 the root),
// which collapse_wide turns into the wide tree. Closest hits do not depend
// on the tree (lexicographic minimum of (t, id) over the triangles the
// conservative boxes admit), so the images are those of the default build;
// only the traversal work differs.
#include <cuda_runtime.h>

#include <cuda/atomic>
#include <cstdint>
#include <utility>

#include "pt_internal.h"

namespace hpt {
namespace {

constexpr int FT = 256;               // threads per block
constexpr int TILE_ITEMS = 4;         // keys per thread in the sort
constexpr int TILE = FT * TILE_ITEMS; // keys per sort tile
constexpr uint32_t FAST_LEAF_MAX = 4;
constexpr uint32_t LARGE_KEY_BIT = 1u << 30;

__device__ __forceinline__ int ford(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float fdeord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

// bounds[0..2] centroid min, [3..5] centroid max, [6..8] box min, [9..11] box max (ordered ints)
__global__ void k_fast_prep(const float4* v0, const float4* e1, const float4* e2, uint32_t n, float4* tlo,
                            float4* thi, float4* tc, int* bounds) {
  __shared__ int red[FT / 32][12];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float cmn[3] = {1e30f, 1e30f, 1e30f}, cmx[3] = {-1e30f, -1e30f, -1e30f};
  float bmn[3] = {1e30f, 1e30f, 1e30f}, bmx[3] = {-1e30f, -1e30f, -1e30f};
  if (i < n) {
    const float4 a = v0[i], b4 = e1[i], c4 = e2[i];
    const float bx = __fadd_rn(a.x, b4.x), by = __fadd_rn(a.y, b4.y), bz = __fadd_rn(a.z, b4.z);
    const float cx = __fadd_rn(a.x, c4.x), cy = __fadd_rn(a.y, c4.y), cz = __fadd_rn(a.z, c4.z);
    float lo[3] = {fminf(a.x, fminf(bx, cx)), fminf(a.y, fminf(by, cy)), fminf(a.z, fminf(bz, cz))};
    float hi[3] = {fmaxf(a.x, fmaxf(bx, cx)), fmaxf(a.y, fmaxf(by, cy)), fmaxf(a.z, fmaxf(bz, cz))};
    float c[3];
    for (int k = 0; k < 3; ++k) {
      c[k] = (lo[k] + hi[k]) * 0.5f;
      // widened like the default build's boxes, so the slab test stays conservative
      lo[k] = lo[k] - (fabsf(lo[k]) * 4.8e-7f + 1e-30f);
      hi[k] = hi[k] + (fabsf(hi[k]) * 4.8e-7f + 1e-30f);
      cmn[k] = cmx[k] = c[k];
      bmn[k] = lo[k];
      bmx[k] = hi[k];
    }
    tlo[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    thi[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    tc[i] = make_float4(c[0], c[1], c[2], 0.0f);
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 3; ++k) {
      cmn[k] = fminf(cmn[k], __shfl_xor_sync(0xffffffffu, cmn[k], o));
      cmx[k] = fmaxf(cmx[k], __shfl_xor_sync(0xffffffffu, cmx[k], o));
      bmn[k] = fminf(bmn[k], __shfl_xor_sync(0xffffffffu, bmn[k], o));
      bmx[k] = fmaxf(bmx[k], __shfl_xor_sync(0xffffffffu, bmx[k], o));
    }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; ++k) {
      red[w][k] = ford(cmn[k]);
      red[w][3 + k] = ford(cmx[k]);
      red[w][6 + k] = ford(bmn[k]);
      red[w][9 + k] = ford(bmx[k]);
    }
  __syncthreads();
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    const bool is_min = (k < 3) || (k >= 6 && k < 9);
    int r = red[0][k];
    for (int ww = 1; ww < FT / 32; ++ww) r = is_min ? min(r, red[ww][k]) : max(r, red[ww][k]);
    if (is_min) atomicMin(&bounds[k], r);
    else atomicMax(&bounds[k], r);
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {  // 10 bits -> every third bit
  x &= 0x3FFu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void k_fast_morton(const float4* tlo, const float4* thi, const float4* tc, uint32_t n, const int* bounds,
                              uint32_t* keys, uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 c = tc[i], lo = tlo[i], hi = thi[i];
  const float cl[3] = {fdeord(bounds[0]), fdeord(bounds[1]), fdeord(bounds[2])};
  const float ch[3] = {fdeord(bounds[3]), fdeord(bounds[4]), fdeord(bounds[5])};
  const float bl[3] = {fdeord(bounds[6]), fdeord(bounds[7]), fdeord(bounds[8])};
  const float bh[3] = {fdeord(bounds[9]), fdeord(bounds[10]), fdeord(bounds[11])};
  const float cc[3] = {c.x, c.y, c.z};
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    const float ext = ch[k] - cl[k];
    float f = ext > 0.0f ? (cc[k] - cl[k]) / ext : 0.0f;
    f = fminf(fmaxf(f, 0.0f), 1.0f);
    q[k] = min(1023u, (uint32_t)(f * 1024.0f));
  }
  uint32_t key = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  const float scene = fmaxf(fmaxf(bh[0] - bl[0], bh[1] - bl[1]), bh[2] - bl[2]);
  const float tri = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
  if (tri > scene * (1.0f / 32.0f)) key |= LARGE_KEY_BIT;
  keys[i] = key;
  vals[i] = i;
}

// ---------------------------------------------------------------- radix sort
// hist[digit * ntiles + tile] = keys of `tile` with that 8-bit digit
__global__ void k_rs_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t* hist, uint32_t ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * TILE;
  for (int j = 0; j < TILE_ITEMS; ++j) {
    const uint32_t e = base + j * FT + threadIdx.x;
    if (e < n) atomicAdd(&h[(keys[e] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan, three kernels: per block of 1024 values, the block sums in
// one block, then the block offsets added back.
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_BLOCK = FT * SCAN_ITEMS;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[FT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < FT / 32 ? ws[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < FT / 32) ws[lane] = s;
  }
  __syncthreads();
  const uint32_t before = w > 0 ? ws[w - 1] : 0u;
  *total = ws[FT / 32 - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void k_scan_local(uint32_t* data, uint32_t m, uint32_t* sums) {
  const uint32_t base = blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS], s = 0;
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    v[j] = base + j < m ? data[base + j] : 0u;
    s += v[j];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, &total);
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    if (base + j < m) data[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block scans up to FT * 128 block sums in place.
__global__ void k_scan_sums(uint32_t* sums, uint32_t m) {
  const uint32_t per = (m + FT - 1) / FT;
  const uint32_t base = threadIdx.x * per;
  uint32_t s = 0;
  for (uint32_t j = 0; j < per && base + j < m; ++j) s += sums[base + j];
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, &total);
  for (uint32_t j = 0; j < per && base + j < m; ++j) {
    const uint32_t x = sums[base + j];
    sums[base + j] = run;
    run += x;
  }
}

__global__ void k_scan_add(uint32_t* data, uint32_t m, const uint32_t* sums) {
  const uint32_t base = blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_ITEMS;
  const uint32_t add = sums[blockIdx.x];
  for (int j = 0; j < SCAN_ITEMS; ++j)
    if (base + j < m) data[base + j] += add;
}

// Stable scatter of one tile: its keys are taken in TILE_ITEMS rounds of FT
// consecutive positions; within a round, equal digits are ranked by lane
// (warp match mask) and warp (per-warp counts), and the rounds follow each
// other through a running count per digit, so the tile keeps its order.
__global__ void k_rs_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                             int shift, const uint32_t* offs, uint32_t ntiles) {
  __shared__ uint32_t run[256];
  __shared__ uint32_t cnt[FT / 32][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  run[threadIdx.x] = offs[threadIdx.x * ntiles + blockIdx.x];
  const uint32_t base = blockIdx.x * TILE;
  for (int j = 0; j < TILE_ITEMS; ++j) {
    for (int k = threadIdx.x; k < (FT / 32) * 256; k += FT) (&cnt[0][0])[k] = 0u;
    __syncthreads();
    const uint32_t e = base + j * FT + threadIdx.x;
    const bool valid = e < n;
    const uint32_t key = valid ? kin[e] : 0u;
    const uint32_t d = valid ? (key >> shift) & 0xFFu : 0x100u + (uint32_t)lane;  // invalid lanes never match
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) cnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pos = run[d] + rank;
      for (int ww = 0; ww < w; ++ww) pos += cnt[ww][d];
      kout[pos] = key;
      vout[pos] = vin[e];
    }
    __syncthreads();
    uint32_t add = 0;
    for (int ww = 0; ww < FT / 32; ++ww) add += cnt[ww][threadIdx.x];
    run[threadIdx.x] += add;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- hierarchy
__device__ __forceinline__ int prefix_len(const uint32_t* keys, uint32_t n, int i, int j) {
  if (j < 0 || j >= (int)n) return -1;
  const uint32_t a = keys[i], b = keys[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// link = internal node index, or a leaf link of the range [first, first+count)
__global__ void k_fast_karras(const uint32_t* keys, uint32_t n, int2* links, int2* range, int* parent,
                              uint32_t* needed) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)n - 1) return;
  const int d = prefix_len(keys, n, i, i + 1) - prefix_len(keys, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = prefix_len(keys, n, i, i - d);
  int lmax = 2;
  while (prefix_len(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (prefix_len(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = prefix_len(keys, n, i, j);
  int s = 0;
  for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
    if (s + t <= l && prefix_len(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  range[i] = make_int2(first, last);
  const uint32_t lsize = (uint32_t)(gamma - first + 1), rsize = (uint32_t)(last - gamma);
  int2 lk;
  uint32_t need = 0;
  if (lsize <= FAST_LEAF_MAX) {
    lk.x = make_leaf_link((uint32_t)first, lsize);
  } else {
    lk.x = gamma;
    parent[gamma] = i;
    ++need;
  }
  if (rsize <= FAST_LEAF_MAX) {
    lk.y = make_leaf_link((uint32_t)(gamma + 1), rsize);
  } else {
    lk.y = gamma + 1;
    parent[gamma + 1] = i;
    ++need;
  }
  links[i] = lk;
  needed[i] = need;
}

__device__ __forceinline__ void leaf_box(const float4* tlo, const float4* thi, const uint32_t* ids, int32_t link,
                                         float lo[3], float hi[3]) {
  const uint32_t start = (uint32_t)link & 0x03FFFFFFu, count = ((uint32_t)link >> 26) & 0x1Fu;
  lo[0] = lo[1] = lo[2] = 1e30f;
  hi[0] = hi[1] = hi[2] = -1e30f;
  for (uint32_t k = start; k < start + count; ++k) {
    const uint32_t id = ids[k];
    const float4 a = tlo[id], b = thi[id];
    lo[0] = fminf(lo[0], a.x); lo[1] = fminf(lo[1], a.y); lo[2] = fminf(lo[2], a.z);
    hi[0] = fmaxf(hi[0], b.x); hi[1] = fmaxf(hi[1], b.y); hi[2] = fmaxf(hi[2], b.z);
  }
}

// Bottom-up boxes. `boxes` holds each finished node's own box (lo, hi);
// trav is the binary traversal layout (child boxes and links).
__global__ void k_fast_bounds(const float4* tlo, const float4* thi, const uint32_t* ids, const int2* links,
                              const int2* range, const int* parent, const uint32_t* needed, uint32_t* arrived,
                              float4* boxes, float4* trav, uint32_t n) {
  int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)n - 1) return;
  const int2 r = range[i];
  const bool active = i == 0 || (uint32_t)(r.y - r.x + 1) > FAST_LEAF_MAX;
  if (!active || needed[i] != 0) return;
  for (uint32_t steps = 0; steps < n; ++steps) {  // at most the depth of the tree
    const int2 lk = links[i];
    float clo[2][3], chi[2][3];
    const int32_t l[2] = {lk.x, lk.y};
    for (int c = 0; c < 2; ++c) {
      if (l[c] < 0) {
        leaf_box(tlo, thi, ids, l[c], clo[c], chi[c]);
      } else {
        const float4 a = __ldcg(&boxes[2 * l[c]]), b = __ldcg(&boxes[2 * l[c] + 1]);
        clo[c][0] = a.x; clo[c][1] = a.y; clo[c][2] = a.z;
        chi[c][0] = b.x; chi[c][1] = b.y; chi[c][2] = b.z;
      }
    }
    trav[4 * i] = make_float4(clo[0][0], chi[0][0], clo[0][1], chi[0][1]);
    trav[4 * i + 1] = make_float4(clo[1][0], chi[1][0], clo[1][1], chi[1][1]);
    trav[4 * i + 2] = make_float4(clo[0][2], chi[0][2], clo[1][2], chi[1][2]);
    trav[4 * i + 3] = make_float4(__int_as_float(l[0]), __int_as_float(l[1]), 0.0f, 0.0f);
    __stcg(&boxes[2 * i], make_float4(fminf(clo[0][0], clo[1][0]), fminf(clo[0][1], clo[1][1]),
                                      fminf(clo[0][2], clo[1][2]), 0.0f));
    __stcg(&boxes[2 * i + 1], make_float4(fmaxf(chi[0][0], chi[1][0]), fmaxf(chi[0][1], chi[1][1]),
                                          fmaxf(chi[0][2], chi[1][2]), 0.0f));
    const int p = i == 0 ? -1 : parent[i];
    if (p < 0) return;
    // release: this node's box is visible to whoever continues at p;
    // acquire: if that is this thread, it sees the other child's box
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrivals(arrived[p]);
    const uint32_t before = arrivals.fetch_add(1u, cuda::std::memory_order_acq_rel);
    if (before + 1u < needed[p]) return;  // the other child is not finished: its thread continues
    i = p;
  }
}

__global__ void k_fast_reorder(const uint32_t* ids, uint32_t n, const float4* v0, const float4* e1, const float4* e2,
                               float4* out) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t id = ids[s];
  float4 a = v0[id];
  a.w = __uint_as_float(id);
  out[3 * s] = a;
  out[3 * s + 1] = e1[id];
  out[3 * s + 2] = e2[id];
}

template <class T>
struct FTmp {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(reinterpret_cast<void**>(&p), n * sizeof(T), st);
  }
  ~FTmp() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

int build_bvh_fast(const float4* tri_v0, const float4* tri_e1, const float4* tri_e2, uint32_t n, BvhBuffers& out,
                   uint32_t* num_nodes, cudaStream_t st) {
  if (n < 2) return build_bvh(tri_v0, tri_e1, tri_e2, n, out, num_nodes, st);
  if (out.node_capacity < n - 1) return 5;
  const uint32_t ntiles = (n + TILE - 1) / TILE;
  const uint32_t m = 256u * ntiles;  // histogram entries
  const uint32_t nscan = (m + SCAN_BLOCK - 1) / SCAN_BLOCK;
  if (nscan > (uint32_t)FT * 128u) return 6;
  FTmp<float4> tlo, thi, tc, boxes;
  FTmp<uint32_t> ka, kb, va, vb, hist, sums, needed, arrived;
  FTmp<int> bounds, parent;
  FTmp<int2> links, range;
  if (tlo.alloc(n, st) || thi.alloc(n, st) || tc.alloc(n, st) || boxes.alloc(2 * (size_t)n, st) ||
      ka.alloc(n, st) || kb.alloc(n, st) || va.alloc(n, st) || vb.alloc(n, st) || hist.alloc(m, st) ||
      sums.alloc(nscan, st) || needed.alloc(n, st) || arrived.alloc(n, st) || bounds.alloc(12, st) ||
      parent.alloc(n, st) || links.alloc(n, st) || range.alloc(n, st))
    return 2;
  // ordered-int bounds start at (+max, -max)
  int init[12];
  for (int k = 0; k < 12; ++k) init[k] = (k < 3 || (k >= 6 && k < 9)) ? 0x7F7FFFFF : (int)0x80800000;
  cudaMemcpyAsync(bounds.p, init, sizeof(init), cudaMemcpyHostToDevice, st);
  const uint32_t g = (n + FT - 1) / FT;
  k_fast_prep<<<g, FT, 0, st>>>(tri_v0, tri_e1, tri_e2, n, tlo.p, thi.p, tc.p, bounds.p);
  k_fast_morton<<<g, FT, 0, st>>>(tlo.p, thi.p, tc.p, n, bounds.p, ka.p, va.p);
  uint32_t *kin = ka.p, *kout = kb.p, *vin = va.p, *vout = vb.p;
  for (int shift = 0; shift < 32; shift += 8) {
    k_rs_hist<<<ntiles, FT, 0, st>>>(kin, n, shift, hist.p, ntiles);
    k_scan_local<<<nscan, FT, 0, st>>>(hist.p, m, sums.p);
    k_scan_sums<<<1, FT, 0, st>>>(sums.p, nscan);
    k_scan_add<<<nscan, FT, 0, st>>>(hist.p, m, sums.p);
    k_rs_scatter<<<ntiles, FT, 0, st>>>(kin, vin, kout, vout, n, shift, hist.p, ntiles);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  cudaMemsetAsync(parent.p, 0xFF, sizeof(int) * n, st);
  cudaMemsetAsync(arrived.p, 0, sizeof(uint32_t) * n, st);
  k_fast_karras<<<(n - 1 + FT - 1) / FT, FT, 0, st>>>(kin, n, links.p, range.p, parent.p, needed.p);
  k_fast_bounds<<<(n - 1 + FT - 1) / FT, FT, 0, st>>>(tlo.p, thi.p, vin, links.p, range.p, parent.p, needed.p,
                                                       arrived.p, boxes.p, out.nodes, n);
  k_fast_reorder<<<g, FT, 0, st>>>(vin, n, tri_v0, tri_e1, tri_e2, out.tri_sorted);
  if (cudaGetLastError() != cudaSuccess) return 3;
  if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  *num_nodes = n - 1;
  return 0;
}

}  // namespace hpt
