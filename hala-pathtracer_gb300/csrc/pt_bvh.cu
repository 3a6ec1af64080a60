// pt_bvh.cu -- device BVH build (replaces the RT-core acceleration structure
// that hala-renderer builds for traceRayEXT).
//
// Top-down binned SAH, level-synchronous: every level launches one CTA per
// open task. A CTA bins its task's triangle centroids into 16 bins per axis
// (bin boxes kept as order-preserving integers in shared memory), picks the
// cheapest SAH plane, and stably partitions the task's triangle ids into the
// other ping-pong buffer with a block-wide scan. Leaves (<= 4 triangles, or
// when SAH says so) copy their ids into the final order. Tasks of more than
// LARGE_TASK triangles (the top levels of big scenes) are spread over many
// blocks instead (k_large_*), with the same planes and the same partition
// order. A layout pass then writes the 64-byte binary nodes and the
// triangles in leaf order; k_collapse turns the binary tree into the wide
// traversal nodes.
#include <cuda.h>  // driver types only (the driver call is reached through cudaGetDriverEntryPointByVersion)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "pt_internal.h"

namespace hpt {

namespace {

constexpr int NB = 16;
constexpr int BUILD_THREADS = 256;
constexpr int SAH_LEAF_MAX = 4;
// SAH cost of visiting a node, in units of one triangle test.
constexpr float SAH_NODE_COST = 0.5f;

struct BuildNode {
  float lo[3];
  float hi[3];
  int32_t left, right;
  uint32_t start, count;
};
struct BuildTask {
  uint32_t node, start, count, pad;
};

__device__ __forceinline__ int f2o(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__device__ __forceinline__ float box_area(float lx, float ly, float lz, float hx, float hy, float hz) {
  float ex = hx - lx, ey = hy - ly, ez = hz - lz;
  if (ex < 0.0f) return 0.0f;
  return 2.0f * (ex * ey + ey * ez + ez * ex);
}

// Per-triangle bounds (widened by a few ulp) and centroid.
__global__ void k_prep(const float4* v0, const float4* e1, const float4* e2, uint32_t n, float4* tlo, float4* thi,
                       float4* tc, uint32_t* ids) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = v0[i], b4 = e1[i], c4 = e2[i];
  float bx = __fadd_rn(a.x, b4.x), by = __fadd_rn(a.y, b4.y), bz = __fadd_rn(a.z, b4.z);
  float cx = __fadd_rn(a.x, c4.x), cy = __fadd_rn(a.y, c4.y), cz = __fadd_rn(a.z, c4.z);
  float lx = fminf(a.x, fminf(bx, cx)), ly = fminf(a.y, fminf(by, cy)), lz = fminf(a.z, fminf(bz, cz));
  float hx = fmaxf(a.x, fmaxf(bx, cx)), hy = fmaxf(a.y, fmaxf(by, cy)), hz = fmaxf(a.z, fmaxf(bz, cz));
  tc[i] = make_float4((lx + hx) * 0.5f, (ly + hy) * 0.5f, (lz + hz) * 0.5f, 0.0f);
  auto lo = [](float x) { return x - (fabsf(x) * 4.8e-7f + 1e-30f); };
  auto hi = [](float x) { return x + (fabsf(x) * 4.8e-7f + 1e-30f); };
  tlo[i] = make_float4(lo(lx), lo(ly), lo(lz), 0.0f);
  thi[i] = make_float4(hi(hx), hi(hy), hi(hz), 0.0f);
  ids[i] = i;
}

__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Bins one triangle per valid lane on the three axes into shared bins
// (count, min box, max box as ordered ints). Lanes of the warp that fall into
// the same bin are merged first (__match_any_sync, then reductions over that
// group) and the lowest of them does the atomics: in the multi-block top
// levels neighbouring triangles are close in space and would otherwise hit
// one bin with 32 atomics in a row (2.4x faster there; in the small tasks of
// k_level and k_subtree, where few lanes share a bin, the plain atomics are
// faster). All 32 lanes call it; cext[] is uniform over the warp. Integer
// counts and min/max: the bins do not depend on the order.
__device__ __forceinline__ void bin_warp(bool valid, float4 c, float4 lo, float4 hi, const float clo[3],
                                         const float cext[3], int (*bcnt)[NB], int (*bmin)[NB][3],
                                         int (*bmax)[NB][3]) {
  const unsigned act = __ballot_sync(0xffffffffu, valid);
  if (!valid) return;
  const int lane = threadIdx.x & 31;
  const float cc[3] = {c.x, c.y, c.z};
  const int ilo[3] = {f2o(lo.x), f2o(lo.y), f2o(lo.z)};
  const int ihi[3] = {f2o(hi.x), f2o(hi.y), f2o(hi.z)};
  for (int a = 0; a < 3; ++a) {
    if (!(cext[a] > 0.0f)) continue;
    const int b = min(NB - 1, max(0, (int)((cc[a] - clo[a]) * ((float)NB / cext[a]))));
    const unsigned grp = __match_any_sync(act, b);
    int gl[3], gh[3];
    for (int k = 0; k < 3; ++k) {
      gl[k] = __reduce_min_sync(grp, ilo[k]);
      gh[k] = __reduce_max_sync(grp, ihi[k]);
    }
    if (lane == __ffs(grp) - 1) {
      atomicAdd(&bcnt[a][b], __popc(grp));
      for (int k = 0; k < 3; ++k) {
        atomicMin(&bmin[a][b][k], gl[k]);
        atomicMax(&bmax[a][b][k], gh[k]);
      }
    }
  }
}

constexpr uint32_t MAX_LARGE_TASKS = 1024;  // capacity of the per-level large-task list

// Where the children of a split task go: the next level's list (one block
// per task), the multi-block list (more than large_min triangles), or the
// whole-subtree list (at most sub_max triangles, built to the leaves by one
// warp each after the levels; `dst_parity` records which id buffer holds
// their ranges). A full list spills into the next level's list, which builds
// the same tree more slowly.
struct ChildLists {
  BuildTask* tasks;
  uint32_t* count;
  BuildTask* large = nullptr;
  uint32_t* large_count = nullptr;
  uint32_t large_min = 0xFFFFFFFFu;
  BuildTask* sub = nullptr;
  uint32_t* sub_count = nullptr;
  uint32_t sub_max = 0;
  uint32_t sub_cap = 0;
  uint32_t dst_parity = 0;
};

__device__ __forceinline__ void push_children(uint32_t c, const BuildTask& t, uint32_t nleft, const ChildLists& L) {
  const BuildTask kids[2] = {BuildTask{c, t.start, nleft, 0}, BuildTask{c + 1, t.start + nleft, t.count - nleft, 0}};
  for (int k = 0; k < 2; ++k) {
    if (L.sub && kids[k].count <= L.sub_max) {
      const uint32_t q = atomicAdd(L.sub_count, 1u);
      if (q < L.sub_cap) {
        L.sub[q] = BuildTask{kids[k].node, kids[k].start, kids[k].count, L.dst_parity};
        continue;
      }
    }
    if (L.large && kids[k].count > L.large_min) {
      const uint32_t q = atomicAdd(L.large_count, 1u);
      if (q < MAX_LARGE_TASKS) {
        L.large[q] = kids[k];
        continue;
      }
    }
    L.tasks[atomicAdd(L.count, 1u)] = kids[k];
  }
}

__global__ void __launch_bounds__(BUILD_THREADS) k_level(const BuildTask* tasks, const uint32_t* ntasks_ptr,
                                                         const uint32_t* src, uint32_t* dst, uint32_t* final_ids,
                                                         const float4* tlo, const float4* thi, const float4* tc,
                                                         BuildNode* nodes, uint32_t* node_counter, ChildLists next) {
  __shared__ float red[12][BUILD_THREADS / 32];
  __shared__ float box[12];
  __shared__ int bcnt[3][NB];
  __shared__ int bmin[3][NB][3];
  __shared__ int bmax[3][NB][3];
  __shared__ float cost_s[3 * (NB - 1)];
  __shared__ int best_s;
  __shared__ uint32_t wcount[BUILD_THREADS / 32];
  if (blockIdx.x >= *ntasks_ptr) return;
  const BuildTask t = tasks[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t end = t.start + t.count;

  // 1. box and centroid box
  float v[12];
  for (int k = 0; k < 6; ++k) { v[k] = 1e30f; v[6 + k] = -1e30f; }
  for (uint32_t i = t.start + tid; i < end; i += BUILD_THREADS) {
    uint32_t id = src[i];
    float4 lo = tlo[id], hi = thi[id], c = tc[id];
    v[0] = fminf(v[0], lo.x); v[1] = fminf(v[1], lo.y); v[2] = fminf(v[2], lo.z);
    v[3] = fminf(v[3], c.x);  v[4] = fminf(v[4], c.y);  v[5] = fminf(v[5], c.z);
    v[6] = fmaxf(v[6], hi.x); v[7] = fmaxf(v[7], hi.y); v[8] = fmaxf(v[8], hi.z);
    v[9] = fmaxf(v[9], c.x);  v[10] = fmaxf(v[10], c.y); v[11] = fmaxf(v[11], c.z);
  }
  for (int k = 0; k < 6; ++k) { v[k] = warp_min(v[k]); v[6 + k] = warp_max(v[6 + k]); }
  if (lane == 0)
    for (int k = 0; k < 12; ++k) red[k][warp] = v[k];
  __syncthreads();
  if (tid < 12) {
    float r = red[tid][0];
    for (int w = 1; w < BUILD_THREADS / 32; ++w) r = tid < 6 ? fminf(r, red[tid][w]) : fmaxf(r, red[tid][w]);
    box[tid] = r;
  }
  __syncthreads();
  // box[0..2] lo, [3..5] centroid lo, [6..8] hi, [9..11] centroid hi
  if (tid == 0) {
    BuildNode& nd = nodes[t.node];
    nd.lo[0] = box[0]; nd.lo[1] = box[1]; nd.lo[2] = box[2];
    nd.hi[0] = box[6]; nd.hi[1] = box[7]; nd.hi[2] = box[8];
  }
  const float clo[3] = {box[3], box[4], box[5]};
  const float cext[3] = {box[9] - box[3], box[10] - box[4], box[11] - box[5]};

  bool leaf = t.count <= 2;
  int best = -1;
  if (!leaf) {
    // 2. bins
    for (int k = tid; k < 3 * NB; k += BUILD_THREADS) {
      int a = k / NB, b = k % NB;
      bcnt[a][b] = 0;
      for (int c = 0; c < 3; ++c) { bmin[a][b][c] = f2o(1e30f); bmax[a][b][c] = f2o(-1e30f); }
    }
    __syncthreads();
    for (uint32_t i = t.start + tid; i < end; i += BUILD_THREADS) {
      uint32_t id = src[i];
      float4 c = tc[id], lo = tlo[id], hi = thi[id];
      const float cc[3] = {c.x, c.y, c.z};
      const int ilo[3] = {f2o(lo.x), f2o(lo.y), f2o(lo.z)};
      const int ihi[3] = {f2o(hi.x), f2o(hi.y), f2o(hi.z)};
      for (int a = 0; a < 3; ++a) {
        if (!(cext[a] > 0.0f)) continue;
        int b = min(NB - 1, max(0, (int)((cc[a] - clo[a]) * ((float)NB / cext[a]))));
        atomicAdd(&bcnt[a][b], 1);
        for (int k = 0; k < 3; ++k) {
          atomicMin(&bmin[a][b][k], ilo[k]);
          atomicMax(&bmax[a][b][k], ihi[k]);
        }
      }
    }
    __syncthreads();
    // 3. SAH cost of every plane
    if (tid < 3 * (NB - 1)) {
      int a = tid / (NB - 1), s = tid % (NB - 1);
      float cost = 3.0e38f;
      if (cext[a] > 0.0f) {
        float l[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f}, r[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f};
        int nl = 0, nr = 0;
        for (int b = 0; b < NB; ++b) {
          float* dstb = b <= s ? l : r;
          int cnt = bcnt[a][b];
          if (cnt == 0) continue;
          if (b <= s) nl += cnt; else nr += cnt;
          for (int k = 0; k < 3; ++k) {
            dstb[k] = fminf(dstb[k], o2f(bmin[a][b][k]));
            dstb[3 + k] = fmaxf(dstb[3 + k], o2f(bmax[a][b][k]));
          }
        }
        if (nl > 0 && nr > 0)
          cost = box_area(l[0], l[1], l[2], l[3], l[4], l[5]) * nl + box_area(r[0], r[1], r[2], r[3], r[4], r[5]) * nr;
      }
      cost_s[tid] = cost;
    }
    __syncthreads();
    if (tid == 0) {
      int bi = -1;
      float bc = 3.0e38f;
      for (int k = 0; k < 3 * (NB - 1); ++k)
        if (cost_s[k] < bc) { bc = cost_s[k]; bi = k; }
      float area = box_area(box[0], box[1], box[2], box[6], box[7], box[8]);
      if (bi < 0) {
        best_s = (t.count <= (uint32_t)LEAF_MAX) ? -2 : -1;  // -2 leaf, -1 median split
      } else if (t.count <= (uint32_t)SAH_LEAF_MAX && area * t.count <= bc + SAH_NODE_COST * area) {
        best_s = -2;
      } else {
        best_s = bi;
      }
    }
    __syncthreads();
    best = best_s;
    leaf = best == -2;
  }

  if (leaf) {
    for (uint32_t i = t.start + tid; i < end; i += BUILD_THREADS) final_ids[i] = src[i];
    if (tid == 0) {
      BuildNode& nd = nodes[t.node];
      nd.left = -1;
      nd.right = -1;
      nd.start = t.start;
      nd.count = t.count;
    }
    return;
  }

  // 4. stable partition into dst
  uint32_t nleft;
  if (best < 0) {
    nleft = t.count / 2;
    for (uint32_t i = t.start + tid; i < end; i += BUILD_THREADS) dst[i] = src[i];
  } else {
    const int a = best / (NB - 1), s = best % (NB - 1);
    nleft = 0;
    for (int b = 0; b <= s; ++b) nleft += (uint32_t)bcnt[a][b];
    const float scale = (float)NB / cext[a];
    uint32_t lbase = 0, rbase = 0;
    for (uint32_t base = t.start; base < end; base += BUILD_THREADS) {
      uint32_t i = base + tid;
      bool valid = i < end;
      uint32_t id = valid ? src[i] : 0u;
      bool left = false;
      if (valid) {
        float4 c = tc[id];
        float cc = a == 0 ? c.x : (a == 1 ? c.y : c.z);
        int b = min(NB - 1, max(0, (int)((cc - clo[a]) * scale)));
        left = b <= s;
      }
      unsigned m = __ballot_sync(0xffffffffu, left);
      unsigned mv = __ballot_sync(0xffffffffu, valid);
      if (lane == 0) wcount[warp] = __popc(m);
      __syncthreads();
      uint32_t wl = 0, total_l = 0;
      for (int w = 0; w < BUILD_THREADS / 32; ++w) {
        if (w < warp) wl += wcount[w];
        total_l += wcount[w];
      }
      uint32_t chunk = min((uint32_t)BUILD_THREADS, end - base);
      uint32_t rank_l = wl + __popc(m & ((1u << lane) - 1u));
      uint32_t before = (uint32_t)(warp * 32) + __popc(mv & ((1u << lane) - 1u));
      if (valid) {
        if (left) dst[t.start + lbase + rank_l] = id;
        else dst[t.start + nleft + rbase + (before - rank_l)] = id;
      }
      lbase += total_l;
      rbase += chunk - total_l;
      __syncthreads();
    }
  }
  if (tid == 0) {
    uint32_t c = atomicAdd(node_counter, 2u);
    BuildNode& nd = nodes[t.node];
    nd.left = (int32_t)c;
    nd.right = (int32_t)(c + 1);
    nd.start = 0;
    nd.count = 0;
    push_children(c, t, nleft, next);
  }
}

// ---------------------------------------------------------------------------
// Whole subtrees. The deep levels of a big scene hold hundreds of thousands
// of tasks of a few triangles, and one block per task per level leaves most
// of each block idle. A task of at most SUBTREE_MAX triangles is therefore
// built down to its leaves by one warp, with the same bounds, bins, SAH
// costs, leaf rule and stable partition as k_level, so the tree is the same.
// The warp first copies its triangles' boxes and centroids into shared
// memory; inside the subtree it permutes 16-bit local indices, and only the
// leaves go back to the global ids. It continues with the smaller child and
// keeps the larger one on a short stack: every stacked task is at least as
// large as the current one, so the stack holds at most log2(SUBTREE_MAX)
// entries, and a subtree of c triangles has fewer than 2c nodes, which
// bounds the loop.
constexpr uint32_t SUBTREE_MAX = 128;
constexpr int SUB_WARPS = 8;
constexpr int SUB_STACK = 16;

// Shared memory of one warp of k_subtree.
struct SubtreeSmem {
  float lx[SUBTREE_MAX], ly[SUBTREE_MAX], lz[SUBTREE_MAX];
  float hx[SUBTREE_MAX], hy[SUBTREE_MAX], hz[SUBTREE_MAX];
  float cx[SUBTREE_MAX], cy[SUBTREE_MAX], cz[SUBTREE_MAX];
  uint32_t gid[SUBTREE_MAX];
  uint16_t lid[2][SUBTREE_MAX];
  int bcnt[3][NB];
  int bmin[3][NB][3];
  int bmax[3][NB][3];
  BuildTask stack[SUB_STACK];
};
constexpr size_t SUBTREE_SMEM = SUB_WARPS * sizeof(SubtreeSmem);

// The SAH costs of all 3 x (NB - 1) planes of one task from its bins by
// segmented scans over NB lanes: with 16 bins lanes 0-15 hold the bins of one
// axis and lanes 16-31 of the next (axes 0 and 1, then axis 2); with 32 bins
// one axis per pass. (32 bins measured the same render speed and a 13-21%
// slower build, so NB stays 16.) Each lane's inclusive prefix is the left side
// of its plane and its right neighbour's inclusive suffix the right side.
// min/max are exact and an empty bin holds the identity box, so the sides,
// counts and costs equal k_level's per-plane loops bit for bit. Returns the
// lane's cheapest plane (strictly lower cost wins, so ties keep the lower
// plane index).
__device__ __forceinline__ void sah_scan(const SubtreeSmem& S, const float cext[3], int lane, float& bc, int& bi) {
  const unsigned FULL = 0xffffffffu;
  bc = 3.0e38f;
  bi = -1;
  static_assert(NB == 16 || NB == 32, "segmented scans over 16 or 32 lanes");
  constexpr int AX_PER_PASS = 32 / NB;  // axes scanned at once
  constexpr int PASSES = (3 + AX_PER_PASS - 1) / AX_PER_PASS;
  const int half = lane / NB, b = lane % NB;
  for (int pass = 0; pass < PASSES; ++pass) {
    const int a = AX_PER_PASS * pass + half;
    const bool act = a < 3;
    int cnt = 0;
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    if (act) {
      cnt = S.bcnt[a][b];
      for (int q = 0; q < 3; ++q) {
        mn[q] = o2f(S.bmin[a][b][q]);
        mx[q] = o2f(S.bmax[a][b][q]);
      }
    }
    int pc = cnt, sc = cnt;
    float pmn[3] = {mn[0], mn[1], mn[2]}, pmx[3] = {mx[0], mx[1], mx[2]};
    float smn[3] = {mn[0], mn[1], mn[2]}, smx[3] = {mx[0], mx[1], mx[2]};
    for (int o = 1; o < NB; o <<= 1) {
      const int c_up = __shfl_up_sync(FULL, pc, o, NB), c_dn = __shfl_down_sync(FULL, sc, o, NB);
      float u_mn[3], u_mx[3], d_mn[3], d_mx[3];
      for (int q = 0; q < 3; ++q) {
        u_mn[q] = __shfl_up_sync(FULL, pmn[q], o, NB);
        u_mx[q] = __shfl_up_sync(FULL, pmx[q], o, NB);
        d_mn[q] = __shfl_down_sync(FULL, smn[q], o, NB);
        d_mx[q] = __shfl_down_sync(FULL, smx[q], o, NB);
      }
      if (b >= o) {
        pc += c_up;
        for (int q = 0; q < 3; ++q) { pmn[q] = fminf(pmn[q], u_mn[q]); pmx[q] = fmaxf(pmx[q], u_mx[q]); }
      }
      if (b + o < NB) {
        sc += c_dn;
        for (int q = 0; q < 3; ++q) { smn[q] = fminf(smn[q], d_mn[q]); smx[q] = fmaxf(smx[q], d_mx[q]); }
      }
    }
    const int rc = __shfl_down_sync(FULL, sc, 1, NB);
    float rmn[3], rmx[3];
    for (int q = 0; q < 3; ++q) {
      rmn[q] = __shfl_down_sync(FULL, smn[q], 1, NB);
      rmx[q] = __shfl_down_sync(FULL, smx[q], 1, NB);
    }
    if (act && b < NB - 1 && cext[a] > 0.0f && pc > 0 && rc > 0) {
      const float cost = box_area(pmn[0], pmn[1], pmn[2], pmx[0], pmx[1], pmx[2]) * pc +
                         box_area(rmn[0], rmn[1], rmn[2], rmx[0], rmx[1], rmx[2]) * rc;
      if (cost < bc) {
        bc = cost;
        bi = a * (NB - 1) + b;
      }
    }
  }
}

__global__ void __launch_bounds__(SUB_WARPS * 32) k_subtree(const BuildTask* tasks, const uint32_t* ntasks_ptr,
                                                            uint32_t cap, const uint32_t* ids_a,
                                                            const uint32_t* ids_b, uint32_t* final_ids,
                                                            const float4* tlo, const float4* thi, const float4* tc,
                                                            BuildNode* nodes, uint32_t* node_counter,
                                                            uint32_t* error_flag) {
  extern __shared__ __align__(16) unsigned char sub_smem[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t ti = blockIdx.x * SUB_WARPS + w;
  if (ti >= min(*ntasks_ptr, cap)) return;  // warp-uniform
  SubtreeSmem& S = reinterpret_cast<SubtreeSmem*>(sub_smem)[w];
  const BuildTask root = tasks[ti];
  if (root.count > SUBTREE_MAX) {  // never pushed (see ChildLists); reported, not built
    if (lane == 0) atomicExch(error_flag, 3u);
    return;
  }
  {
    const uint32_t* src = root.pad ? ids_b : ids_a;
    for (uint32_t k = lane; k < root.count; k += 32) {
      const uint32_t id = src[root.start + k];
      const float4 lo = tlo[id], hi = thi[id], c = tc[id];
      S.lx[k] = lo.x; S.ly[k] = lo.y; S.lz[k] = lo.z;
      S.hx[k] = hi.x; S.hy[k] = hi.y; S.hz[k] = hi.z;
      S.cx[k] = c.x;  S.cy[k] = c.y;  S.cz[k] = c.z;
      S.gid[k] = id;
      S.lid[0][k] = (uint16_t)k;
    }
  }
  __syncwarp();
  // The subtree's nodes come from one reservation: its splits number at most
  // count - 1, two nodes each. Unused slots are marked as leaves at the end
  // so that the layout pass reads only valid links.
  const uint32_t reserved = 2u * (root.count - 1u);
  uint32_t nbase = 0, used = 0;
  if (lane == 0 && reserved > 0) nbase = atomicAdd(node_counter, reserved);
  nbase = __shfl_sync(FULL, nbase, 0);
  // tasks below use start relative to the subtree and pad = local buffer
  BuildTask t{root.node, 0u, root.count, 0u};
  int sp = 0;
  for (uint32_t iter = 0; iter < 2 * SUBTREE_MAX; ++iter) {
    const uint16_t* src = S.lid[t.pad];
    uint16_t* dst = S.lid[t.pad ^ 1u];
    const uint32_t end = t.start + t.count;
    // 1. box and centroid box (every value below is uniform over the warp)
    float v[12];
    for (int k = 0; k < 6; ++k) { v[k] = 1e30f; v[6 + k] = -1e30f; }
    for (uint32_t i = t.start + lane; i < end; i += 32) {
      const uint32_t j = src[i];
      v[0] = fminf(v[0], S.lx[j]); v[1] = fminf(v[1], S.ly[j]); v[2] = fminf(v[2], S.lz[j]);
      v[3] = fminf(v[3], S.cx[j]); v[4] = fminf(v[4], S.cy[j]); v[5] = fminf(v[5], S.cz[j]);
      v[6] = fmaxf(v[6], S.hx[j]); v[7] = fmaxf(v[7], S.hy[j]); v[8] = fmaxf(v[8], S.hz[j]);
      v[9] = fmaxf(v[9], S.cx[j]); v[10] = fmaxf(v[10], S.cy[j]); v[11] = fmaxf(v[11], S.cz[j]);
    }
    for (int k = 0; k < 6; ++k) { v[k] = warp_min(v[k]); v[6 + k] = warp_max(v[6 + k]); }
    BuildNode& nd = nodes[t.node];
    if (lane == 0) {
      nd.lo[0] = v[0]; nd.lo[1] = v[1]; nd.lo[2] = v[2];
      nd.hi[0] = v[6]; nd.hi[1] = v[7]; nd.hi[2] = v[8];
    }
    const float clo[3] = {v[3], v[4], v[5]};
    const float cext[3] = {v[9] - v[3], v[10] - v[4], v[11] - v[5]};
    bool leaf = t.count <= 2;
    int best = -1;
    if (!leaf) {
      // 2. bins
      for (int k = lane; k < 3 * NB; k += 32) {
        int a = k / NB, b = k % NB;
        S.bcnt[a][b] = 0;
        for (int c = 0; c < 3; ++c) { S.bmin[a][b][c] = f2o(1e30f); S.bmax[a][b][c] = f2o(-1e30f); }
      }
      __syncwarp();
      for (uint32_t i = t.start + lane; i < end; i += 32) {
        const uint32_t j = src[i];
        const float cc[3] = {S.cx[j], S.cy[j], S.cz[j]};
        const int ilo[3] = {f2o(S.lx[j]), f2o(S.ly[j]), f2o(S.lz[j])};
        const int ihi[3] = {f2o(S.hx[j]), f2o(S.hy[j]), f2o(S.hz[j])};
        for (int a = 0; a < 3; ++a) {
          if (!(cext[a] > 0.0f)) continue;
          int b = min(NB - 1, max(0, (int)((cc[a] - clo[a]) * ((float)NB / cext[a]))));
          atomicAdd(&S.bcnt[a][b], 1);
          for (int k = 0; k < 3; ++k) {
            atomicMin(&S.bmin[a][b][k], ilo[k]);
            atomicMax(&S.bmax[a][b][k], ihi[k]);
          }
        }
      }
      __syncwarp();
      // 3. SAH cost of every plane (lane k: planes k and k + 32), then the
      // cheapest, ties to the lower plane index as k_level scans them
      float bc;
      int bi;
      sah_scan(S, cext, lane, bc, bi);
      for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(FULL, bc, o);
        const int oi = __shfl_xor_sync(FULL, bi, o);
        if (oi >= 0 && (oc < bc || (oc == bc && (bi < 0 || oi < bi)))) { bc = oc; bi = oi; }
      }
      const float area = box_area(v[0], v[1], v[2], v[6], v[7], v[8]);
      if (bi < 0) best = (t.count <= (uint32_t)LEAF_MAX) ? -2 : -1;  // -2 leaf, -1 median split
      else if (t.count <= (uint32_t)SAH_LEAF_MAX && area * t.count <= bc + SAH_NODE_COST * area) best = -2;
      else best = bi;
      leaf = best == -2;
    }
    if (!leaf) {
      // 4. stable partition into the other local buffer
      uint32_t nleft;
      if (best < 0) {
        nleft = t.count / 2;
        for (uint32_t i = t.start + lane; i < end; i += 32) dst[i] = src[i];
      } else {
        const int a = best / (NB - 1), s = best % (NB - 1);
        nleft = 0;
        for (int b = 0; b <= s; ++b) nleft += (uint32_t)S.bcnt[a][b];
        const float scale = (float)NB / cext[a];
        const float* ca = a == 0 ? S.cx : (a == 1 ? S.cy : S.cz);
        const unsigned lt = (1u << lane) - 1u;
        uint32_t lbase = 0, rbase = 0;
        for (uint32_t base = t.start; base < end; base += 32) {
          const uint32_t i = base + lane;
          const bool valid = i < end;
          const uint16_t j = valid ? src[i] : (uint16_t)0;
          bool left = false;
          if (valid) {
            int b = min(NB - 1, max(0, (int)((ca[j] - clo[a]) * scale)));
            left = b <= s;
          }
          const unsigned m = __ballot_sync(FULL, left), mv = __ballot_sync(FULL, valid);
          if (valid) {
            if (left) dst[t.start + lbase + __popc(m & lt)] = j;
            else dst[t.start + nleft + rbase + __popc(mv & ~m & lt)] = j;
          }
          lbase += __popc(m);
          rbase += __popc(mv & ~m);
        }
      }
      if (used + 2 > reserved) {  // cannot happen (see above); reported, never written out of bounds
        if (lane == 0) atomicExch(error_flag, 4u);
        return;
      }
      const uint32_t c = nbase + used;
      used += 2;
      if (lane == 0) {
        nd.left = (int32_t)c;
        nd.right = (int32_t)(c + 1);
        nd.start = 0;
        nd.count = 0;
      }
      const BuildTask L{c, t.start, nleft, t.pad ^ 1u};
      const BuildTask R{c + 1, t.start + nleft, t.count - nleft, t.pad ^ 1u};
      const bool go_left = L.count <= R.count;
      if (sp >= SUB_STACK) {  // cannot happen (see above); reported, never written out of bounds
        if (lane == 0) atomicExch(error_flag, 1u);
        return;
      }
      __syncwarp();
      if (lane == 0) S.stack[sp] = go_left ? R : L;
      __syncwarp();
      ++sp;
      t = go_left ? L : R;
      continue;
    }
    for (uint32_t i = t.start + lane; i < end; i += 32) final_ids[root.start + i] = S.gid[src[i]];
    if (lane == 0) {
      nd.left = -1;
      nd.right = -1;
      nd.start = root.start + t.start;
      nd.count = t.count;
    }
    if (sp == 0) {
      for (uint32_t k = used + lane; k < reserved; k += 32) {
        nodes[nbase + k].left = -1;
        nodes[nbase + k].count = 0;
      }
      return;
    }
    --sp;
    t = S.stack[sp];
    __syncwarp();
  }
  if (lane == 0) atomicExch(error_flag, 2u);  // loop bound reached: cannot happen for a well-formed task
}

// ---------------------------------------------------------------------------
// Large tasks (the top levels of big scenes): one task would keep a single
// block busy for millions of triangles while the rest of the GPU idles, so
// tasks above LARGE_TASK triangles are split over blocks of CHUNK triangles:
// bounds and bins are merged into per-task state with order-preserving
// integer atomics, one thread per task picks the plane, and the stable
// partition uses per-chunk left counts (each chunk sums the counts of the
// chunks before it).
constexpr uint32_t LARGE_TASK = 1u << 13;
constexpr uint32_t CHUNK = 4096;
constexpr uint32_t MAX_LARGE = MAX_LARGE_TASKS;

struct LargeState {
  int box[12];  // lo xyz, centroid lo xyz, hi xyz, centroid hi xyz (ordered ints)
  int bcnt[3][NB];
  int bmin[3][NB][3];
  int bmax[3][NB][3];
  int best;        // plane a * (NB - 1) + s, or -1 for a median split
  uint32_t nleft;
};

// Block -> (large task, chunk) through the per-task first-chunk prefix.
__device__ __forceinline__ uint32_t chunk_task(const uint32_t* first_chunk, uint32_t nlarge, uint32_t block) {
  uint32_t lo = 0, hi = nlarge;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) / 2;
    if (first_chunk[mid] <= block) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void k_large_init(LargeState* st, uint32_t nlarge) {
  LargeState& S = st[blockIdx.x];
  for (int k = threadIdx.x; k < 12; k += blockDim.x) S.box[k] = f2o(k < 6 ? 1e30f : -1e30f);
  for (int k = threadIdx.x; k < 3 * NB; k += blockDim.x) {
    int a = k / NB, b = k % NB;
    S.bcnt[a][b] = 0;
    for (int c = 0; c < 3; ++c) {
      S.bmin[a][b][c] = f2o(1e30f);
      S.bmax[a][b][c] = f2o(-1e30f);
    }
  }
}

__global__ void __launch_bounds__(BUILD_THREADS) k_large_bounds(const BuildTask* large, const uint32_t* first_chunk,
                                                                uint32_t nlarge, const uint32_t* src,
                                                                const float4* tlo, const float4* thi,
                                                                const float4* tc, LargeState* st) {
  __shared__ float red[12][BUILD_THREADS / 32];
  const uint32_t j = chunk_task(first_chunk, nlarge, blockIdx.x);
  const BuildTask t = large[j];
  const uint32_t b0 = t.start + (blockIdx.x - first_chunk[j]) * CHUNK;
  const uint32_t b1 = min(t.start + t.count, b0 + CHUNK);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float v[12];
  for (int k = 0; k < 6; ++k) { v[k] = 1e30f; v[6 + k] = -1e30f; }
  for (uint32_t i = b0 + tid; i < b1; i += BUILD_THREADS) {
    uint32_t id = src[i];
    float4 lo = tlo[id], hi = thi[id], c = tc[id];
    v[0] = fminf(v[0], lo.x); v[1] = fminf(v[1], lo.y); v[2] = fminf(v[2], lo.z);
    v[3] = fminf(v[3], c.x);  v[4] = fminf(v[4], c.y);  v[5] = fminf(v[5], c.z);
    v[6] = fmaxf(v[6], hi.x); v[7] = fmaxf(v[7], hi.y); v[8] = fmaxf(v[8], hi.z);
    v[9] = fmaxf(v[9], c.x);  v[10] = fmaxf(v[10], c.y); v[11] = fmaxf(v[11], c.z);
  }
  for (int k = 0; k < 6; ++k) { v[k] = warp_min(v[k]); v[6 + k] = warp_max(v[6 + k]); }
  if (lane == 0)
    for (int k = 0; k < 12; ++k) red[k][warp] = v[k];
  __syncthreads();
  if (tid < 12) {
    float r = red[tid][0];
    for (int w = 1; w < BUILD_THREADS / 32; ++w) r = tid < 6 ? fminf(r, red[tid][w]) : fmaxf(r, red[tid][w]);
    if (tid < 6) atomicMin(&st[j].box[tid], f2o(r));
    else atomicMax(&st[j].box[tid], f2o(r));
  }
}

__global__ void __launch_bounds__(BUILD_THREADS) k_large_bin(const BuildTask* large, const uint32_t* first_chunk,
                                                             uint32_t nlarge, const uint32_t* src,
                                                             const float4* tlo, const float4* thi,
                                                             const float4* tc, LargeState* st) {
  __shared__ int bcnt[3][NB];
  __shared__ int bmin[3][NB][3];
  __shared__ int bmax[3][NB][3];
  const uint32_t j = chunk_task(first_chunk, nlarge, blockIdx.x);
  const BuildTask t = large[j];
  const uint32_t b0 = t.start + (blockIdx.x - first_chunk[j]) * CHUNK;
  const uint32_t b1 = min(t.start + t.count, b0 + CHUNK);
  const int tid = threadIdx.x;
  float clo[3], cext[3];
  for (int a = 0; a < 3; ++a) {
    clo[a] = o2f(st[j].box[3 + a]);
    cext[a] = o2f(st[j].box[9 + a]) - clo[a];
  }
  for (int k = tid; k < 3 * NB; k += BUILD_THREADS) {
    int a = k / NB, b = k % NB;
    bcnt[a][b] = 0;
    for (int c = 0; c < 3; ++c) { bmin[a][b][c] = f2o(1e30f); bmax[a][b][c] = f2o(-1e30f); }
  }
  __syncthreads();
  for (uint32_t base = b0; base < b1; base += BUILD_THREADS) {
    const uint32_t i = base + tid;
    const bool valid = i < b1;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f), lo = c, hi = c;
    if (valid) {
      const uint32_t id = src[i];
      c = tc[id];
      lo = tlo[id];
      hi = thi[id];
    }
    bin_warp(valid, c, lo, hi, clo, cext, bcnt, bmin, bmax);
  }
  __syncthreads();
  for (int k = tid; k < 3 * NB; k += BUILD_THREADS) {
    int a = k / NB, b = k % NB;
    if (bcnt[a][b] == 0) continue;
    atomicAdd(&st[j].bcnt[a][b], bcnt[a][b]);
    for (int c = 0; c < 3; ++c) {
      atomicMin(&st[j].bmin[a][b][c], bmin[a][b][c]);
      atomicMax(&st[j].bmax[a][b][c], bmax[a][b][c]);
    }
  }
}

// One warp per large task: SAH over the merged bins (the same costs as
// k_level; lane k prices planes k and k + 32, the cheapest wins with ties to
// the lower plane index), node box, children.
__global__ void k_large_split(const BuildTask* large, uint32_t nlarge, LargeState* st, BuildNode* nodes,
                              uint32_t* node_counter, ChildLists next) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= nlarge) return;  // warp-uniform
  const BuildTask t = large[j];
  LargeState& S = st[j];
  float box[12];
  for (int k = 0; k < 12; ++k) box[k] = o2f(S.box[k]);
  BuildNode& nd = nodes[t.node];
  float bc = 3.0e38f;
  int bi = -1;
  for (int k = lane; k < 3 * (NB - 1); k += 32) {
    const int a = k / (NB - 1), s = k % (NB - 1);
    if (!(box[9 + a] - box[3 + a] > 0.0f)) continue;
    float l[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f}, r[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f};
    int nl = 0, nr = 0;
    for (int b = 0; b < NB; ++b) {
      int cnt = S.bcnt[a][b];
      if (cnt == 0) continue;
      const bool lb = b <= s;
      if (lb) nl += cnt; else nr += cnt;
      for (int q = 0; q < 3; ++q) {
        const float mn = o2f(S.bmin[a][b][q]), mx = o2f(S.bmax[a][b][q]);
        if (lb) { l[q] = fminf(l[q], mn); l[3 + q] = fmaxf(l[3 + q], mx); }
        else { r[q] = fminf(r[q], mn); r[3 + q] = fmaxf(r[3 + q], mx); }
      }
    }
    if (nl > 0 && nr > 0) {
      float cost = box_area(l[0], l[1], l[2], l[3], l[4], l[5]) * nl + box_area(r[0], r[1], r[2], r[3], r[4], r[5]) * nr;
      if (cost < bc) { bc = cost; bi = k; }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float oc = __shfl_xor_sync(FULL, bc, o);
    const int oi = __shfl_xor_sync(FULL, bi, o);
    if (oi >= 0 && (oc < bc || (oc == bc && (bi < 0 || oi < bi)))) { bc = oc; bi = oi; }
  }
  if (lane != 0) return;
  nd.lo[0] = box[0]; nd.lo[1] = box[1]; nd.lo[2] = box[2];
  nd.hi[0] = box[6]; nd.hi[1] = box[7]; nd.hi[2] = box[8];
  uint32_t nleft = t.count / 2;  // median split when no plane separates the centroids
  if (bi >= 0) {
    const int a = bi / (NB - 1), s = bi % (NB - 1);
    nleft = 0;
    for (int b = 0; b <= s; ++b) nleft += (uint32_t)S.bcnt[a][b];
  }
  S.best = bi;
  S.nleft = nleft;
  uint32_t c = atomicAdd(node_counter, 2u);
  nd.left = (int32_t)c;
  nd.right = (int32_t)(c + 1);
  nd.start = 0;
  nd.count = 0;
  push_children(c, t, nleft, next);
}

__device__ __forceinline__ bool large_goes_left(const LargeState& S, float4 c, int a, int s) {
  const float clo = o2f(S.box[3 + a]);
  const float cext = o2f(S.box[9 + a]) - clo;
  const float cc = a == 0 ? c.x : (a == 1 ? c.y : c.z);
  const int b = min(NB - 1, max(0, (int)((cc - clo) * ((float)NB / cext))));
  return b <= s;
}

__global__ void __launch_bounds__(BUILD_THREADS) k_large_count(const BuildTask* large, const uint32_t* first_chunk,
                                                               uint32_t nlarge, const uint32_t* src,
                                                               const float4* tc, const LargeState* st,
                                                               uint32_t* chunk_left) {
  __shared__ uint32_t wsum[BUILD_THREADS / 32];
  const uint32_t j = chunk_task(first_chunk, nlarge, blockIdx.x);
  const BuildTask t = large[j];
  const LargeState& S = st[j];
  const uint32_t b0 = t.start + (blockIdx.x - first_chunk[j]) * CHUNK;
  const uint32_t b1 = min(t.start + t.count, b0 + CHUNK);
  uint32_t n = 0;
  if (S.best >= 0) {
    const int a = S.best / (NB - 1), s = S.best % (NB - 1);
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += BUILD_THREADS) n += large_goes_left(S, tc[src[i]], a, s);
  } else {
    // median split: the first nleft positions of the task go left
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += BUILD_THREADS) n += (i - t.start) < S.nleft;
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < BUILD_THREADS / 32; ++w) tot += wsum[w];
    chunk_left[blockIdx.x] = tot;
  }
}

__global__ void __launch_bounds__(BUILD_THREADS) k_large_scatter(const BuildTask* large, const uint32_t* first_chunk,
                                                                 uint32_t nlarge, const uint32_t* src, uint32_t* dst,
                                                                 const float4* tc, const LargeState* st,
                                                                 const uint32_t* chunk_left) {
  __shared__ uint32_t wcount[BUILD_THREADS / 32];
  __shared__ uint32_t base_s;
  const uint32_t j = chunk_task(first_chunk, nlarge, blockIdx.x);
  const BuildTask t = large[j];
  const LargeState& S = st[j];
  const uint32_t b0 = t.start + (blockIdx.x - first_chunk[j]) * CHUNK;
  const uint32_t b1 = min(t.start + t.count, b0 + CHUNK);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    uint32_t l = 0;
    for (uint32_t c = first_chunk[j]; c < blockIdx.x; ++c) l += chunk_left[c];
    base_s = l;
  }
  __syncthreads();
  uint32_t lbase = base_s;                    // left elements before this position
  uint32_t rbase = (b0 - t.start) - base_s;   // right elements before this position
  const int a = S.best >= 0 ? S.best / (NB - 1) : 0, s = S.best >= 0 ? S.best % (NB - 1) : 0;
  for (uint32_t base = b0; base < b1; base += BUILD_THREADS) {
    const uint32_t i = base + tid;
    const bool valid = i < b1;
    const uint32_t id = valid ? src[i] : 0u;
    bool left = false;
    if (valid) left = S.best >= 0 ? large_goes_left(S, tc[id], a, s) : (i - t.start) < S.nleft;
    const unsigned m = __ballot_sync(0xffffffffu, left);
    const unsigned mv = __ballot_sync(0xffffffffu, valid);
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    uint32_t wl = 0, total_l = 0;
    for (int w = 0; w < BUILD_THREADS / 32; ++w) {
      if (w < warp) wl += wcount[w];
      total_l += wcount[w];
    }
    const uint32_t chunk = min((uint32_t)BUILD_THREADS, b1 - base);
    const uint32_t rank_l = wl + __popc(m & ((1u << lane) - 1u));
    const uint32_t before = (uint32_t)(warp * 32) + __popc(mv & ((1u << lane) - 1u));
    if (valid) {
      if (left) dst[t.start + lbase + rank_l] = id;
      else dst[t.start + S.nleft + rbase + (before - rank_l)] = id;
    }
    lbase += total_l;
    rbase += chunk - total_l;
    __syncthreads();
  }
}

__global__ void k_layout(const BuildNode* nodes, uint32_t nnodes, float4* trav) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnodes) return;
  const BuildNode nd = nodes[i];
  if (nd.left < 0) {
    if (i == 0) {  // the whole scene is one leaf: wrap it under an internal root
      trav[0] = make_float4(nd.lo[0], nd.hi[0], nd.lo[1], nd.hi[1]);
      trav[1] = make_float4(1e30f, 1e30f, 1e30f, 1e30f);
      trav[2] = make_float4(nd.lo[2], nd.hi[2], 1e30f, 1e30f);
      trav[3] = make_float4(__int_as_float(make_leaf_link(nd.start, nd.count)),
                            __int_as_float(make_leaf_link(0, 0)), 0.0f, 0.0f);
    }
    return;
  }
  const BuildNode L = nodes[nd.left], R = nodes[nd.right];
  int32_t l0 = L.left < 0 ? make_leaf_link(L.start, L.count) : nd.left;
  int32_t l1 = R.left < 0 ? make_leaf_link(R.start, R.count) : nd.right;
  trav[4 * i] = make_float4(L.lo[0], L.hi[0], L.lo[1], L.hi[1]);
  trav[4 * i + 1] = make_float4(R.lo[0], R.hi[0], R.lo[1], R.hi[1]);
  trav[4 * i + 2] = make_float4(L.lo[2], L.hi[2], R.lo[2], R.hi[2]);
  trav[4 * i + 3] = make_float4(__int_as_float(l0), __int_as_float(l1), 0.0f, 0.0f);
}

__global__ void k_reorder(const uint32_t* final_ids, uint32_t n, const float4* v0, const float4* e1, const float4* e2,
                          float4* out) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint32_t id = final_ids[s];
  float4 a = v0[id];
  a.w = __uint_as_float(id);
  out[3 * s] = a;
  out[3 * s + 1] = e1[id];
  out[3 * s + 2] = e2[id];
}

// Build scratch from the stream-ordered allocator of the build stream: no
// allocation or free here waits for work on other streams.
// ---------------------------------------------------------------------------
// Collapse of the binary BVH into the wide traversal layout (pt_types.h):
// each wide node takes a binary node's two children and keeps replacing
// its internal child of largest surface area by that child's two children
// until it has BVH_WIDTH. One launch per level of the wide tree (the host
// reads the remaining work once per eight levels).
struct CollapseWork {
  int32_t bin;  // binary node
  int32_t out;  // its wide node
};

__device__ __forceinline__ float bin_child_area(const float4* bin, int32_t node, int c) {
  const float4* nd = bin + 4 * node;
  float4 a = nd[c], z = nd[2];
  float lz = c ? z.z : z.x, hz = c ? z.w : z.y;
  return box_area(a.x, a.z, lz, a.y, a.w, hz);
}

// One wide node: binary node w.bin's children, opening the largest-area
// internal child until there are BVH_WIDTH; internal children are queued
// for the next level.
__device__ __forceinline__ void collapse_one(const float4* bin, const CollapseWork w, float4* out4,
                                             uint32_t* node_counter, uint32_t cap4, CollapseWork* next,
                                             uint32_t* next_count, uint32_t* overflow, uint32_t* leaves) {
  float lo[BVH_WIDTH][3], hi[BVH_WIDTH][3], area[BVH_WIDTH];
  int32_t link[BVH_WIDTH];
  int n = 0;
  // child c of binary node `node` into slot k
  auto load = [&](int32_t node, int c, int k) {
    const float4* nd = bin + 4 * node;
    float4 a = nd[c], z = nd[2];
    int4 l = *reinterpret_cast<const int4*>(nd + 3);
    lo[k][0] = a.x;
    hi[k][0] = a.y;
    lo[k][1] = a.z;
    hi[k][1] = a.w;
    lo[k][2] = c ? z.z : z.x;
    hi[k][2] = c ? z.w : z.y;
    link[k] = c ? l.y : l.x;
    area[k] = bin_child_area(bin, node, c);
  };
  load(w.bin, 0, 0);
  load(w.bin, 1, 1);
  n = 2;
  while (n < BVH_WIDTH) {
    int best = -1;
    float ba = -1.0f;
    for (int k = 0; k < n; ++k)
      if (link[k] >= 0 && area[k] > ba) {
        ba = area[k];
        best = k;
      }
    if (best < 0) break;
    const int32_t node = link[best];
    load(node, 1, n);     // second child appended (n < BVH_WIDTH here)
    load(node, 0, best);  // first child replaces its parent
    ++n;
  }
  float4* o = out4 + NODE_F4 * (size_t)w.out;
  float q[6][BVH_WIDTH];
  int32_t ol[BVH_WIDTH];
  for (int k = 0; k < BVH_WIDTH; ++k) {
    if (k < n) {
      for (int c = 0; c < 3; ++c) {
        q[2 * c][k] = lo[k][c];
        q[2 * c + 1][k] = hi[k][c];
      }
      int32_t l = link[k];
      if (l < 0) atomicAdd(leaves, 1u);
      if (l >= 0) {
        uint32_t slot = atomicAdd(node_counter, 1u);
        if (slot >= cap4) {
          atomicAdd(overflow, 1u);
          l = EMPTY_LINK;
        } else {
          uint32_t qi = atomicAdd(next_count, 1u);
          next[qi] = CollapseWork{l, (int32_t)slot};
          l = (int32_t)slot;
        }
      }
      ol[k] = l;
    } else {
      for (int c = 0; c < 6; ++c) q[c][k] = INFINITY;  // never intersected (see pt_types.h)
      ol[k] = EMPTY_LINK;
    }
  }
  for (int g = 0; g < BVH_GROUPS; ++g) {
    for (int c = 0; c < 6; ++c)
      o[6 * g + c] = make_float4(q[c][4 * g], q[c][4 * g + 1], q[c][4 * g + 2], q[c][4 * g + 3]);
    o[6 * BVH_GROUPS + g] = make_float4(__int_as_float(ol[4 * g]), __int_as_float(ol[4 * g + 1]),
                                        __int_as_float(ol[4 * g + 2]), __int_as_float(ol[4 * g + 3]));
    o[7 * BVH_GROUPS + g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

__global__ void k_collapse(const float4* bin, const CollapseWork* work, const uint32_t* work_count, float4* out4,
                           uint32_t* node_counter, uint32_t cap4, CollapseWork* next, uint32_t* next_count,
                           uint32_t* overflow, uint32_t* leaves) {
  const uint32_t nwork = *work_count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwork; i += gridDim.x * blockDim.x)
    collapse_one(bin, work[i], out4, node_counter, cap4, next, next_count, overflow, leaves);
}

template <class T>
struct Tmp {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(reinterpret_cast<void**>(&p), n * sizeof(T), st);
  }
  ~Tmp() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

int build_bvh(const float4* tri_v0, const float4* tri_e1, const float4* tri_e2, uint32_t n, BvhBuffers& out,
              uint32_t* num_nodes, cudaStream_t st) {
  if (n == 0) return 0;
  Tmp<float4> tlo, thi, tc;
  Tmp<uint32_t> ids_a, ids_b, final_ids, counters, first_chunk, chunk_left;
  Tmp<BuildTask> tasks_a, tasks_b, large_a, large_b, sub;
  Tmp<BuildNode> nodes;
  Tmp<LargeState> lstate;
  const uint32_t cap = 2 * n;
  const uint32_t max_chunks = n / CHUNK + MAX_LARGE + 1;
  if (tlo.alloc(n, st) || thi.alloc(n, st) || tc.alloc(n, st) || ids_a.alloc(n, st) || ids_b.alloc(n, st) ||
      final_ids.alloc(n, st) || counters.alloc(8, st) || tasks_a.alloc(n + 1, st) || tasks_b.alloc(n + 1, st) ||
      nodes.alloc(cap, st) || large_a.alloc(MAX_LARGE, st) || large_b.alloc(MAX_LARGE, st) ||
      lstate.alloc(MAX_LARGE, st) || first_chunk.alloc(MAX_LARGE + 1, st) || chunk_left.alloc(max_chunks, st) ||
      sub.alloc(n + 1, st))
    return 2;
  k_prep<<<(n + 255) / 256, 256, 0, st>>>(tri_v0, tri_e1, tri_e2, n, tlo.p, thi.p, tc.p, ids_a.p);
  // counters: [0] node counter, [1]/[2] small-task counts A/B, [3]/[4] large-task counts A/B,
  // [5] whole-subtree tasks, [6] subtree error flag
  const BuildTask root{0, 0, n, 0};
  const bool root_sub = n <= SUBTREE_MAX;
  const bool root_large = n > LARGE_TASK;
  uint32_t init[8] = {1, (root_large || root_sub) ? 0u : 1u, 0, root_large ? 1u : 0u, 0, root_sub ? 1u : 0u, 0, 0};
  cudaMemcpyAsync(root_sub ? sub.p : (root_large ? large_a.p : tasks_a.p), &root, sizeof(root), cudaMemcpyHostToDevice,
                  st);
  cudaMemcpyAsync(counters.p, init, sizeof(init), cudaMemcpyHostToDevice, st);
  uint32_t ntasks = (root_large || root_sub) ? 0 : 1, nlarge = root_large ? 1 : 0;
  std::vector<BuildTask> hlarge(MAX_LARGE);
  hlarge[0] = root;
  std::vector<uint32_t> hfirst(MAX_LARGE + 1);
  BuildTask* cur = tasks_a.p;
  BuildTask* nxt = tasks_b.p;
  BuildTask* lcur = large_a.p;
  BuildTask* lnxt = large_b.p;
  uint32_t* src = ids_a.p;
  uint32_t* dst = ids_b.p;
  int cur_slot = 1, nxt_slot = 2;
  uint32_t host_counts[8];
  for (int level = 0; level < 200 && (ntasks > 0 || nlarge > 0); ++level) {
    cudaMemsetAsync(counters.p + nxt_slot, 0, sizeof(uint32_t), st);
    cudaMemsetAsync(counters.p + nxt_slot + 2, 0, sizeof(uint32_t), st);
    ChildLists next;
    next.tasks = nxt;
    next.count = counters.p + nxt_slot;
    next.large = lnxt;
    next.large_count = counters.p + nxt_slot + 2;
    next.large_min = LARGE_TASK;
    next.sub = sub.p;
    next.sub_count = counters.p + 5;
    next.sub_max = SUBTREE_MAX;
    next.sub_cap = n + 1;
    next.dst_parity = dst == ids_b.p ? 1u : 0u;
    if (ntasks > 0)
      k_level<<<ntasks, BUILD_THREADS, 0, st>>>(cur, counters.p + cur_slot, src, dst, final_ids.p, tlo.p, thi.p,
                                                tc.p, nodes.p, counters.p, next);
    if (nlarge > 0) {
      uint32_t nchunks = 0;
      for (uint32_t j = 0; j < nlarge; ++j) {
        hfirst[j] = nchunks;
        nchunks += (hlarge[j].count + CHUNK - 1) / CHUNK;
      }
      hfirst[nlarge] = nchunks;
      if (nchunks > max_chunks) return 6;
      cudaMemcpyAsync(first_chunk.p, hfirst.data(), (nlarge + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
      k_large_init<<<nlarge, 64, 0, st>>>(lstate.p, nlarge);
      k_large_bounds<<<nchunks, BUILD_THREADS, 0, st>>>(lcur, first_chunk.p, nlarge, src, tlo.p, thi.p, tc.p,
                                                        lstate.p);
      k_large_bin<<<nchunks, BUILD_THREADS, 0, st>>>(lcur, first_chunk.p, nlarge, src, tlo.p, thi.p, tc.p, lstate.p);
      k_large_split<<<(nlarge + 1) / 2, 64, 0, st>>>(lcur, nlarge, lstate.p, nodes.p, counters.p, next);
      k_large_count<<<nchunks, BUILD_THREADS, 0, st>>>(lcur, first_chunk.p, nlarge, src, tc.p, lstate.p,
                                                       chunk_left.p);
      k_large_scatter<<<nchunks, BUILD_THREADS, 0, st>>>(lcur, first_chunk.p, nlarge, src, dst, tc.p, lstate.p,
                                                         chunk_left.p);
    }
    cudaMemcpyAsync(host_counts, counters.p, sizeof(host_counts), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hlarge.data(), lnxt, MAX_LARGE * sizeof(BuildTask), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
    ntasks = host_counts[nxt_slot];
    nlarge = std::min(host_counts[nxt_slot + 2], MAX_LARGE);
    std::swap(cur, nxt);
    std::swap(lcur, lnxt);
    std::swap(src, dst);
    std::swap(cur_slot, nxt_slot);
  }
  if (ntasks != 0 || nlarge != 0) return 4;
  // the whole subtrees, one warp each, in one launch
  cudaMemcpyAsync(host_counts, counters.p, sizeof(host_counts), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  const uint32_t nsub = std::min(host_counts[5], n + 1);
  if (nsub > 0 &&
      cudaFuncSetAttribute(k_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SUBTREE_SMEM) != cudaSuccess)
    return 3;
  if (nsub > 0)
    k_subtree<<<(nsub + SUB_WARPS - 1) / SUB_WARPS, SUB_WARPS * 32, SUBTREE_SMEM, st>>>(
        sub.p, counters.p + 5, n + 1, ids_a.p, ids_b.p, final_ids.p, tlo.p, thi.p, tc.p, nodes.p, counters.p,
        counters.p + 6);
  cudaMemcpyAsync(host_counts, counters.p, sizeof(host_counts), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  if (host_counts[6] != 0) return 7;
  const uint32_t nn = host_counts[0];
  if (nn > out.node_capacity) return 5;
  k_layout<<<(nn + 255) / 256, 256, 0, st>>>(nodes.p, nn, out.nodes);
  k_reorder<<<(n + 255) / 256, 256, 0, st>>>(final_ids.p, n, tri_v0, tri_e1, tri_e2, out.tri_sorted);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  *num_nodes = nn;
  return 0;
}

int collapse_wide(const float4* bin, uint32_t nn_bin, float4* out4, uint32_t cap4, uint32_t* num4, cudaStream_t st,
                  uint32_t* num_leaves) {
  if (nn_bin == 0 || cap4 == 0) return 2;
  Tmp<CollapseWork> qa, qb;
  Tmp<uint32_t> counters;  // [0] wide nodes, [1] next queue A, [2] next queue B, [3] overflow, [4] leaves
  const uint32_t qcap = nn_bin + 1;
  if (qa.alloc(qcap, st) || qb.alloc(qcap, st) || counters.alloc(5, st)) return 2;
  CollapseWork root{0, 0};
  uint32_t init[5] = {1, 1, 0, 0, 0};
  cudaMemcpyAsync(qa.p, &root, sizeof(root), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(counters.p, init, sizeof(init), cudaMemcpyHostToDevice, st);
  // Levels run in batches without a host round trip: each launch reads its
  // work count from the level before (a level past the last one finds none),
  // and the host looks at the count once per batch.
  const int grid = std::max(1, std::min<int>((int)((qcap + 255) / 256), device_sm_count() * 8));
  CollapseWork* cur = qa.p;
  CollapseWork* nxt = qb.p;
  uint32_t* cnt_cur = counters.p + 1;
  uint32_t* cnt_nxt = counters.p + 2;
  uint32_t host = 1;
  for (int level = 0; host > 0;) {
    if (level >= 256) return 4;
    for (int k = 0; k < 8; ++k, ++level) {
      cudaMemsetAsync(cnt_nxt, 0, sizeof(uint32_t), st);
      k_collapse<<<grid, 256, 0, st>>>(bin, cur, cnt_cur, out4, counters.p, cap4, nxt, cnt_nxt, counters.p + 3,
                                       counters.p + 4);
      std::swap(cur, nxt);
      std::swap(cnt_cur, cnt_nxt);
    }
    cudaMemcpyAsync(&host, cnt_cur, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  }
  uint32_t res[5];
  cudaMemcpyAsync(res, counters.p, sizeof(res), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
  if (res[3] != 0) return 5;
  *num4 = res[0];
  if (num_leaves) *num_leaves = res[4];
  return 0;
}


// ---------------------------------------------------------------------------
// Allocation-free build (pt_bvh_build_noalloc).
//
// Hosts that own all device memory themselves -- engines that reserve their
// pools up front and may not call cudaMalloc/cudaFree inside the frame loop,
// or code that must not touch the allocator while other work is being
// recorded -- still need the per-frame BVH rebuild of animated geometry. For
// them the build's scratch (bounds, centroids, id ping-pong buffers, task
// lists, build nodes) lives in this file-scope device array instead of
// cudaMalloc'ed memory. It holds the scratch of up to
// PT_NOALLOC_MAX_TRIANGLES triangles (about 11.3 MB) and stays resident on
// every device that loads the library until the process exits.
namespace {

constexpr size_t NA_MAX = PT_NOALLOC_MAX_TRIANGLES;
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t NA_OFF_TLO = 0;
constexpr size_t NA_OFF_THI = align256(NA_OFF_TLO + NA_MAX * sizeof(float4));
constexpr size_t NA_OFF_TC = align256(NA_OFF_THI + NA_MAX * sizeof(float4));
constexpr size_t NA_OFF_IDA = align256(NA_OFF_TC + NA_MAX * sizeof(float4));
constexpr size_t NA_OFF_IDB = align256(NA_OFF_IDA + NA_MAX * sizeof(uint32_t));
constexpr size_t NA_OFF_FIN = align256(NA_OFF_IDB + NA_MAX * sizeof(uint32_t));
constexpr size_t NA_OFF_CNT = align256(NA_OFF_FIN + NA_MAX * sizeof(uint32_t));
constexpr size_t NA_OFF_TKA = align256(NA_OFF_CNT + 4 * sizeof(uint32_t));
constexpr size_t NA_OFF_TKB = align256(NA_OFF_TKA + (NA_MAX + 1) * sizeof(BuildTask));
constexpr size_t NA_OFF_NOD = align256(NA_OFF_TKB + (NA_MAX + 1) * sizeof(BuildTask));
constexpr size_t NA_BYTES = align256(NA_OFF_NOD + 2 * NA_MAX * sizeof(BuildNode));

static __device__ __align__(256) unsigned char g_bvh_noalloc_scratch[NA_BYTES];

// Device address of the scratch array, looked up with the device current
// the first time a context uses it. In host code the symbol itself is only a
// host-side stand-in. The cache is keyed by the context's unique id as well
// as the device: after cudaDeviceReset the module is loaded again in a new
// context, possibly at another address, and the lookup is repeated.
std::mutex g_na_mutex;
void* g_na_ptr[64] = {};
unsigned long long g_na_ctx[64] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current context (0 when the driver cannot say).
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      get_id = reinterpret_cast<CtxGetIdFn>(f2);
    } else {
      cudaGetLastError();
    }
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

cudaError_t noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  // makes the device's primary context current (initialising it) before its id is read
  if ((e = cudaSetDevice(dev)) != cudaSuccess) return e;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev] || ctx == 0 || g_na_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_bvh_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_ptr[dev] = p;
    g_na_ctx[dev] = ctx;
  }
  *out = static_cast<unsigned char*>(g_na_ptr[dev]);
  return cudaSuccess;
}

pt_status na_fail(char* msg, size_t cap, pt_status st, const char* text) {
  if (msg && cap) std::snprintf(msg, cap, "%s", text);
  return st;
}

}  // namespace

}  // namespace hpt

extern "C" pt_status pt_bvh_build_noalloc(const void* tri_v0, const void* tri_e1, const void* tri_e2,
                                          uint32_t num_triangles, void* nodes_out, uint32_t node_capacity,
                                          void* tri_sorted_out, uint32_t* num_nodes_out, void* stream,
                                          char* error_message, size_t error_capacity) {
  using namespace hpt;
  if (error_message && error_capacity) error_message[0] = '\0';
  if (!num_nodes_out) return na_fail(error_message, error_capacity, PT_ERR_INVALID_ARG, "num_nodes_out is null");
  *num_nodes_out = 0;
  if (num_triangles > PT_NOALLOC_MAX_TRIANGLES) {
    char buf[160];
    std::snprintf(buf, sizeof(buf),
                  "num_triangles %u exceeds the allocation-free limit of %u (PT_NOALLOC_MAX_TRIANGLES)",
                  num_triangles, (unsigned)PT_NOALLOC_MAX_TRIANGLES);
    return na_fail(error_message, error_capacity, PT_ERR_INVALID_ARG, buf);
  }
  if (num_triangles == 0) return PT_OK;
  if (!tri_v0 || !tri_e1 || !tri_e2 || !nodes_out || !tri_sorted_out)
    return na_fail(error_message, error_capacity, PT_ERR_INVALID_ARG, "a device pointer is null");
  if (node_capacity < 2 * num_triangles)
    return na_fail(error_message, error_capacity, PT_ERR_INVALID_ARG, "node_capacity must be >= 2 * num_triangles");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_scratch(&base);
  if (e != cudaSuccess) return na_fail(error_message, error_capacity, PT_ERR_CUDA, cudaGetErrorString(e));
  const uint32_t n = num_triangles;
  float4* tlo = reinterpret_cast<float4*>(base + NA_OFF_TLO);
  float4* thi = reinterpret_cast<float4*>(base + NA_OFF_THI);
  float4* tc = reinterpret_cast<float4*>(base + NA_OFF_TC);
  uint32_t* ids_a = reinterpret_cast<uint32_t*>(base + NA_OFF_IDA);
  uint32_t* ids_b = reinterpret_cast<uint32_t*>(base + NA_OFF_IDB);
  uint32_t* final_ids = reinterpret_cast<uint32_t*>(base + NA_OFF_FIN);
  uint32_t* counters = reinterpret_cast<uint32_t*>(base + NA_OFF_CNT);
  BuildTask* tasks_a = reinterpret_cast<BuildTask*>(base + NA_OFF_TKA);
  BuildTask* tasks_b = reinterpret_cast<BuildTask*>(base + NA_OFF_TKB);
  BuildNode* nodes = reinterpret_cast<BuildNode*>(base + NA_OFF_NOD);
  const float4* v0 = static_cast<const float4*>(tri_v0);
  const float4* e1 = static_cast<const float4*>(tri_e1);
  const float4* e2 = static_cast<const float4*>(tri_e2);
  // The array keeps the previous call's contents: the root task and the
  // counters are rewritten here; every other word is written before it is read.
  auto cuda_err = [&](cudaError_t x) { return na_fail(error_message, error_capacity, PT_ERR_CUDA, cudaGetErrorString(x)); };
  k_prep<<<(n + 255) / 256, 256, 0, st>>>(v0, e1, e2, n, tlo, thi, tc, ids_a);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e);
  // pageable sources: the copies have finished reading them when the calls return
  BuildTask root{0, 0, n, 0};
  uint32_t init[4] = {1, 1, 0, 0};
  if ((e = cudaMemcpyAsync(tasks_a, &root, sizeof(root), cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_err(e);
  if ((e = cudaMemcpyAsync(counters, init, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_err(e);
  uint32_t ntasks = 1;
  BuildTask* cur = tasks_a;
  BuildTask* nxt = tasks_b;
  uint32_t* src = ids_a;
  uint32_t* dst = ids_b;
  int cur_slot = 1, nxt_slot = 2;
  uint32_t host_count = 0;
  for (int level = 0; level < 200 && ntasks > 0; ++level) {
    if ((e = cudaMemsetAsync(counters + nxt_slot, 0, sizeof(uint32_t), st)) != cudaSuccess) return cuda_err(e);
    ChildLists next;
    next.tasks = nxt;
    next.count = counters + nxt_slot;
    k_level<<<ntasks, BUILD_THREADS, 0, st>>>(cur, counters + cur_slot, src, dst, final_ids, tlo, thi, tc, nodes,
                                              counters, next);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e);
    if ((e = cudaMemcpyAsync(&host_count, counters + nxt_slot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess)
      return cuda_err(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e);
    ntasks = host_count;
    std::swap(cur, nxt);
    std::swap(src, dst);
    std::swap(cur_slot, nxt_slot);
  }
  if (ntasks != 0) return na_fail(error_message, error_capacity, PT_ERR_CUDA, "BVH build did not terminate");
  uint32_t nn = 0;
  if ((e = cudaMemcpyAsync(&nn, counters, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_err(e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e);
  if (nn == 0 || nn > node_capacity)
    return na_fail(error_message, error_capacity, PT_ERR_CUDA, "BVH build produced an invalid node count");
  k_layout<<<(nn + 255) / 256, 256, 0, st>>>(nodes, nn, static_cast<float4*>(nodes_out));
  k_reorder<<<(n + 255) / 256, 256, 0, st>>>(final_ids, n, v0, e1, e2, static_cast<float4*>(tri_sorted_out));
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return na_fail(error_message, error_capacity, PT_ERR_CUDA, cudaGetErrorString(e));
  *num_nodes_out = nn;
  return PT_OK;
}

namespace hpt {

}  // namespace hpt
