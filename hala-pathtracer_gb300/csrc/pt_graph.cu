// pt_graph.cu -- the bounce loop of one wave as one CUDA graph launch.
//
//   root:  k_graph_init -> while (go) {
//            switch (grid bucket) { bounce, even queue parity }  -> k_graph_step(even)
//            switch (grid bucket) { bounce, odd queue parity }   -> k_graph_step(odd)
//          }
//
// A bounce is the same kernel sequence the host-driven loop launches
// (closest hit, surface logic, the three material kernels, shadow rays); the
// bounce kernels read their queue lengths from device memory, so a grid at
// least as large as the queue gives the same result as an exact one. The
// one-thread control kernels read the continuing-path count, clear the
// counters the next bounce will fill, and choose the next grid bucket and
// whether the loop goes on, so the host does one read-back per wave instead
// of one per bounce. The loop ends when no path continues or after
// `bounce_cap` bounces: every body iteration either runs a bounce (and
// counts it) or ends the loop. The cases of the buckets of at most
// `tail_paths` paths run the wave's tail instead of one bounce: one k_tail
// launch that carries every remaining path to its end (as the host-driven
// loop does once that few paths are left) and records the bounces it ran in
// G_TAIL, which the next control kernel adds to the count and which ends
// the loop.
#include <cuda_runtime.h>

#include <cstring>

#include "pt_impl.h"

namespace hpt {
namespace {

constexpr uint32_t BUCKET0 = 4096;  // paths of the smallest grid bucket; bucket k holds 4096 * 4^k

// Grid buckets for a wavefront of `cap` paths: the last one is the capacity.
uint32_t bucket_count(uint32_t cap) {
  uint32_t nb = 1;
  for (uint64_t lim = BUCKET0; lim < cap; lim <<= 2) ++nb;
  return nb;
}

uint32_t bucket_limit(uint32_t k, uint32_t nb, uint32_t cap) {
  return k + 1 >= nb ? cap : (BUCKET0 << (2 * k));
}

__device__ uint32_t bucket_of(uint32_t live, uint32_t nb) {
  uint32_t k = 0;
  for (uint64_t lim = BUCKET0; k + 1 < nb && live > lim; lim <<= 2) ++k;
  return k;
}

// Before the loop: the camera kernel left the first bounce's input count in
// the odd counter set; the even set is the first bounce's output.
__global__ void k_graph_init(uint32_t* gctl, const uint32_t* cnt_odd, uint32_t* cnt_even, uint32_t nb, uint32_t cap,
                             cudaGraphConditionalHandle h_first, cudaGraphConditionalHandle h_loop) {
  const uint32_t live = cnt_odd[Q_NEXT];
  const bool go = live > 0 && cap > 0;
  for (int k = 0; k < Q_COUNT; ++k) cnt_even[k] = 0;
  gctl[G_DONE] = 0;
  gctl[G_LIVE] = live;
  gctl[G_GO] = go ? 1u : 0u;
  gctl[G_TAIL] = 0;
  cudaGraphSetConditional(h_first, go ? bucket_of(live, nb) : nb);
  cudaGraphSetConditional(h_loop, go ? 1u : 0u);
}

// After the bounce of one parity (or after its switch ran no case).
// `cnt_this` is that bounce's output set, `cnt_other` its input set, which
// becomes the next bounce's output and is cleared here.
__global__ void k_graph_step(uint32_t* gctl, const uint32_t* cnt_this, uint32_t* cnt_other, uint32_t nb,
                             uint32_t cap, cudaGraphConditionalHandle h_next, cudaGraphConditionalHandle h_loop,
                             int last) {
  bool go = false;
  if (gctl[G_GO]) {  // the bounce before this kernel ran (or the wave's tail, G_TAIL bounces)
    const uint32_t live = cnt_this[Q_NEXT];
    const uint32_t tail = gctl[G_TAIL];
    const uint32_t done = gctl[G_DONE] + (tail ? tail : 1u);
    go = live > 0 && done < cap;
    for (int k = 0; k < Q_COUNT; ++k) cnt_other[k] = 0;
    gctl[G_DONE] = done;
    gctl[G_LIVE] = live;
    gctl[G_GO] = go ? 1u : 0u;
    cudaGraphSetConditional(h_next, go ? bucket_of(cnt_this[Q_NEXT], nb) : nb);
  } else {
    cudaGraphSetConditional(h_next, nb);
  }
  if (last) cudaGraphSetConditional(h_loop, go ? 1u : 0u);
}

QueueSet queues_for(WaveBuffers& W, uint32_t parity) {
  uint32_t* cnt0 = W.counters.p;
  uint32_t* cnt1 = W.counters.p + Q_COUNT;
  uint32_t* out = parity ? cnt1 : cnt0;
  uint32_t* in_cnt = (parity ? cnt0 : cnt1) + Q_NEXT;
  uint32_t* qin = parity ? W.q_b.p : W.q_a.p;
  uint32_t* qnext = parity ? W.q_a.p : W.q_b.p;
  return QueueSet{qin, in_cnt, qnext, W.q_diff.p, W.q_dis.p, W.q_glass.p, W.q_shadow.p, out,
                  W.rays.p};
}

void append(std::vector<unsigned char>& k, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  k.insert(k.end(), b, b + n);
}

// Everything the captured kernels received by value, plus the graph shape.
std::vector<unsigned char> graph_key(const DevScene& S, WaveBuffers& W, uint32_t bounce_cap, uint32_t tail) {
  std::vector<unsigned char> k;
  append(k, &S, sizeof(S));
  append(k, &W.P, sizeof(W.P));
  for (uint32_t parity = 0; parity < 2; ++parity) {
    const QueueSet Q = queues_for(W, parity);
    append(k, &Q, sizeof(Q));
  }
  const uint32_t shape[3] = {W.cap, bounce_cap, tail};
  append(k, shape, sizeof(shape));
  return k;
}

cudaError_t add_kernel_node(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* dep, void* func,
                            void** args) {
  cudaKernelNodeParams kp{};
  kp.func = func;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(1);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &kp);
}

cudaError_t build_graph(const DevScene& S, WaveBuffers& W, uint32_t bounce_cap, uint32_t tail, cudaStream_t st,
                        cudaGraph_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  auto fail = [&](cudaError_t x) {
    cudaGraphDestroy(g);
    return x;
  };
  uint32_t nb = bucket_count(W.cap);
  uint32_t cap = bounce_cap;
  uint32_t* cnt0 = W.counters.p;
  uint32_t* cnt1 = W.counters.p + Q_COUNT;
  uint32_t* gctl = W.counters.p + 2 * Q_COUNT;
  cudaGraphConditionalHandle h_loop, h_sw[2];
  if ((e = cudaGraphConditionalHandleCreate(&h_loop, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess ||
      (e = cudaGraphConditionalHandleCreate(&h_sw[0], g, nb, cudaGraphCondAssignDefault)) != cudaSuccess ||
      (e = cudaGraphConditionalHandleCreate(&h_sw[1], g, nb, cudaGraphCondAssignDefault)) != cudaSuccess)
    return fail(e);
  cudaGraphNode_t n_init;
  {
    void* args[] = {&gctl, &cnt1, &cnt0, &nb, &cap, &h_sw[0], &h_loop};
    if ((e = add_kernel_node(&n_init, g, nullptr, reinterpret_cast<void*>(k_graph_init), args)) != cudaSuccess)
      return fail(e);
  }
  cudaGraphNodeParams wp{};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = h_loop;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t n_while;
  if ((e = cudaGraphAddNode(&n_while, g, &n_init, nullptr, 1, &wp)) != cudaSuccess) return fail(e);
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  cudaGraphNode_t prev = nullptr;
  for (uint32_t parity = 0; parity < 2; ++parity) {
    cudaGraphNodeParams sp{};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = h_sw[parity];
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = nb;
    cudaGraphNode_t n_sw;
    if ((e = cudaGraphAddNode(&n_sw, body, prev ? &prev : nullptr, nullptr, prev ? 1 : 0, &sp)) != cudaSuccess)
      return fail(e);
    const QueueSet Q = queues_for(W, parity);
    for (uint32_t k = 0; k < nb; ++k) {
      cudaGraph_t cg = sp.conditional.phGraph_out[k];
      if ((e = cudaStreamBeginCaptureToGraph(st, cg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
          cudaSuccess)
        return fail(e);
      const uint32_t lim = bucket_limit(k, nb, W.cap);
      if (lim <= tail) {
        // few paths left: the rest of the wave in one kernel
        launch_tail(S, W.P, Q, lim, gctl + G_DONE, 0u, bounce_cap, gctl + G_TAIL, st);
      } else {
        launch_trace(S, W.P, Q, lim, false, st);
        launch_shade(S, W.P, Q, lim, st);
      }
      cudaError_t le = cudaGetLastError();
      cudaGraph_t captured = nullptr;
      e = cudaStreamEndCapture(st, &captured);
      if (le != cudaSuccess) return fail(le);
      if (e != cudaSuccess) return fail(e);
    }
    uint32_t* cnt_this = parity ? cnt1 : cnt0;
    uint32_t* cnt_other = parity ? cnt0 : cnt1;
    int last = parity == 1 ? 1 : 0;
    void* args[] = {&gctl, &cnt_this, &cnt_other, &nb, &cap, &h_sw[parity ^ 1], &h_loop, &last};
    cudaGraphNode_t n_step;
    if ((e = add_kernel_node(&n_step, body, &n_sw, reinterpret_cast<void*>(k_graph_step), args)) != cudaSuccess)
      return fail(e);
    prev = n_step;
  }
  *out = g;
  return cudaSuccess;
}

}  // namespace

void BounceGraph::reset() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  key.clear();
}

cudaError_t run_bounces_graph(const DevScene& S, WaveBuffers& W, uint32_t bounce_cap, BounceLoop& L,
                              uint32_t* pinned, cudaStream_t st) {
  BounceGraph& G = W.graph;
  const uint32_t tail = tail_paths(L, W);
  std::vector<unsigned char> key = graph_key(S, W, bounce_cap, tail);
  cudaError_t e;
  if (!G.exec || key != G.key) {
    cudaGraph_t g = nullptr;
    if ((e = build_graph(S, W, bounce_cap, tail, st, &g)) != cudaSuccess) {
      G.reset();
      return e;
    }
    bool updated = false;
    if (G.exec) {
      cudaGraphExecUpdateResultInfo info{};
      updated = cudaGraphExecUpdate(G.exec, g, &info) == cudaSuccess;
      if (!updated) cudaGetLastError();  // an update that does not fit is not an error: instantiate instead
    }
    if (!updated) {
      if (G.exec) cudaGraphExecDestroy(G.exec);
      G.exec = nullptr;
      if ((e = cudaGraphInstantiate(&G.exec, g, 0)) != cudaSuccess) {
        cudaGraphDestroy(g);
        G.reset();
        return e;
      }
    }
    if (G.graph) cudaGraphDestroy(G.graph);
    G.graph = g;
    G.key.swap(key);
    ++G.builds;
  }
  if ((e = cudaGraphLaunch(G.exec, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(pinned, W.counters.p + 2 * Q_COUNT, G_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           st)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  const uint32_t done = pinned[G_DONE], live = pinned[G_LIVE], tail_bounces = pinned[G_TAIL];
  const bool med_tr = (S.features & PT_FEATURE_MEDIUM) && (S.features & PT_FEATURE_TRANSPARENT);
  const uint64_t per_bounce = med_tr ? 4 : 5;
  const uint64_t cases = done - tail_bounces + (tail_bounces ? 1 : 0);  // switch cases that ran
  L.bounces = done;
  L.timed_out = live > 0;
  // bounces, the tail, init, two control kernels per loop iteration
  L.launches = per_bounce * (done - tail_bounces) + (tail_bounces ? 1 : 0) + 1 + 2ull * ((cases + 1) / 2);
  return cudaSuccess;
}

}  // namespace hpt
