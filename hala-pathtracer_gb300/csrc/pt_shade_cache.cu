// pt_shade_cache.cu -- material shading kernels (and the wave-tail kernel) of single-scene wavefronts
// with a radiance cache attached (no media).
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_cache(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                            cudaStream_t st) {
  launch_permutation<false, false, true>(S, P, Q, g, tr, tex, st);
}

void launch_tail_cache(const DevScene& S, const PathState& P, const QueueSet& Q, uint32_t max_items,
                       const uint32_t* done_ptr, uint32_t done, uint32_t cap, uint32_t* tail_bounces, bool tr, bool tex,
                       cudaStream_t st) {
  launch_tail_permutation<false, false, true>(S, P, Q, max_items, done_ptr, done, cap, tail_bounces, tr, tex, st);
}

}  // namespace hpt
