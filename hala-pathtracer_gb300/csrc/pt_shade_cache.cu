// pt_shade_cache.cu -- material shading kernels of single-scene wavefronts
// with a radiance cache attached (no media).
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_cache(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                            cudaStream_t st) {
  launch_permutation<false, false, true>(S, P, Q, g, tr, tex, st);
}

}  // namespace hpt
