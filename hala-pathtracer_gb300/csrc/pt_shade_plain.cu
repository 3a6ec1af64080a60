// pt_shade_plain.cu -- material shading kernels of single-scene wavefronts
// without media or radiance cache.
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_plain(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                            cudaStream_t st) {
  launch_permutation<false, false, false>(S, P, Q, g, tr, tex, st);
}

}  // namespace hpt
