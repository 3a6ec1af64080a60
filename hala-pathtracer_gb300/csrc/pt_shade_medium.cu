// pt_shade_medium.cu -- material shading kernels of single-scene wavefronts
// of scenes with media.
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_medium(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                             cudaStream_t st) {
  launch_permutation<true, false, false>(S, P, Q, g, tr, tex, st);
}

}  // namespace hpt
