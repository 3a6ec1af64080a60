// pt_shade_multi_medium.cu -- material shading kernels of shared wavefronts
// of jobs with media.
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_multi_medium(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                                   cudaStream_t st) {
  launch_permutation<true, true, false>(S, P, Q, g, tr, tex, st);
}

}  // namespace hpt
