// pt_shade_multi.cu -- material shading kernels of shared wavefronts (paths
// of several jobs; each path reads its job's scene record) without media.
// One translation unit per combination so that the variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {

void launch_materials_multi(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tr, bool tex,
                            cudaStream_t st) {
  launch_permutation<false, true, false>(S, P, Q, g, tr, tex, st);
}

}  // namespace hpt
