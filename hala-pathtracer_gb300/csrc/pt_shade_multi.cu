// pt_shade_multi.cu -- material shading kernels of shared wavefronts
// (paths of several jobs; each path reads its job's scene record).
// Separate translation unit so that the kernel variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {
namespace {

template <bool MED, bool TR, bool TEX>
void two(const DevScene& S, const PathState& P, const QueueSet& Q, int g, cudaStream_t st) {
  k_shade<PT_MATERIAL_DIFFUSE, MED, TR, true, false, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<PT_MATERIAL_DISNEY, MED, TR, true, false, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<SHADE_DISNEY_GLASS, MED, TR, true, false, TEX><<<g, 256, 0, st>>>(S, P, Q);
}

template <bool MED, bool TR>
void by_tex(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tex, cudaStream_t st) {
  if (tex) two<MED, TR, true>(S, P, Q, g, st);
  else two<MED, TR, false>(S, P, Q, g, st);
}

}  // namespace

void launch_materials_multi(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool med, bool tr,
                            bool tex, cudaStream_t st) {
  if (med) {
    if (tr) by_tex<true, true>(S, P, Q, g, tex, st);
    else by_tex<true, false>(S, P, Q, g, tex, st);
  } else {
    if (tr) by_tex<false, true>(S, P, Q, g, tex, st);
    else by_tex<false, false>(S, P, Q, g, tex, st);
  }
}

}  // namespace hpt
