// pt_shade_single.cu -- material shading kernels of single-scene wavefronts
// (every feature permutation, with and without the radiance cache).
// Separate translation unit so that the kernel variants compile in parallel.
#include "pt_shade.cuh"

namespace hpt {
namespace {

template <bool MED, bool TR, bool CACHE, bool TEX>
void two(const DevScene& S, const PathState& P, const QueueSet& Q, int g, cudaStream_t st) {
  k_shade<PT_MATERIAL_DIFFUSE, MED, TR, false, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<PT_MATERIAL_DISNEY, MED, TR, false, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
  k_shade<SHADE_DISNEY_GLASS, MED, TR, false, CACHE, TEX><<<g, 256, 0, st>>>(S, P, Q);
}

template <bool MED, bool TR, bool CACHE>
void by_tex(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool tex, cudaStream_t st) {
  if (tex) two<MED, TR, CACHE, true>(S, P, Q, g, st);
  else two<MED, TR, CACHE, false>(S, P, Q, g, st);
}

}  // namespace

void launch_materials_single(const DevScene& S, const PathState& P, const QueueSet& Q, int g, bool med, bool tr,
                             bool tex, bool cache, cudaStream_t st) {
  if (cache) {  // the cache is refused for scenes with media
    if (tr) by_tex<false, true, true>(S, P, Q, g, tex, st);
    else by_tex<false, false, true>(S, P, Q, g, tex, st);
  } else if (med) {
    if (tr) by_tex<true, true, false>(S, P, Q, g, tex, st);
    else by_tex<true, false, false>(S, P, Q, g, tex, st);
  } else {
    if (tr) by_tex<false, true, false>(S, P, Q, g, tex, st);
    else by_tex<false, false, false>(S, P, Q, g, tex, st);
  }
}

}  // namespace hpt
