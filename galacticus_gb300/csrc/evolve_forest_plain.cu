// evolve_forest_plain.cu -- instantiations of evolve_kernel for whole-forest
// evolution in the plain form (FP64 rates, CIE table), and the dispatch over
// the forest forms.
#include "evolve_kernel.cuh"

namespace gal {

cudaError_t evolve_launch_forest_fast(int threads, const LaunchArgs& a);
cudaError_t evolve_launch_forest_fast_surrogate(int threads, const LaunchArgs& a);

cudaError_t evolve_launch_forest_plain(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return threads == 128 ? launch_evolve<128, MODE_PLAIN, true, false, true>(a) : cudaErrorInvalidConfiguration;
  switch (threads) {
    case 64: return launch_evolve<64, MODE_PLAIN, true>(a);
    case 128: return launch_evolve<128, MODE_PLAIN, true>(a);
    case 256: return launch_evolve<256, MODE_PLAIN, true>(a);
    case 512: return launch_evolve<512, MODE_PLAIN, true>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

cudaError_t evolve_launch_forest(int mode, int threads, const LaunchArgs& a) {
  switch (mode) {
    case MODE_PLAIN: return evolve_launch_forest_plain(threads, a);
    case MODE_FAST: return evolve_launch_forest_fast(threads, a);
    case MODE_FAST_SURROGATE: return evolve_launch_forest_fast_surrogate(threads, a);
    default: return cudaErrorInvalidConfiguration;  // the FP64-rate surrogate form has no forest build
  }
}

}  // namespace gal
