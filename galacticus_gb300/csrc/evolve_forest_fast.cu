// evolve_forest_fast.cu -- instantiations of evolve_kernel for whole-forest
// evolution in the FP32-rate forms (with and without the cooling surrogate).
#include "evolve_kernel.cuh"

namespace gal {

cudaError_t evolve_launch_forest_fast(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return threads == 128 ? launch_evolve<128, MODE_FAST, true, false, true>(a) : cudaErrorInvalidConfiguration;
  switch (threads) {
    case 128: return launch_evolve<128, MODE_FAST, true>(a);
    case 256: return launch_evolve<256, MODE_FAST, true>(a);
    case 512: return launch_evolve<512, MODE_FAST, true>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

cudaError_t evolve_launch_forest_fast_surrogate(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return cudaErrorInvalidConfiguration;
  switch (threads) {
    case 128: return launch_evolve<128, MODE_FAST_SURROGATE, true>(a);
    case 256: return launch_evolve<256, MODE_FAST_SURROGATE, true>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace gal
