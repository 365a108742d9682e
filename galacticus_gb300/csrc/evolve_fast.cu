// evolve_fast.cu -- instantiations of evolve_kernel for the fast form
// (FP32 rates, FP32 CIE table).
#include "evolve_kernel.cuh"

namespace gal {

cudaError_t evolve_launch_fast(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return threads == 128 ? launch_evolve<128, MODE_FAST, false, false, true>(a) : cudaErrorInvalidConfiguration;
  switch (threads) {
    case 128: return launch_evolve<128, MODE_FAST>(a);
    case 256: return launch_evolve<256, MODE_FAST>(a);
    case 512: return launch_evolve<512, MODE_FAST>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace gal
