// evolve_fast_surrogate.cu -- instantiations of evolve_kernel for the fast surrogate form
// (FP32 rates, cooling function from the MLP surrogate).
#include "evolve_kernel.cuh"

namespace gal {

cudaError_t evolve_launch_fast_surrogate(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return cudaErrorInvalidConfiguration;
  switch (threads) {
    case 128: return launch_evolve<128, MODE_FAST_SURROGATE>(a);
    case 256: return launch_evolve<256, MODE_FAST_SURROGATE>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace gal
