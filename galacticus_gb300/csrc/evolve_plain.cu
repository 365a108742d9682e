// evolve_plain.cu -- instantiations of evolve_kernel for the plain form
// (FP64 rates, CIE table: the parity form).
#include "evolve_kernel.cuh"

namespace gal {

cudaError_t evolve_launch_plain(int threads, const LaunchArgs& a) {
  if (krumholz(a)) return threads == 128 ? launch_evolve<128, MODE_PLAIN, false, false, true>(a) : cudaErrorInvalidConfiguration;
  switch (threads) {
    case 64: return launch_evolve<64, MODE_PLAIN>(a);
    case 128: return launch_evolve<128, MODE_PLAIN>(a);
    case 256: return launch_evolve<256, MODE_PLAIN>(a);
    case 512: return launch_evolve<512, MODE_PLAIN>(a);
    default: return cudaErrorInvalidConfiguration;
  }
}

cudaError_t evolve_launch_plain_interrupt(const LaunchArgs& a) {
  if (krumholz(a)) return cudaErrorInvalidConfiguration;
  return launch_evolve<128, MODE_PLAIN, false, true>(a);
}

}  // namespace gal
