// Kernel instantiations of one group of (la lb | lc ld) classes with an f shell (FP64 only).
// Generated layout: each group is its own translation unit so the build compiles them in parallel.
#include "oqpg_launch.cuh"

namespace oqpg {

cudaError_t launch_group11(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 41: return launch_cls<2, 2, 2, 3>(pure, mode, a, nsm, st);
    case 42: return launch_cls<0, 3, 2, 3>(pure, mode, a, nsm, st);
    case 43: return launch_cls<1, 3, 2, 3>(pure, mode, a, nsm, st);
    case 44: return launch_cls<2, 3, 2, 3>(pure, mode, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
