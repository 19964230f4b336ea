// Kernel instantiations of one group of (la lb | lc ld) classes with an f shell (FP64 only).
// Generated layout: each group is its own translation unit so the build compiles them in parallel.
#include "oqpg_launch.cuh"

namespace oqpg {

cudaError_t launch_group10(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 36: return launch_cls<0, 0, 2, 3>(pure, mode, a, nsm, st);
    case 37: return launch_cls<0, 1, 2, 3>(pure, mode, a, nsm, st);
    case 38: return launch_cls<0, 2, 2, 3>(pure, mode, a, nsm, st);
    case 39: return launch_cls<1, 1, 2, 3>(pure, mode, a, nsm, st);
    case 40: return launch_cls<1, 2, 2, 3>(pure, mode, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
