// Kernel instantiations of one group of (la lb | lc ld) classes with an f shell (FP64 only).
// Generated layout: each group is its own translation unit so the build compiles them in parallel.
#include "oqpg_launch.cuh"

namespace oqpg {

cudaError_t launch_group8(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 21: return launch_cls<0, 0, 0, 3>(pure, mode, a, nsm, st);
    case 22: return launch_cls<0, 1, 0, 3>(pure, mode, a, nsm, st);
    case 23: return launch_cls<0, 2, 0, 3>(pure, mode, a, nsm, st);
    case 24: return launch_cls<1, 1, 0, 3>(pure, mode, a, nsm, st);
    case 25: return launch_cls<1, 2, 0, 3>(pure, mode, a, nsm, st);
    case 26: return launch_cls<2, 2, 0, 3>(pure, mode, a, nsm, st);
    case 27: return launch_cls<0, 3, 0, 3>(pure, mode, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
