// Kernel instantiations of one group of (la lb | lc ld) classes with an f shell (FP64 only).
// Generated layout: each group is its own translation unit so the build compiles them in parallel.
#include "oqpg_launch.cuh"

namespace oqpg {

cudaError_t launch_group9(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 28: return launch_cls<0, 0, 1, 3>(pure, mode, a, nsm, st);
    case 29: return launch_cls<0, 1, 1, 3>(pure, mode, a, nsm, st);
    case 30: return launch_cls<0, 2, 1, 3>(pure, mode, a, nsm, st);
    case 31: return launch_cls<1, 1, 1, 3>(pure, mode, a, nsm, st);
    case 32: return launch_cls<1, 2, 1, 3>(pure, mode, a, nsm, st);
    case 33: return launch_cls<2, 2, 1, 3>(pure, mode, a, nsm, st);
    case 34: return launch_cls<0, 3, 1, 3>(pure, mode, a, nsm, st);
    case 35: return launch_cls<1, 3, 1, 3>(pure, mode, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
