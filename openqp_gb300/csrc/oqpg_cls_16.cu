// Kernel instantiations of one group of (la lb | lc ld) classes.
// Generated layout: each group is its own translation unit so the build compiles them in parallel.
#include "oqpg_launch.cuh"

namespace oqpg {

cudaError_t launch_group16(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 12: return launch_cls<0, 2, 1, 1>(pure, mode, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
