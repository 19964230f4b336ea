// The double-float shell-family kernels (the df precision modes), in their
// own translation unit so that the build compiles them in parallel.
#include "oqpg_family.cuh"

namespace oqpg {

cudaError_t launch_family_df(int c, bool pure, bool warp, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 0: return launch_fam_t<0, 0, 0, 0, false, dfl>(warp, a, nsm, st);
    case 1: return launch_fam_t<0, 0, 0, 1, false, dfl>(warp, a, nsm, st);
    case 2: return pure ? launch_fam_t<0, 0, 0, 2, true, dfl>(warp, a, nsm, st)
                        : launch_fam_t<0, 0, 0, 2, false, dfl>(warp, a, nsm, st);
    case 3: return launch_fam_t<0, 0, 1, 1, false, dfl>(warp, a, nsm, st);
    case 4: return pure ? launch_fam_t<0, 0, 1, 2, true, dfl>(warp, a, nsm, st)
                        : launch_fam_t<0, 0, 1, 2, false, dfl>(warp, a, nsm, st);
    case 6: return launch_fam_t<0, 1, 0, 1, false, dfl>(warp, a, nsm, st);
    case 7: return pure ? launch_fam_t<0, 1, 0, 2, true, dfl>(warp, a, nsm, st)
                        : launch_fam_t<0, 1, 0, 2, false, dfl>(warp, a, nsm, st);
    case 8: return launch_fam_t<0, 1, 1, 1, false, dfl>(warp, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
