// Gradient class kernels of the classes with an f shell (FP64), group 0.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_f0(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  switch (c) {
    case 21: return launch_grad_t<0, 0, 0, 3, double>(g, nsm, st);
    case 22: return launch_grad_t<0, 1, 0, 3, double>(g, nsm, st);
    case 23: return launch_grad_t<0, 2, 0, 3, double>(g, nsm, st);
    case 24: return launch_grad_t<1, 1, 0, 3, double>(g, nsm, st);
    case 25: return launch_grad_t<1, 2, 0, 3, double>(g, nsm, st);
    case 26: return launch_grad_t<2, 2, 0, 3, double>(g, nsm, st);
    case 27: return launch_grad_t<0, 3, 0, 3, double>(g, nsm, st);
    case 28: return launch_grad_t<0, 0, 1, 3, double>(g, nsm, st);
    case 29: return launch_grad_t<0, 1, 1, 3, double>(g, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
