// Gradient class kernels of the classes with an f shell (FP64), group 2.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_f2(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  switch (c) {
    case 38: return launch_grad_t<0, 2, 2, 3, double>(g, nsm, st);
    case 39: return launch_grad_t<1, 1, 2, 3, double>(g, nsm, st);
    case 40: return launch_grad_t<1, 2, 2, 3, double>(g, nsm, st);
    case 41: return launch_grad_t<2, 2, 2, 3, double>(g, nsm, st);
    case 42: return launch_grad_t<0, 3, 2, 3, double>(g, nsm, st);
    case 43: return launch_grad_t<1, 3, 2, 3, double>(g, nsm, st);
    case 44: return launch_grad_t<2, 3, 2, 3, double>(g, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
