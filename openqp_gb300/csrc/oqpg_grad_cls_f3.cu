// Gradient class kernels of the classes with an f shell (FP64), group 3.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_f3(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  switch (c) {
    case 45: return launch_grad_t<0, 0, 3, 3, double>(g, nsm, st);
    case 46: return launch_grad_t<0, 1, 3, 3, double>(g, nsm, st);
    case 47: return launch_grad_t<0, 2, 3, 3, double>(g, nsm, st);
    case 48: return launch_grad_t<1, 1, 3, 3, double>(g, nsm, st);
    case 49: return launch_grad_t<1, 2, 3, 3, double>(g, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
