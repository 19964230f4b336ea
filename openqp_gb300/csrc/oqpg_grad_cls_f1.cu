// Gradient class kernels of the classes with an f shell (FP64), group 1.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_f1(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  switch (c) {
    case 30: return launch_grad_t<0, 2, 1, 3, double>(g, nsm, st);
    case 31: return launch_grad_t<1, 1, 1, 3, double>(g, nsm, st);
    case 32: return launch_grad_t<1, 2, 1, 3, double>(g, nsm, st);
    case 33: return launch_grad_t<2, 2, 1, 3, double>(g, nsm, st);
    case 34: return launch_grad_t<0, 3, 1, 3, double>(g, nsm, st);
    case 35: return launch_grad_t<1, 3, 1, 3, double>(g, nsm, st);
    case 36: return launch_grad_t<0, 0, 2, 3, double>(g, nsm, st);
    case 37: return launch_grad_t<0, 1, 2, 3, double>(g, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
