// Gradient class kernels of the classes with an f shell (FP64), group 4.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_f4(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  switch (c) {
    case 50: return launch_grad_t<2, 2, 3, 3, double>(g, nsm, st);
    case 51: return launch_grad_t<0, 3, 3, 3, double>(g, nsm, st);
    case 52: return launch_grad_t<1, 3, 3, 3, double>(g, nsm, st);
    case 53: return launch_grad_t<2, 3, 3, 3, double>(g, nsm, st);
    case 54: return launch_grad_t<3, 3, 3, 3, double>(g, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
