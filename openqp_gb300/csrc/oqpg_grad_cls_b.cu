// Gradient class kernels, classes 15-20.
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_b(int c, const GradArgs& g, bool f32, int nsm, cudaStream_t st) {
  switch (c) {
    case 15: return launch_grad_cls<1, 1, 1, 1>(g, f32, nsm, st);
    case 16: return launch_grad_cls<1, 1, 1, 2>(g, f32, nsm, st);
    case 17: return launch_grad_cls<1, 1, 2, 2>(g, f32, nsm, st);
    case 18: return launch_grad_cls<1, 2, 1, 2>(g, f32, nsm, st);
    case 19: return launch_grad_cls<1, 2, 2, 2>(g, f32, nsm, st);
    case 20: return launch_grad_cls<2, 2, 2, 2>(g, f32, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
