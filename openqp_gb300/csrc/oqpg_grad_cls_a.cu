// Gradient class kernels, classes 0-14 (one translation unit per group keeps
// the parallel build short).
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

cudaError_t launch_grad_a(int c, const GradArgs& g, bool f32, int nsm, cudaStream_t st) {
  switch (c) {
    case 0: return launch_grad_cls<0, 0, 0, 0>(g, f32, nsm, st);
    case 1: return launch_grad_cls<0, 0, 0, 1>(g, f32, nsm, st);
    case 2: return launch_grad_cls<0, 0, 0, 2>(g, f32, nsm, st);
    case 3: return launch_grad_cls<0, 0, 1, 1>(g, f32, nsm, st);
    case 4: return launch_grad_cls<0, 0, 1, 2>(g, f32, nsm, st);
    case 5: return launch_grad_cls<0, 0, 2, 2>(g, f32, nsm, st);
    case 6: return launch_grad_cls<0, 1, 0, 1>(g, f32, nsm, st);
    case 7: return launch_grad_cls<0, 1, 0, 2>(g, f32, nsm, st);
    case 8: return launch_grad_cls<0, 1, 1, 1>(g, f32, nsm, st);
    case 9: return launch_grad_cls<0, 1, 1, 2>(g, f32, nsm, st);
    case 10: return launch_grad_cls<0, 1, 2, 2>(g, f32, nsm, st);
    case 11: return launch_grad_cls<0, 2, 0, 2>(g, f32, nsm, st);
    case 12: return launch_grad_cls<0, 2, 1, 1>(g, f32, nsm, st);
    case 13: return launch_grad_cls<0, 2, 1, 2>(g, f32, nsm, st);
    case 14: return launch_grad_cls<0, 2, 2, 2>(g, f32, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oqpg
