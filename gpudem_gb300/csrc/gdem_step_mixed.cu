// Mixed-precision instantiation of the step kernel (gdem_step.cuh): FP64
// positions and integration, FP32 contact math, compensated spring history.
// Compiled with multiply-add contraction on.
#include "gdem_step.cuh"

namespace gdem {

void launch_step(const View<Mixed>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    launch_step_any<Mixed>(v, st, cond, use_cond);
}

void* step_kernel(const View<Mixed>& v) { return step_kernel_any<Mixed>(v); }

}  // namespace gdem
