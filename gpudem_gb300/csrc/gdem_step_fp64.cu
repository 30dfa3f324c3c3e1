// FP64 instantiation of the step kernel (gdem_step.cuh).  Compiled with
// -fmad=false: no multiply-add is contracted, so the linear law reproduces
// the reference CPU build (cpu_dem.cu, -ffp-contract=off) bit for bit.
#include "gdem_step.cuh"

namespace gdem {

void launch_step(const View<FP64>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    launch_step_any<FP64>(v, st, cond, use_cond);
}

StepLaunch step_launch(const View<FP64>& v, int) {
    return StepLaunch{step_kernel_any<FP64>(v), dim3((v.n + kBlock - 1) / kBlock), dim3(kBlock), 0};
}

}  // namespace gdem
