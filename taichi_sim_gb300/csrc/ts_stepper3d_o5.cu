// Array-coefficient launches of the 3D kernels for stencil order 5, in a
// translation unit of their own so that the orders compile in parallel.
#include "ts_stepper3d_arrays.cuh"

namespace ts {

void launch_step_3d_arrays_5(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    launch_arrays<5>(p, zen_mode, j, st, parts);
}

}  // namespace ts
