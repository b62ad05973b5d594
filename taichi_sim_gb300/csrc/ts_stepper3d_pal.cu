// Palette instantiations of the 3D stress kernels (32-bit offsets), in their
// own translation unit so that they compile in parallel with the array ones.
#include "ts_kernels3d.cuh"

namespace ts {

void launch_step_3d_pal(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts) {
    switch (ord) {
    case 2: launch_idx<2, int, true>(p, zen_mode, j, st, parts); break;
    case 3: launch_idx<3, int, true>(p, zen_mode, j, st, parts); break;
    case 4: launch_idx<4, int, true>(p, zen_mode, j, st, parts); break;
    case 5: launch_idx<5, int, true>(p, zen_mode, j, st, parts); break;
    case 6: launch_idx<6, int, true>(p, zen_mode, j, st, parts); break;
    default: break;
    }
}

}  // namespace ts
