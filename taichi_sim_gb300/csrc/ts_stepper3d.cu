// 3D staggered-grid (visco)elastic time step on sm_103a: launch dispatch of
// the kernels in ts_kernels3d.cuh.  Per-coefficient arrays: order 2 here,
// orders 3 to 6 in ts_stepper3d_o<N>.cu; the palette instantiations are in
// ts_stepper3d_pal.cu (all compiled in parallel).
#include "ts_stepper3d_arrays.cuh"

namespace ts {

int blocks_3d(const StepParams &p) {
    return ((p.nz + kZB3 - 1) / kZB3) * ((p.ny + kYB3 - 1) / kYB3) * ((p.nx + p.tx - 1) / p.tx);
}

void launch_step_3d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts) {
    if (p.pal) {   // palette stress kernels, then the velocity kernel
        if (parts & 1) launch_step_3d_pal(p, ord, zen_mode, j, st, 1);
        if (!(parts & 2)) return;
        parts = 2;
    }
    switch (ord) {
    case 2: launch_arrays<2>(p, zen_mode, j, st, parts); break;
    case 3: launch_step_3d_arrays_3(p, zen_mode, j, st, parts); break;
    case 4: launch_step_3d_arrays_4(p, zen_mode, j, st, parts); break;
    case 5: launch_step_3d_arrays_5(p, zen_mode, j, st, parts); break;
    case 6: launch_step_3d_arrays_6(p, zen_mode, j, st, parts); break;
    default: break;
    }
}

}  // namespace ts
