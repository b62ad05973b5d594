// 3D staggered-grid (visco)elastic time step on sm_103a: launches of the
// kernels in ts_kernels3d.cuh with per-coefficient arrays (the palette
// instantiations are in ts_stepper3d_pal.cu, compiled in parallel).
#include "ts_kernels3d.cuh"

namespace ts {
namespace {

// 32-bit offsets when every array (memory variables included) has fewer
// than 2^31 elements: fewer integer instructions per load.
template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    if (p.grid_elems * (int64_t)(p.zen.n > 0 ? p.zen.n : 1) < ((int64_t)1 << 31))
        launch_idx<ORD, int, false>(p, zen_mode, j, st, parts);
    else
        launch_idx<ORD, int64_t, false>(p, zen_mode, j, st, parts);
}

}  // namespace

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
    case 2: launch_ord<2>(p, zen_mode, j, st, parts); break;
    case 3: launch_ord<3>(p, zen_mode, j, st, parts); break;
    case 4: launch_ord<4>(p, zen_mode, j, st, parts); break;
    case 5: launch_ord<5>(p, zen_mode, j, st, parts); break;
    case 6: launch_ord<6>(p, zen_mode, j, st, parts); break;
    default: break;
    }
}

}  // namespace ts
