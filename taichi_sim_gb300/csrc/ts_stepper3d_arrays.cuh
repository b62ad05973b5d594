// The array-coefficient launches of the 3D kernels for one stencil order
// (internal header: ts_stepper3d.cu serves order 2, ts_stepper3d_o<N>.cu
// order N, so that the orders compile in parallel).
#pragma once
#include "ts_kernels3d.cuh"

namespace ts {
namespace {

// 32-bit offsets when every array (memory variables included) has fewer
// than 2^31 elements: fewer integer instructions per load.
template <int ORD>
void launch_arrays(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    if (p.grid_elems * (int64_t)(p.zen.n > 0 ? p.zen.n : 1) < ((int64_t)1 << 31))
        launch_idx<ORD, int, false>(p, zen_mode, j, st, parts);
    else
        launch_idx<ORD, int64_t, false>(p, zen_mode, j, st, parts);
}

}  // namespace
}  // namespace ts
