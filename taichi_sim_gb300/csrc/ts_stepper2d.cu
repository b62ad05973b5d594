// 2D staggered-grid (visco)elastic time step on sm_103a: launch dispatch of
// the kernels in ts_kernels2d.cuh over order, family, attenuation model and
// nodes per thread.
#include <cuda_runtime.h>
#include "ts_kernels2d.cuh"

namespace ts {
namespace {

// Register budgets: the compiler's choice, except for the order-2 WGSL
// velocity kernel and the order-2 per-cell-Q three-mechanism stress kernel,
// compiled for 4 resident blocks per SM (64 registers; measured on the
// 1024^2 viscoelastic case: 43.5 against 40.1 Gcell/s).
template <int ORD, int TX>
void launch_tx(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    dim3 block(kBX2, kBY2);
    dim3 grid((p.ny + kBX2 - 1) / kBX2, (p.nx + kBY2 * TX - 1) / (kBY2 * TX));
    const bool three = p.zen.n == 3;
    if (p.family == kTaichi) {   // Taichi semantics: exact or unbiased arithmetic
        if (p.taichi_exact) {
            if (parts & 1) launch_pdl(k_stress2d<ORD, kTaichi, 0, 0, TX>, grid, block, st, p);
            if (parts & 2) launch_pdl(k_velocity2d<ORD, kTaichi, TX>, grid, block, st, p, j);
        } else {
            if (parts & 1) launch_pdl(k_stress2d<ORD, kTaichiU, 0, 0, TX>, grid, block, st, p);
            if (parts & 2) launch_pdl(k_velocity2d<ORD, kTaichiU, TX>, grid, block, st, p, j);
        }
        return;
    }
    if constexpr (ORD == 2) {   // coefficient palette (order 2 only, the benchmark's)
        if ((parts & 1) && p.pal) {
            if (zen_mode == 0) launch_pdl(k_stress2d<ORD, kWgsl, 0, 0, TX, false, 0, true>, grid, block, st, p);
            else if (zen_mode == 1 && three) launch_pdl(k_stress2d<ORD, kWgsl, 1, 3, TX, false, 0, true>, grid, block, st, p);
            else if (zen_mode == 1) launch_pdl(k_stress2d<ORD, kWgsl, 1, kMaxSls, TX, false, 0, true>, grid, block, st, p);
            else if (three) launch_pdl(k_stress2d<ORD, kWgsl, 2, 3, TX, false, 4, true>, grid, block, st, p);
            else launch_pdl(k_stress2d<ORD, kWgsl, 2, kMaxSls, TX, false, 0, true>, grid, block, st, p);
            parts &= ~1;
        }
    }
    if (parts & 1) {
        if (zen_mode == 0) launch_pdl(k_stress2d<ORD, kWgsl, 0, 0, TX>, grid, block, st, p);
        else if (zen_mode == 1 && three) launch_pdl(k_stress2d<ORD, kWgsl, 1, 3, TX>, grid, block, st, p);
        else if (zen_mode == 1) launch_pdl(k_stress2d<ORD, kWgsl, 1, kMaxSls, TX>, grid, block, st, p);
        else if (three) launch_pdl(k_stress2d<ORD, kWgsl, 2, 3, TX, false, (ORD == 2 ? 4 : 0)>, grid, block, st, p);
        else launch_pdl(k_stress2d<ORD, kWgsl, 2, kMaxSls, TX>, grid, block, st, p);
    }
    if (parts & 2) launch_pdl(k_velocity2d<ORD, kWgsl, TX, false, (ORD == 2 ? 4 : 0)>, grid, block, st, p, j);
}

template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    if (p.tx == 4) launch_tx<ORD, 4>(p, zen_mode, j, st, parts);
    else if (p.tx == 2) launch_tx<ORD, 2>(p, zen_mode, j, st, parts);
    else launch_tx<ORD, 1>(p, zen_mode, j, st, parts);
}

}  // namespace

int blocks_2d(const StepParams &p) {
    return ((p.ny + kBX2 - 1) / kBX2) * ((p.nx + kBY2 * p.tx - 1) / (kBY2 * p.tx));
}

void launch_step_2d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts) {
    switch (ord) {
    case 2: launch_ord<2>(p, zen_mode, j, st, parts); break;
    case 3: launch_ord<3>(p, zen_mode, j, st, parts); break;
    case 4: launch_ord<4>(p, zen_mode, j, st, parts); break;
    case 5: launch_ord<5>(p, zen_mode, j, st, parts); break;
    case 6: launch_ord<6>(p, zen_mode, j, st, parts); break;
    default: break;  // rejected at creation
    }
}

}  // namespace ts
