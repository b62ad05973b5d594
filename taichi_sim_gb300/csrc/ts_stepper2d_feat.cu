// The 2D step kernels of the adjoint's forward pass (family TS_WGSL2D with
// the coefficients folded with dt, kWgslFolded; p.tx nodes per thread):
// with and without the record of the per-node quantities the adjoint
// multiplies by, in their own translation unit so that they compile in
// parallel with the stepper's.
#include <cuda_runtime.h>
#include "ts_kernels2d.cuh"

namespace ts {
namespace {

template <int ORD, int MINB, int MINB_Q, int TX>
void launch_feat_mb(const StepParams &p, int zen_mode, int j, cudaStream_t st) {
    const dim3 block(kBX2, kBY2), grid((p.ny + kBX2 - 1) / kBX2, (p.nx + kBY2 * TX - 1) / (kBY2 * TX));
    const bool three = p.zen.n == 3;
    if (zen_mode == 0) launch_pdl(k_stress2d<ORD, kWgslFolded, 0, 0, TX, true, MINB>, grid, block, st, p);
    else if (zen_mode == 1 && three) launch_pdl(k_stress2d<ORD, kWgslFolded, 1, 3, TX, true, MINB>, grid, block, st, p);
    else if (zen_mode == 1) launch_pdl(k_stress2d<ORD, kWgslFolded, 1, kMaxSls, TX, true, MINB_Q>, grid, block, st, p);
    else if (three) launch_pdl(k_stress2d<ORD, kWgslFolded, 2, 3, TX, true, MINB_Q>, grid, block, st, p);
    else launch_pdl(k_stress2d<ORD, kWgslFolded, 2, kMaxSls, TX, true, MINB_Q>, grid, block, st, p);
    launch_pdl(k_velocity2d<ORD, kWgslFolded, TX, true, MINB>, grid, block, st, p, j);
}

// the same step without the record (the forward's unrecorded segments)
template <int ORD, int TX>
void launch_folded_tx(const StepParams &p, int zen_mode, int j, cudaStream_t st) {
    constexpr int MB = ORD == 2 ? 4 : 0;
    const dim3 block(kBX2, kBY2), grid((p.ny + kBX2 - 1) / kBX2, (p.nx + kBY2 * TX - 1) / (kBY2 * TX));
    const bool three = p.zen.n == 3;
    if (zen_mode == 0) launch_pdl(k_stress2d<ORD, kWgslFolded, 0, 0, TX>, grid, block, st, p);
    else if (zen_mode == 1 && three) launch_pdl(k_stress2d<ORD, kWgslFolded, 1, 3, TX>, grid, block, st, p);
    else if (zen_mode == 1) launch_pdl(k_stress2d<ORD, kWgslFolded, 1, kMaxSls, TX>, grid, block, st, p);
    else if (three) launch_pdl(k_stress2d<ORD, kWgslFolded, 2, 3, TX, false, MB>, grid, block, st, p);
    else launch_pdl(k_stress2d<ORD, kWgslFolded, 2, kMaxSls, TX>, grid, block, st, p);
    launch_pdl(k_velocity2d<ORD, kWgslFolded, TX, false, MB>, grid, block, st, p, j);
}

// Nodes per thread (p.tx): 1 or 2 at order 2 (adjoint_nodes_per_thread), 2 above.
template <int ORD>
void launch_folded(const StepParams &p, int zen_mode, int j, cudaStream_t st) {
    if (ORD == 2 && p.tx == 1) launch_folded_tx<ORD, 1>(p, zen_mode, j, st);
    else launch_folded_tx<ORD, 2>(p, zen_mode, j, st);
}

// Register budget: order 2 takes 4 resident blocks per SM (64 registers:
// the velocity kernel and the elastic and three-mechanism stress kernels
// spill at most 12 bytes) except where the per-cell scales or eight
// mechanisms would spill more (3 blocks); orders 3 and 4 take 3 blocks,
// which spills nothing; orders 5 and 6 keep the compiler's choice.
template <int ORD>
void launch_feat(const StepParams &p, int zen_mode, int j, cudaStream_t st) {
    constexpr int mb = ORD == 2 ? 4 : (ORD <= 4 ? 3 : 0);
    constexpr int mbq = ORD <= 4 ? 3 : 0;
    if (ORD == 2 && p.tx == 1) launch_feat_mb<ORD, mb, mbq, 1>(p, zen_mode, j, st);
    else launch_feat_mb<ORD, mb, mbq, 2>(p, zen_mode, j, st);
}

}  // namespace

void launch_step_2d_folded(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st) {
    switch (ord) {   // the adjoint serves orders 2 and 4
    case 2: launch_folded<2>(p, zen_mode, j, st); break;
    case 4: launch_folded<4>(p, zen_mode, j, st); break;
    default: break;
    }
}

void launch_step_2d_feat(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st) {
    switch (ord) {
    case 2: launch_feat<2>(p, zen_mode, j, st); break;
    case 3: launch_feat<3>(p, zen_mode, j, st); break;
    case 4: launch_feat<4>(p, zen_mode, j, st); break;
    case 5: launch_feat<5>(p, zen_mode, j, st); break;
    case 6: launch_feat<6>(p, zen_mode, j, st); break;
    default: break;  // rejected at creation
    }
}

}  // namespace ts
