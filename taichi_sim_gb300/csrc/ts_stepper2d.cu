// 2D staggered-grid (visco)elastic time step on sm_103a.
//
// One time step = two launches on one stream:
//   k_stress2d   : sxx, syy (normal node) and sxy (shear node) from the
//                  velocities, with the CPML convolution in the boundary
//                  strips and the Zener memory-variable update fused in;
//   k_velocity2d : vx, vy from the stresses, with CPML, Dirichlet zeroing,
//                  source injection, receiver sampling of syy and the
//                  stability bookkeeping fused in.
// Both kernels are HBM-streaming: thread (threadIdx.x, threadIdx.y) owns
// grid node (y = 32 bx + tx, x = 8 by + ty); y is the contiguous axis, so a
// warp reads 128 contiguous bytes per row and the +-ORD neighbours in x hit
// L1/L2 from the rows the block's other warps stream.
//
// Semantics follow the reference (family TS_TAICHI2D:
// sim_taichi_elastic.py:138-309; family TS_WGSL2D:
// shader_webgpu_viscoelastic.wgsl:829-1072 and :1118-1134) with the
// division by dx/dy/rho/k replaced by multiplication with precomputed
// reciprocals and a*b+c contracted to fma: results agree with the
// reference's float arithmetic to rounding (checked against the CPU oracle).
#include <cuda_runtime.h>
#include "ts_internal.cuh"

namespace ts {
namespace {

constexpr int kTaichi = 0;

__device__ __forceinline__ float cpml_update(float d, float *psi, const Cpml &t) {
    float p = fmaf(t.b, *psi, t.a * d);
    *psi = p;
    return fmaf(d, t.ik, p);
}

template <int ORD, int FAM, int ZM>
__global__ void __launch_bounds__(kBX2 *kBY2) k_stress2d(const StepParams p) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x = blockIdx.y * kBY2 + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const int P = p.pitch;
    const int64_t i = (int64_t)x * P + y;
    const float *__restrict__ vx = p.v[0];
    const float *__restrict__ vy = p.v[1];

    // ---- normal stresses: x in [ORD-1, nx-ORD), y in [ORD, ny-ORD+1) ----
    if (x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1) {
        float ddx = 0.f, ddy = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            ddx = fmaf(p.cd[0][c], __ldg(vx + i + (int64_t)(c + 1) * P) - __ldg(vx + i - (int64_t)c * P), ddx);
            ddy = fmaf(p.cd[1][c], __ldg(vy + i + c) - __ldg(vy + i - c - 1), ddy);
        }
        const int sx = strip_index(p.strip[0], x);
        if (sx >= 0) ddx = cpml_update(ddx, p.psi[0] + (int64_t)sx * P + y, p.tab_h[0][x]);
        const int sy = strip_index(p.strip[1], y);
        if (sy >= 0) ddy = cpml_update(ddy, p.psi[2] + (int64_t)x * p.strip[1].width + sy, p.tab_f[1][y]);
        const float L = __ldg(p.lam_dt + i), M = __ldg(p.mu_dt + i);
        float sxx = p.s[0][i], syy = p.s[1][i];
        if (FAM == kTaichi) {
            const float dl = L * (ddx + ddy);
            sxx += fmaf(2.f * M, ddx, dl);
            syy += fmaf(2.f * M, ddy, dl);
        } else {
            const float L2M = fmaf(2.f, M, L);
            float ux = fmaf(L2M, ddx, L * ddy);
            float uy = fmaf(L, ddx, L2M * ddy);
            if (ZM != 0) {
                float srxx = 0.f, sryy = 0.f;
                const float dsum = ddx + ddy, ddif = 0.5f * (ddx - ddy);
                const float gp = ZM == 2 ? __ldg(p.g_p + i) : 1.f;
                const float gs = ZM == 2 ? __ldg(p.g_s + i) : 1.f;
#pragma unroll
                for (int l = 0; l < kMaxSls; ++l) {
                    if (l >= p.zen.n) break;
                    float *rx = p.r[0] + l * p.grid_elems + i;
                    float *ry = p.r[1] + l * p.grid_elems + i;
                    const float ox = *rx, oy = *ry;
                    const float nx_ = fmaf(p.zen.Ap[l], ox, (p.zen.Bp[l] * gp) * dsum);
                    const float ny_ = fmaf(p.zen.As[l], oy, (p.zen.Bs[l] * gs) * ddif);
                    srxx += ox + nx_;
                    sryy += oy + ny_;
                    *rx = nx_;
                    *ry = ny_;
                }
                const float half_lpm = 0.5f * (L + M);
                ux = fmaf(half_lpm, srxx, fmaf(M, sryy, ux));
                uy = fmaf(half_lpm, srxx, fmaf(-M, sryy, uy));
            }
            sxx += ux;
            syy += uy;
        }
        p.s[0][i] = sxx;
        p.s[1][i] = syy;
    }

    // ---- shear stress: x in [ORD, nx-ORD+1), y in [ORD-1, ny-ORD) ----
    if (x >= ORD && x < p.nx - ORD + 1 && y >= ORD - 1 && y < p.ny - ORD) {
        float dvy_dx = 0.f, dvx_dy = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            dvy_dx = fmaf(p.cd[0][c], __ldg(vy + i + (int64_t)c * P) - __ldg(vy + i - (int64_t)(c + 1) * P), dvy_dx);
            dvx_dy = fmaf(p.cd[1][c], __ldg(vx + i + c + 1) - __ldg(vx + i - c), dvx_dy);
        }
        const int sx = strip_index(p.strip[0], x);
        if (sx >= 0) dvy_dx = cpml_update(dvy_dx, p.psi[1] + (int64_t)sx * P + y, p.tab_f[0][x]);
        const int sy = strip_index(p.strip[1], y);
        if (sy >= 0) dvx_dy = cpml_update(dvx_dy, p.psi[3] + (int64_t)x * p.strip[1].width + sy, p.tab_h[1][y]);
        const float Ms = __ldg(p.mus_dt[0] + i);
        const float e = dvy_dx + dvx_dy;
        float u = Ms * e;
        if (FAM != kTaichi && ZM != 0) {
            float sr = 0.f;
            const float gs = ZM == 2 ? __ldg(p.g_s + i) : 1.f;
#pragma unroll
            for (int l = 0; l < kMaxSls; ++l) {
                if (l >= p.zen.n) break;
                float *rr = p.r[2] + l * p.grid_elems + i;
                const float o = *rr;
                const float n_ = fmaf(p.zen.As[l], o, (p.zen.Bs[l] * gs) * e);
                sr += o + n_;
                *rr = n_;
            }
            u = fmaf(0.5f * Ms, sr, u);
        }
        p.s[3][i] += u;
    }
}

template <int ORD, int FAM>
__global__ void __launch_bounds__(kBX2 *kBY2) k_velocity2d(const StepParams p, const int j) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x = blockIdx.y * kBY2 + threadIdx.y;
    const int tid = threadIdx.y * kBX2 + threadIdx.x;
    const int blk = blockIdx.y * gridDim.x + blockIdx.x;
    const int k = *p.step_base + j;
    const bool live = x < p.nx && y < p.ny;
    const int P = p.pitch;
    const int64_t i = (int64_t)x * P + y;
    const float *__restrict__ sxx = p.s[0];
    const float *__restrict__ syy = p.s[1];
    const float *__restrict__ sxy = p.s[3];
    float v2 = 0.f;

    if (live) {
        const bool in_vy = x >= ORD - 1 && x < p.nx - ORD && y >= ORD - 1 && y < p.ny - ORD;
        // Taichi zeroes each component outside its own region; the WGSL
        // kernel zeroes both outside the vy region (wgsl:1054-1057).
        const bool in_vx = FAM == kTaichi ? (x >= ORD && x < p.nx - ORD + 1 && y >= ORD && y < p.ny - ORD + 1)
                                          : (in_vy && x >= ORD && y >= ORD);
        float vxn = 0.f, vyn = 0.f;
        if (in_vx) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                a = fmaf(p.cd[0][c], __ldg(sxx + i + (int64_t)c * P) - __ldg(sxx + i - (int64_t)(c + 1) * P), a);
                b = fmaf(p.cd[1][c], __ldg(sxy + i + c) - __ldg(sxy + i - c - 1), b);
            }
            const int sx = strip_index(p.strip[0], x);
            if (sx >= 0) a = cpml_update(a, p.psi[4] + (int64_t)sx * P + y, p.tab_f[0][x]);
            const int sy = strip_index(p.strip[1], y);
            if (sy >= 0) b = cpml_update(b, p.psi[6] + (int64_t)x * p.strip[1].width + sy, p.tab_f[1][y]);
            vxn = fmaf(a + b, __ldg(p.dtr[0] + i), p.v[0][i]);
        }
        if (in_vy) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                a = fmaf(p.cd[0][c], __ldg(sxy + i + (int64_t)(c + 1) * P) - __ldg(sxy + i - (int64_t)c * P), a);
                b = fmaf(p.cd[1][c], __ldg(syy + i + c + 1) - __ldg(syy + i - c), b);
            }
            const int sx = strip_index(p.strip[0], x);
            if (sx >= 0) a = cpml_update(a, p.psi[5] + (int64_t)sx * P + y, p.tab_h[0][x]);
            const int sy = strip_index(p.strip[1], y);
            if (sy >= 0) b = cpml_update(b, p.psi[7] + (int64_t)x * p.strip[1].width + sy, p.tab_h[1][y]);
            vyn = fmaf(a + b, __ldg(p.dtr[1] + i), p.v[1][i]);
        }
        // sources binned to this block (few or none)
        const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
        for (int q = q0; q < q1; ++q) {
            const Source s = p.src[q];
            if (s.cell == i && k < p.src_rows) vyn = fmaf(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, vyn);
        }
        p.v[0][i] = vxn;
        p.v[1][i] = vyn;
        v2 = fmaf(vxn, vxn, vyn * vyn);
    }

    // receivers: global thread g samples receiver g (syy is final for step k)
    const int g = blk * (kBX2 * kBY2) + tid;
    if (g < p.n_rec && k >= __ldg(p.rec_first_step + g)) {
        float acc = 0.f;
        for (int q = __ldg(p.rec_start + g); q < __ldg(p.rec_start + g + 1); ++q) acc += syy[__ldg(p.rec_cell + q)];
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }

    // stability bookkeeping: block max of |v|^2 and first unstable step
    const bool bad = live && !(v2 <= p.v2_threshold);
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v2));
    __shared__ unsigned wmax[kBX2 * kBY2 / 32];
    if ((tid & 31) == 0) wmax[tid >> 5] = m;
    const int any_bad = __syncthreads_or(bad);
    if (tid == 0) {
        unsigned bm = wmax[0];
#pragma unroll
        for (int w = 1; w < kBX2 * kBY2 / 32; ++w) bm = max(bm, wmax[w]);
        unsigned *slot = reinterpret_cast<unsigned *>(p.block_max) + blk;
        *slot = max(*slot, bm);
        if (any_bad) atomicMin(p.first_bad, k);
    }
}

template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    dim3 block(kBX2, kBY2);
    dim3 grid((p.ny + kBX2 - 1) / kBX2, (p.nx + kBY2 - 1) / kBY2);
    if (p.family == kTaichi) {
        if (parts & 1) k_stress2d<ORD, 0, 0><<<grid, block, 0, st>>>(p);
        if (parts & 2) k_velocity2d<ORD, 0><<<grid, block, 0, st>>>(p, j);
    } else {
        if (parts & 1) {
            if (zen_mode == 0) k_stress2d<ORD, 1, 0><<<grid, block, 0, st>>>(p);
            else if (zen_mode == 1) k_stress2d<ORD, 1, 1><<<grid, block, 0, st>>>(p);
            else k_stress2d<ORD, 1, 2><<<grid, block, 0, st>>>(p);
        }
        if (parts & 2) k_velocity2d<ORD, 1><<<grid, block, 0, st>>>(p, j);
    }
}

}  // namespace

int blocks_2d(const StepParams &p) { return ((p.ny + kBX2 - 1) / kBX2) * ((p.nx + kBY2 - 1) / kBY2); }

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
