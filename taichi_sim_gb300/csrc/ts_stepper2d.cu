// 2D staggered-grid (visco)elastic time step on sm_103a.
//
// One time step = two launches on one stream:
//   k_stress2d   : sxx, syy (normal node) and sxy (shear node) from the
//                  velocities, with the CPML convolution in the boundary
//                  strips and the Zener memory-variable update fused in;
//   k_velocity2d : vx, vy from the stresses, with CPML, Dirichlet zeroing,
//                  source injection, receiver sampling of syy and the
//                  stability bookkeeping fused in.
// Thread (threadIdx.x, threadIdx.y) owns grid node (y = 32 bx + tx,
// x = 8 by + ty); y is the contiguous axis, so a warp reads 128 contiguous
// bytes per row and the +-ORD neighbours in x come from L1/L2.
//
// Both kernels are bandwidth kernels whose speed depends on how many bytes
// each SM keeps in flight: every load a node needs (stencil values, old
// stresses, moduli, all memory variables, strip memories) is issued before
// the first store, so one memory latency is paid per node instead of one per
// dependent load.  The mechanism count is a template parameter (3, or a
// generic 8 with a runtime bound) so the memory variables live in registers.
//
// Semantics follow the reference (family TS_TAICHI2D:
// sim_taichi_elastic.py:138-309; family TS_WGSL2D:
// shader_webgpu_viscoelastic.wgsl:829-1072 and :1118-1134) with the
// divisions by dx/dy/rho/k replaced by multiplications with precomputed
// reciprocals and a*b+c contracted to fma: results agree with the
// reference's float arithmetic to rounding (checked against the CPU oracle).
#include <cuda_runtime.h>
#include "ts_internal.cuh"

namespace ts {
namespace {

constexpr int kTaichi = 0;

__device__ __forceinline__ float ldg(const float *p) { return __ldg(p); }

// b * psi + a * d, then d / k + psi
__device__ __forceinline__ float cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = fmaf(t.b, psi_old, t.a * d);
    return fmaf(d, t.ik, psi_new);
}

template <int ORD, int FAM, int ZM, int NS>
__global__ void __launch_bounds__(kBX2 *kBY2) k_stress2d(const StepParams p) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x = blockIdx.y * kBY2 + threadIdx.y;
    const bool in_n = x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1;
    const bool in_s = x >= ORD && x < p.nx - ORD + 1 && y >= ORD - 1 && y < p.ny - ORD;
    if (!in_n && !in_s) return;
    const int P = p.pitch;
    const int64_t i = (int64_t)x * P + y;
    const float *__restrict__ vx = p.v[0];
    const float *__restrict__ vy = p.v[1];
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
    const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;

    // ---------------- loads ----------------
    // per-node coefficients: no kernel writes them, so they are read before
    // waiting for the previous kernel
    float L = 0.f, M = 0.f, Ms = 0.f, gp = 1.f, gs = 1.f;
    if (in_n) {
        L = ldg(p.lam_dt + i);
        M = ldg(p.mu_dt + i);
        if (ZM == 2) gp = ldg(p.g_p + i);
    }
    if (in_s) Ms = ldg(p.mus_dt[0] + i);
    if (ZM == 2) gs = ldg(p.g_s + i);
    pdl_wait();
    float nvx[ORD][2], nvy[ORD][2], svy[ORD][2], svx[ORD][2];
    float sxx = 0.f, syy = 0.f, sxy = 0.f;
    float rxx[NS > 0 ? NS : 1], ryy[NS > 0 ? NS : 1], rxy[NS > 0 ? NS : 1];
    float psi_n[2] = {0.f, 0.f}, psi_s[2] = {0.f, 0.f};
    if (in_n) {
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            nvx[c][0] = ldg(vx + i + (int64_t)(c + 1) * P);
            nvx[c][1] = ldg(vx + i - (int64_t)c * P);
            nvy[c][0] = ldg(vy + i + c);
            nvy[c][1] = ldg(vy + i - c - 1);
        }
        sxx = p.s[0][i];
        syy = p.s[1][i];
        if (sx >= 0) psi_n[0] = p.psi[0][ix];
        if (sy >= 0) psi_n[1] = p.psi[2][iy];
        if (ZM != 0) {
#pragma unroll
            for (int l = 0; l < NS; ++l)
                if (l < n_mech) {
                    rxx[l] = p.r[0][l * p.grid_elems + i];
                    ryy[l] = p.r[1][l * p.grid_elems + i];
                }
        }
    }
    if (in_s) {
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            svy[c][0] = ldg(vy + i + (int64_t)c * P);
            svy[c][1] = ldg(vy + i - (int64_t)(c + 1) * P);
            svx[c][0] = ldg(vx + i + c + 1);
            svx[c][1] = ldg(vx + i - c);
        }
        sxy = p.s[3][i];
        if (sx >= 0) psi_s[0] = p.psi[1][ix];
        if (sy >= 0) psi_s[1] = p.psi[3][iy];
        if (ZM != 0) {
#pragma unroll
            for (int l = 0; l < NS; ++l)
                if (l < n_mech) rxy[l] = p.r[2][l * p.grid_elems + i];
        }
    }

    // ---------------- normal stresses ----------------
    if (in_n) {
        float ddx = 0.f, ddy = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            ddx = fmaf(p.cd[0][c], nvx[c][0] - nvx[c][1], ddx);
            ddy = fmaf(p.cd[1][c], nvy[c][0] - nvy[c][1], ddy);
        }
        if (sx >= 0) {
            float np_;
            ddx = cpml(ddx, psi_n[0], np_, p.tab_h[0][x]);
            p.psi[0][ix] = np_;
        }
        if (sy >= 0) {
            float np_;
            ddy = cpml(ddy, psi_n[1], np_, p.tab_f[1][y]);
            p.psi[2][iy] = np_;
        }
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
#pragma unroll
                for (int l = 0; l < NS; ++l)
                    if (l < n_mech) {
                        const float nx_ = fmaf(p.zen.Ap[l], rxx[l], (p.zen.Bp[l] * gp) * dsum);
                        const float ny_ = fmaf(p.zen.As[l], ryy[l], (p.zen.Bs[l] * gs) * ddif);
                        srxx += rxx[l] + nx_;
                        sryy += ryy[l] + ny_;
                        p.r[0][l * p.grid_elems + i] = nx_;
                        p.r[1][l * p.grid_elems + i] = ny_;
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

    // ---------------- shear stress ----------------
    if (in_s) {
        float dvy_dx = 0.f, dvx_dy = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            dvy_dx = fmaf(p.cd[0][c], svy[c][0] - svy[c][1], dvy_dx);
            dvx_dy = fmaf(p.cd[1][c], svx[c][0] - svx[c][1], dvx_dy);
        }
        if (sx >= 0) {
            float np_;
            dvy_dx = cpml(dvy_dx, psi_s[0], np_, p.tab_f[0][x]);
            p.psi[1][ix] = np_;
        }
        if (sy >= 0) {
            float np_;
            dvx_dy = cpml(dvx_dy, psi_s[1], np_, p.tab_h[1][y]);
            p.psi[3][iy] = np_;
        }
        const float e = dvy_dx + dvx_dy;
        float u = Ms * e;
        if (FAM != kTaichi && ZM != 0) {
            float sr = 0.f;
#pragma unroll
            for (int l = 0; l < NS; ++l)
                if (l < n_mech) {
                    const float n_ = fmaf(p.zen.As[l], rxy[l], (p.zen.Bs[l] * gs) * e);
                    sr += rxy[l] + n_;
                    p.r[2][l * p.grid_elems + i] = n_;
                }
            u = fmaf(0.5f * Ms, sr, u);
        }
        p.s[3][i] = sxy + u;
    }
    pdl_trigger();
}

template <int ORD, int FAM>
__global__ void __launch_bounds__(kBX2 *kBY2) k_velocity2d(const StepParams p, const int j) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x = blockIdx.y * kBY2 + threadIdx.y;
    const int tid = threadIdx.y * kBX2 + threadIdx.x;
    const int blk = blockIdx.y * gridDim.x + blockIdx.x;
    const bool live = x < p.nx && y < p.ny;
    const int P = p.pitch;
    const int64_t i = (int64_t)x * P + y;
    const float *__restrict__ sxx = p.s[0];
    const float *__restrict__ syy = p.s[1];
    const float *__restrict__ sxy = p.s[3];
    const bool in_vy = x >= ORD - 1 && x < p.nx - ORD && y >= ORD - 1 && y < p.ny - ORD;
    // Taichi zeroes each component outside its own region; the WGSL kernel
    // zeroes both outside the vy region (wgsl:1054-1057).
    const bool in_vx = FAM == kTaichi ? (x >= ORD && x < p.nx - ORD + 1 && y >= ORD && y < p.ny - ORD + 1)
                                      : (in_vy && x >= ORD && y >= ORD);
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
    const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;
    const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
    const float dx0 = in_vx ? ldg(p.dtr[0] + i) : 0.f;
    const float dy0 = in_vy ? ldg(p.dtr[1] + i) : 0.f;
    pdl_wait();
    const int k = *p.step_base + j;

    // ---------------- loads ----------------
    float ax[ORD][2], bx[ORD][2], ay[ORD][2], by[ORD][2];
    float vx0 = 0.f, vy0 = 0.f;
    float pxa = 0.f, pxb = 0.f, pya = 0.f, pyb = 0.f;
    if (in_vx) {
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            ax[c][0] = ldg(sxx + i + (int64_t)c * P);
            ax[c][1] = ldg(sxx + i - (int64_t)(c + 1) * P);
            bx[c][0] = ldg(sxy + i + c);
            bx[c][1] = ldg(sxy + i - c - 1);
        }
        vx0 = p.v[0][i];
        if (sx >= 0) pxa = p.psi[4][ix];
        if (sy >= 0) pxb = p.psi[6][iy];
    }
    if (in_vy) {
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            ay[c][0] = ldg(sxy + i + (int64_t)(c + 1) * P);
            ay[c][1] = ldg(sxy + i - (int64_t)c * P);
            by[c][0] = ldg(syy + i + c + 1);
            by[c][1] = ldg(syy + i - c);
        }
        vy0 = p.v[1][i];
        if (sx >= 0) pya = p.psi[5][ix];
        if (sy >= 0) pyb = p.psi[7][iy];
    }

    // ---------------- update ----------------
    float v2 = 0.f;
    if (live) {
        float vxn = 0.f, vyn = 0.f;
        if (in_vx) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                a = fmaf(p.cd[0][c], ax[c][0] - ax[c][1], a);
                b = fmaf(p.cd[1][c], bx[c][0] - bx[c][1], b);
            }
            if (sx >= 0) {
                float np_;
                a = cpml(a, pxa, np_, p.tab_f[0][x]);
                p.psi[4][ix] = np_;
            }
            if (sy >= 0) {
                float np_;
                b = cpml(b, pxb, np_, p.tab_f[1][y]);
                p.psi[6][iy] = np_;
            }
            vxn = fmaf(a + b, dx0, vx0);
        }
        if (in_vy) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                a = fmaf(p.cd[0][c], ay[c][0] - ay[c][1], a);
                b = fmaf(p.cd[1][c], by[c][0] - by[c][1], b);
            }
            if (sx >= 0) {
                float np_;
                a = cpml(a, pya, np_, p.tab_h[0][x]);
                p.psi[5][ix] = np_;
            }
            if (sy >= 0) {
                float np_;
                b = cpml(b, pyb, np_, p.tab_h[1][y]);
                p.psi[7][iy] = np_;
            }
            vyn = fmaf(a + b, dy0, vy0);
        }
        // sources binned to this block (few or none)
        for (int q = q0; q < q1; ++q) {
            const Source s = p.src[q];
            if (s.cell == i && k < p.src_rows)
                vyn = fmaf(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, vyn);
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

    warp_stability(v2, live && !(v2 <= p.v2_threshold), reinterpret_cast<unsigned *>(p.block_max) + blk,
                   p.first_bad, k);
    pdl_trigger();
}

template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    dim3 block(kBX2, kBY2);
    dim3 grid((p.ny + kBX2 - 1) / kBX2, (p.nx + kBY2 - 1) / kBY2);
    const bool three = p.zen.n == 3;
    if (p.family == kTaichi) {
        if (parts & 1) launch_pdl(k_stress2d<ORD, 0, 0, 0>, grid, block, st, p);
        if (parts & 2) launch_pdl(k_velocity2d<ORD, 0>, grid, block, st, p, j);
        return;
    }
    if (parts & 1) {
        if (zen_mode == 0) launch_pdl(k_stress2d<ORD, 1, 0, 0>, grid, block, st, p);
        else if (zen_mode == 1 && three) launch_pdl(k_stress2d<ORD, 1, 1, 3>, grid, block, st, p);
        else if (zen_mode == 1) launch_pdl(k_stress2d<ORD, 1, 1, kMaxSls>, grid, block, st, p);
        else if (three) launch_pdl(k_stress2d<ORD, 1, 2, 3>, grid, block, st, p);
        else launch_pdl(k_stress2d<ORD, 1, 2, kMaxSls>, grid, block, st, p);
    }
    if (parts & 2) launch_pdl(k_velocity2d<ORD, 1>, grid, block, st, p, j);
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
