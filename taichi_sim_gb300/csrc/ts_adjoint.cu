// Discrete adjoint of the 2D (visco)elastic stepper (family TS_WGSL2D):
// gradient of a receiver-trace misfit with respect to the per-node
// coefficients the stepper uses, L = lambda*dt and M = mu*dt at the normal
// node, Ms = mu*dt at the shear node, Bx = dt/rho at the vx node and
// By = dt/rho at the vy node.  (A caller maps per-cell lambda, mu, rho to
// these with the reference's averaging and chains the gradient back.)
//
// Forward step n (shader_webgpu_viscoelastic.wgsl:829-1072), run by the
// stepper's own kernels (ts_kernels2d.cuh):
//   stress:   d~ = ik d + p',  p' = b p + a d         (CPML, per derivative)
//             r'_l = A_l r_l + C_l g drive,  S = sum_l (r_l + r'_l)
//             sxx' = sxx + (L+2M) dx + L dy + (L+M)/2 Sxx + M Syy
//             syy' = syy + L dx + (L+2M) dy + (L+M)/2 Sxx - M Syy
//             sxy' = sxy + Ms e + Ms/2 Sxy,  e = dvy/dx~ + dvx/dy~
//   velocity: vx' = vx + Bx ax,  vy' = vy + By ay (+ source f_n By),
//             zero outside their regions
//   receivers: trace_n = sum of syy' over each receiver's nodes.
// The update is linear in the state, so the adjoint runs the transposed
// operators backward in time and needs from the forward pass only what
// multiplies the coefficients (the record, 6 floats per node and step; see
// kFeat*).  The record of every step is kept when the caller asks for it
// (GB300's HBM holds a 512 x 1024 x 3000-step record in 38 GB); otherwise
// the forward state is checkpointed every K steps and each K-step segment
// is recomputed, recording, before its adjoint sweep (revolve-style,
// K ~ sqrt(steps)); the last segment records during the forward pass, since
// its sweep comes first.
//
// Adjoint step n, from the adjoints of the state after step n, as two
// launches (same block shape and x-marching as the forward):
//   k_adj_velocity: velocity nodes - vbar gathers the transposed stress
//       stencils of step n+1 (their CPML-adjusted adjoints, written by the
//       previous k_adj_stress; zero before the first); then abar = B vbar,
//       gB += vbar * record, CPML adjoint (q = pbar + abar,
//       dbar = ik abar + a q, pbar <- b q) -> the velocity-node adjoint
//       arrays; the receiver residuals of step n enter syy^bar.
//   k_adj_stress: stress nodes - sbar gathers the transposed velocity
//       stencils; gL, gM, gMs accumulate; Zener adjoint
//       (rho_l = rbar_l + Sbar, rbar_l <- A_l rho_l + Sbar,
//       drive^bar += C_l g rho_l); CPML adjoint -> the stress-node arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/taichi_sim_gb300.h"
#include "ts_internal.cuh"
#include "ts_kernels2d.cuh"
#include "ts_prep.h"

namespace ts {
namespace {

constexpr int kAdjTx = 1;  // nodes per thread along x of the adjoint kernels

// Everything the adjoint kernels read, passed by value.
struct AdjState {
    int nx, ny, P;
    int64_t G;
    float cd[2][kMaxOrd];
    Zener zen;
    const Cpml *tab_f[2], *tab_h[2];
    Strip strip[2];
    const float *L, *M, *Ms, *Bx, *By, *gp, *gs;
    // sources, binned by block as for the forward
    const Source *src;
    const int *src_block_start;
    const float *src_tab;
    int src_rows, src_ncol;
    // receivers and their residuals [rows][n_rec]
    int n_rec;
    const int *rec_start;
    const int64_t *rec_cell;
    const int *rec_first;
    const float *res;
    // adjoint state: fields, memory variables, strip memories
    float *avx, *avy, *asxx, *asyy, *asxy, *ar[3], *apsi[8];
    // CPML-adjusted adjoints of the stencil outputs, zero outside their regions:
    // stress nodes: dx~ (normal), dy~ (normal), dvy/dx~ (shear), dvx/dy~ (shear)
    float *dv[4];
    // velocity nodes: dsxx/dx~, dsxy/dy~ (vx), dsxy/dx~, dsyy/dy~ (vy)
    float *ds[4];
    float *gL, *gM, *gMs, *gBx, *gBy;
};

// adjoint of cpml(): given the adjoint of d~ and the carried adjoint of p',
// returns the adjoint of d and leaves in pbar the adjoint of the previous p'
__device__ __forceinline__ float cpml_adj(float dt_bar, float &pbar, const Cpml &t) {
    const float q = pbar + dt_bar;
    pbar = t.b * q;
    return fmaf(t.ik, dt_bar, t.a * q);
}

// f[row + yy], zero outside [0, ny) (no wrap into the neighbouring row); f
// is written by the previous kernel of the stream: a coherent load
__device__ __forceinline__ float ld_y(const float *f, int64_t row, int yy, int ny) {
    return (yy >= 0 && yy < ny) ? __ldca(f + row + yy) : 0.f;
}

template <int ORD, int TX, int MINB>
__global__ void __launch_bounds__(kBX2 *kBY2, MINB) k_adj_velocity(const AdjState a, const float *rec, int k) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x0 = (blockIdx.y * kBY2 + threadIdx.y) * TX;
    const int tid = threadIdx.y * kBX2 + threadIdx.x;
    const int blk = blockIdx.y * gridDim.x + blockIdx.x;
    const int P = a.P, nx = a.nx, ny = a.ny;
    const int64_t G = a.G;
    const bool live_col = y < ny;
    const bool yvy = y >= ORD - 1 && y < ny - ORD;
    const bool yvx = yvy && y >= ORD;
    const int sy = live_col ? strip_index(a.strip[1], y) : -1;
    const int q0 = __ldg(a.src_block_start + blk), q1 = __ldg(a.src_block_start + blk + 1);
    // warps wholly in the interior (no source node in the block) sweep
    // without per-node region, strip, bounds or source tests
    const bool fast = interior_warp<ORD, TX>(a, y, x0, sy) && q0 == q1;
    pdl_wait();
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // dx~ adjoints rows [x-ORD, x+ORD-1] (vx), dvy/dx~ adjoints rows [x-ORD+1, x+ORD] (vy)
        float wdx[2 * ORD], wex[2 * ORD];
        load_window<ORD, !FAST>(wdx, a.dv[0], x0 - ORD, nx, P, y);
        load_window<ORD, !FAST>(wex, a.dv[2], x0 - ORD + 1, nx, P, y);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (!FAST && x >= nx) break;
            const int64_t row = (int64_t)x * P, i = row + y;
            const bool in_vy = FAST || (yvy && x >= ORD - 1 && x < nx - ORD);
            const bool in_vx = FAST || (yvx && in_vy && x >= ORD);
            const int sx = FAST ? -1 : strip_index(a.strip[0], x);
            const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * a.strip[1].width + syl;
            // ---- loads ----
            float dey[2 * ORD], dvy[2 * ORD];
#pragma unroll
            for (int c = 0; c < 2 * ORD; ++c)   // y-ORD .. y+ORD-1
                dey[c] = FAST ? __ldca(a.dv[3] + row + y - ORD + c) : ld_y(a.dv[3], row, y - ORD + c, ny);
#pragma unroll
            for (int c = 0; c < 2 * ORD; ++c)   // y-ORD+1 .. y+ORD
                dvy[c] = FAST ? __ldca(a.dv[1] + row + y - ORD + 1 + c) : ld_y(a.dv[1], row, y - ORD + 1 + c, ny);
            float avx = a.avx[i], avy = a.avy[i];
            float bx = 0.f, by = 0.f, fax = 0.f, fay = 0.f, gbx = 0.f, gby = 0.f;
            float pxa = 0.f, pxb = 0.f, pya = 0.f, pyb = 0.f;
            if (in_vx) {
                bx = __ldg(a.Bx + i);
                fax = __ldca(rec + kFeatVx * G + i);
                gbx = a.gBx[i];
                if (sx >= 0) pxa = a.apsi[4][ix];
                if (syl >= 0) pxb = a.apsi[6][iy];
            }
            if (in_vy) {
                by = __ldg(a.By + i);
                fay = __ldca(rec + kFeatVy * G + i);
                if (sx >= 0) pya = a.apsi[5][ix];
                if (syl >= 0) pyb = a.apsi[7][iy];
            }
            // ---- transposed stress stencils of the next step ----
            float gx = 0.f, gy = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                gx = fmaf(a.cd[0][c], wdx[ORD - 1 - c] - wdx[ORD + c], gx);
                gx = fmaf(a.cd[1][c], dey[ORD - 1 - c] - dey[ORD + c], gx);
                gy = fmaf(a.cd[1][c], dvy[ORD - 1 - c] - dvy[ORD + c], gy);
                gy = fmaf(a.cd[0][c], wex[ORD - 1 - c] - wex[ORD + c], gy);
            }
            avx += gx;
            avy += gy;
            // ---- velocity update of this step, transposed ----
            float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
            if (in_vx) {
                const float ab = bx * avx;
                a.gBx[i] = fmaf(avx, fax, gbx);
                d0 = ab;
                d1 = ab;
                if (sx >= 0) {
                    d0 = cpml_adj(ab, pxa, a.tab_f[0][x]);
                    a.apsi[4][ix] = pxa;
                }
                if (syl >= 0) {
                    d1 = cpml_adj(ab, pxb, a.tab_f[1][y]);
                    a.apsi[6][iy] = pxb;
                }
            }
            float gsrc = 0.f;
            if constexpr (!FAST) {
                for (int q = q0; q < q1; ++q) {
                    const Source s = a.src[q];
                    if (s.cell == i && k < a.src_rows)
                        gsrc = fmaf(avy, __ldg(a.src_tab + (int64_t)k * a.src_ncol + s.col), gsrc);
                }
            }
            if (in_vy) {
                const float ab = by * avy;
                gby = fmaf(avy, fay, gsrc);
                d2 = ab;
                d3 = ab;
                if (sx >= 0) {
                    d2 = cpml_adj(ab, pya, a.tab_h[0][x]);
                    a.apsi[5][ix] = pya;
                }
                if (syl >= 0) {
                    d3 = cpml_adj(ab, pyb, a.tab_h[1][y]);
                    a.apsi[7][iy] = pyb;
                }
                a.gBy[i] += gby;
            } else if (q1 > q0 && gsrc != 0.f) {
                a.gBy[i] += gsrc;   // a source outside the vy region: vy = f By
            }
            a.ds[0][i] = d0;
            a.ds[1][i] = d1;
            a.ds[2][i] = d2;
            a.ds[3][i] = d3;
            // the forward overwrote v outside the updated regions
            a.avx[i] = in_vx ? avx : 0.f;
            a.avy[i] = in_vy ? avy : 0.f;
            if (t + 1 < TX) {
                shift_window<ORD, !FAST>(wdx, a.dv[0], x + ORD, nx, P, y);
                shift_window<ORD, !FAST>(wex, a.dv[2], x + ORD + 1, nx, P, y);
            }
        }
    };
    if (fast) sweep(std::true_type{});
    else if (live_col && x0 < nx) sweep(std::false_type{});
    // residuals of step k into syy^bar: global thread g injects receiver g
    const int g = blk * (kBX2 * kBY2) + tid;
    if (g < a.n_rec && k >= __ldg(a.rec_first + g)) {
        const float r = __ldg(a.res + (int64_t)k * a.n_rec + g);
        for (int q = __ldg(a.rec_start + g); q < __ldg(a.rec_start + g + 1); ++q)
            atomicAdd(a.asyy + __ldg(a.rec_cell + q), r);
    }
    pdl_trigger();
}

template <int ORD, int ZM, int NS, int TX, int MINB>
__global__ void __launch_bounds__(kBX2 *kBY2, MINB) k_adj_stress(const AdjState a, const float *rec) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x0 = (blockIdx.y * kBY2 + threadIdx.y) * TX;
    const int sy = y < a.ny ? strip_index(a.strip[1], y) : -1;
    const bool fast = interior_warp<ORD, TX>(a, y, x0, sy);
    if (y >= a.ny || x0 >= a.nx) return;
    const int P = a.P, nx = a.nx, ny = a.ny;
    const int64_t G = a.G;
    const int n_mech = NS == 3 ? 3 : a.zen.n;
    constexpr int R = NS > 0 ? NS : 1;
    const bool yn = y >= ORD && y < ny - ORD + 1;
    const bool ys = y >= ORD - 1 && y < ny - ORD;
    pdl_wait();
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // dsxx/dx~ adjoints rows [x-ORD+1, x+ORD], dsxy/dx~ adjoints rows [x-ORD, x+ORD-1]
        float wax[2 * ORD], way[2 * ORD];
        load_window<ORD, !FAST>(wax, a.ds[0], x0 - ORD + 1, nx, P, y);
        load_window<ORD, !FAST>(way, a.ds[2], x0 - ORD, nx, P, y);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (!FAST && x >= nx) break;
            const int64_t row = (int64_t)x * P, i = row + y;
            const bool in_n = FAST || (yn && x >= ORD - 1 && x < nx - ORD);
            const bool in_s = FAST || (ys && x >= ORD && x < nx - ORD + 1);
            const int sx = FAST ? -1 : strip_index(a.strip[0], x);
            const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * a.strip[1].width + syl;
            // ---- loads ----
            float axy[2 * ORD], ayy[2 * ORD];
#pragma unroll
            for (int c = 0; c < 2 * ORD; ++c)   // y-ORD+1 .. y+ORD
                axy[c] = FAST ? __ldca(a.ds[1] + row + y - ORD + 1 + c) : ld_y(a.ds[1], row, y - ORD + 1 + c, ny);
#pragma unroll
            for (int c = 0; c < 2 * ORD; ++c)   // y-ORD .. y+ORD-1
                ayy[c] = FAST ? __ldca(a.ds[3] + row + y - ORD + c) : ld_y(a.ds[3], row, y - ORD + c, ny);
            float sxx = a.asxx[i], syy = a.asyy[i], sxy = a.asxy[i];
            float L = 0.f, M = 0.f, Ms = 0.f, gp = 1.f, gs = 1.f, fl = 0.f, fmx = 0.f, fmy = 0.f, fsh = 0.f;
            float gl = 0.f, gm = 0.f, gms = 0.f, pn0 = 0.f, pn1 = 0.f, ps0 = 0.f, ps1 = 0.f;
            float rxx[R], ryy[R], rxy[R];
            if (in_n) {
                L = __ldg(a.L + i);
                M = __ldg(a.M + i);
                if (ZM == 2) gp = __ldg(a.gp + i);
                fl = __ldca(rec + kFeatLam * G + i);
                fmx = __ldca(rec + kFeatMuX * G + i);
                fmy = __ldca(rec + kFeatMuY * G + i);
                gl = a.gL[i];
                gm = a.gM[i];
                if (sx >= 0) pn0 = a.apsi[0][ix];
                if (syl >= 0) pn1 = a.apsi[2][iy];
                if (ZM != 0) {
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            rxx[l] = a.ar[0][l * G + i];
                            ryy[l] = a.ar[1][l * G + i];
                        }
                }
            }
            if (in_s) {
                Ms = __ldg(a.Ms + i);
                fsh = __ldca(rec + kFeatShear * G + i);
                gms = a.gMs[i];
                if (sx >= 0) ps0 = a.apsi[1][ix];
                if (syl >= 0) ps1 = a.apsi[3][iy];
                if (ZM != 0) {
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) rxy[l] = a.ar[2][l * G + i];
                }
            }
            if (ZM == 2 && (in_n || in_s)) gs = __ldg(a.gs + i);
            // ---- transposed velocity stencils of this step ----
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                sxx = fmaf(a.cd[0][c], wax[ORD - 1 - c] - wax[ORD + c], sxx);
                sxy = fmaf(a.cd[1][c], axy[ORD - 1 - c] - axy[ORD + c], sxy);
                sxy = fmaf(a.cd[0][c], way[ORD - 1 - c] - way[ORD + c], sxy);
                syy = fmaf(a.cd[1][c], ayy[ORD - 1 - c] - ayy[ORD + c], syy);
            }
            a.asxx[i] = sxx;
            a.asyy[i] = syy;
            a.asxy[i] = sxy;
            // ---- stress update of this step, transposed ----
            float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
            if (in_n) {
                a.gL[i] = fmaf(sxx + syy, fl, gl);
                a.gM[i] = fmaf(sxx, fmx, fmaf(syy, fmy, gm));
                const float L2M = fmaf(2.f, M, L);
                float bx = fmaf(L2M, sxx, L * syy), by = fmaf(L, sxx, L2M * syy);
                if (ZM != 0) {
                    const float Sx = 0.5f * (L + M) * (sxx + syy), Sy = M * (sxx - syy);
                    float drx = 0.f, dry = 0.f;
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            const float qx = rxx[l] + Sx, qy = ryy[l] + Sy;
                            a.ar[0][l * G + i] = fmaf(a.zen.Ap[l], qx, Sx);
                            a.ar[1][l * G + i] = fmaf(a.zen.As[l], qy, Sy);
                            drx = fmaf(a.zen.Bp[l] * gp, qx, drx);
                            dry = fmaf(a.zen.Bs[l] * gs, qy, dry);
                        }
                    bx += fmaf(0.5f, dry, drx);
                    by += fmaf(-0.5f, dry, drx);
                }
                o0 = bx;
                o1 = by;
                if (sx >= 0) {
                    o0 = cpml_adj(bx, pn0, a.tab_h[0][x]);
                    a.apsi[0][ix] = pn0;
                }
                if (syl >= 0) {
                    o1 = cpml_adj(by, pn1, a.tab_f[1][y]);
                    a.apsi[2][iy] = pn1;
                }
            }
            if (in_s) {
                a.gMs[i] = fmaf(sxy, fsh, gms);
                float eb = Ms * sxy;
                if (ZM != 0) {
                    const float S = 0.5f * Ms * sxy;
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            const float q = rxy[l] + S;
                            a.ar[2][l * G + i] = fmaf(a.zen.As[l], q, S);
                            eb = fmaf(a.zen.Bs[l] * gs, q, eb);
                        }
                }
                o2 = eb;
                o3 = eb;
                if (sx >= 0) {
                    o2 = cpml_adj(eb, ps0, a.tab_f[0][x]);
                    a.apsi[1][ix] = ps0;
                }
                if (syl >= 0) {
                    o3 = cpml_adj(eb, ps1, a.tab_h[1][y]);
                    a.apsi[3][iy] = ps1;
                }
            }
            a.dv[0][i] = o0;
            a.dv[1][i] = o1;
            a.dv[2][i] = o2;
            a.dv[3][i] = o3;
            if (t + 1 < TX) {
                shift_window<ORD, !FAST>(wax, a.ds[0], x + ORD + 1, nx, P, y);
                shift_window<ORD, !FAST>(way, a.ds[2], x + ORD, nx, P, y);
            }
        }
    };
    if (fast) sweep(std::true_type{});
    else sweep(std::false_type{});
    pdl_trigger();
}

template <int ORD, int TX, int MINB>
void launch_adj_shape(const AdjState &a, int zm, const float *rec, int k, cudaStream_t st) {
    const dim3 block(kBX2, kBY2), grid((a.ny + kBX2 - 1) / kBX2, (a.nx + kBY2 * TX - 1) / (kBY2 * TX));
    launch_pdl(k_adj_velocity<ORD, TX, MINB>, grid, block, st, a, rec, k);
    const bool three = a.zen.n == 3;
    if (zm == 0) launch_pdl(k_adj_stress<ORD, 0, 0, TX, MINB>, grid, block, st, a, rec);
    else if (zm == 1 && three) launch_pdl(k_adj_stress<ORD, 1, 3, TX, MINB>, grid, block, st, a, rec);
    else if (zm == 1) launch_pdl(k_adj_stress<ORD, 1, kMaxSls, TX, MINB>, grid, block, st, a, rec);
    else if (three) launch_pdl(k_adj_stress<ORD, 2, 3, TX, MINB>, grid, block, st, a, rec);
    else launch_pdl(k_adj_stress<ORD, 2, kMaxSls, TX, MINB>, grid, block, st, a, rec);
}

// Block shape of the adjoint kernels: one node per thread, and a register
// budget that keeps 3 blocks resident per SM (measured on the 512 x 1024
// three-mechanism case against 4 blocks and two nodes per thread).
template <int ORD>
void launch_adj_ord(const AdjState &a, int zm, const float *rec, int k, cudaStream_t st) {
    launch_adj_shape<ORD, kAdjTx, 3>(a, zm, rec, k, st);
}

void launch_adjoint_step(const AdjState &a, int ord, int zm, const float *rec, int k, cudaStream_t st) {
    switch (ord) {
    case 2: launch_adj_ord<2>(a, zm, rec, k, st); break;
    case 3: launch_adj_ord<3>(a, zm, rec, k, st); break;
    case 4: launch_adj_ord<4>(a, zm, rec, k, st); break;
    case 5: launch_adj_ord<5>(a, zm, rec, k, st); break;
    case 6: launch_adj_ord<6>(a, zm, rec, k, st); break;
    default: break;  // rejected at creation
    }
}

// the source force enters vy scaled by dt / rho at the node, i.e. By
__global__ void k_source_scales(Source *src, int n, const float *By) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) src[q].scale = By[src[q].cell];
}

thread_local std::string g_adj_error;
int afail(int code, const std::string &m) {
    g_adj_error = m;
    return code;
}

}  // namespace
}  // namespace ts

using namespace ts;

struct ts_adj {
    int device = 0, rows = 0, nx = 0, ny = 0, P = 0, ord = 2, zm = 0, ckpt = 0, n_ckpt = 0, n_rec = 0;
    int src_cols = 0, src_rows = 0, n_src_el = 0, n_src = 0, n_blocks = 0;
    int64_t G = 0, state_floats = 0, adj_floats = 0, launches = 0;
    std::vector<void *> allocs;
    StepParams sp{};   // forward, run by the stepper's kernels
    AdjState as{};     // adjoint kernels
    float *state = nullptr;     // forward state, one block: v, s, r, psi
    float *astate = nullptr;    // adjoint state, one block
    float *coefs = nullptr;     // own copy of L, M, Ms, Bx, By, g_p, g_s
    float *record = nullptr;    // [n_record_steps][kFeat][G]
    int n_record_steps = 0;

    float *checkpoints = nullptr;  // [n_ckpt][state_floats]
    Source *src = nullptr;
    float *src_tab = nullptr;
    int *scalars = nullptr;     // first_bad, step_base
    int forward_done = 0;
    int rec_segs = 1;           // trailing segments the forward pass records (checkpointed runs)
    int tail_recorded = 0;      // the record holds those segments, written by the forward pass

    template <typename T>
    int alloc(T **ptr, size_t n) {
        void *d = nullptr;
        cudaError_t e = cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return afail(TS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(d);
        *ptr = static_cast<T *>(d);
        return TS_OK;
    }
    template <typename T>
    int upload(T **ptr, const std::vector<T> &h) {
        int rc = alloc(ptr, h.size());
        if (rc) return rc;
        if (!h.empty() && cudaMemcpy(*ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
            return afail(TS_E_CUDA, "cudaMemcpy");
        return TS_OK;
    }
    float *record_of(int k_in_segment) const { return record + (int64_t)k_in_segment * kFeat * G; }
    int recompute(int s, cudaStream_t st) {
        const int k0 = s * ckpt, k1 = std::min(rows, k0 + ckpt);
        const int rc = copy_state(checkpoints + (int64_t)s * state_floats, false, st);
        if (rc) return rc;
        for (int k = k0; k < k1; ++k) forward_step(k, record_of(k - k0), st);
        return TS_OK;
    }
    // first step of the trailing segments the forward pass records
    int tail0() const { return std::max(0, n_ckpt - rec_segs) * ckpt; }
    // sweep of segment s; its record starts at step `base` of the record buffer
    void sweep(int s, int base, cudaStream_t st) {
        const int k0 = s * ckpt, k1 = std::min(rows, k0 + ckpt);
        for (int k = k1 - 1; k >= k0; --k) adjoint_step(k, record_of(k - base), st);
    }
    void forward_step(int k, float *rec, cudaStream_t st) {
        sp.feat = rec;
        if (rec) launch_step_2d_feat(sp, ord, zm, k, st);
        else launch_step_2d_folded(sp, ord, zm, k, st);
        sp.feat = nullptr;
        launches += 2;
    }
    void adjoint_step(int k, const float *rec, cudaStream_t st) {
        launch_adjoint_step(as, ord, zm, rec, k, st);
        launches += 2;
    }
    int copy_state(float *ckpt_slot, bool to_ckpt, cudaStream_t st) {
        cudaError_t e = to_ckpt ? cudaMemcpyAsync(ckpt_slot, state, state_floats * 4, cudaMemcpyDeviceToDevice, st)
                                : cudaMemcpyAsync(state, ckpt_slot, state_floats * 4, cudaMemcpyDeviceToDevice, st);
        return e == cudaSuccess ? TS_OK : afail(TS_E_CUDA, std::string("state copy: ") + cudaGetErrorString(e));
    }
    // source values of every source column for every step, in the reference's
    // flat indexing source_term[k * n_src_el + idx] (shader_webgpu_viscoelastic.wgsl:1050-1060)
    std::vector<float> source_table(const float *term) const {
        const int ncol = sp.src_ncol;
        std::vector<float> tab((size_t)rows * ncol, 0.f);
        for (int k = 0; k < rows; ++k)
            for (int c = 0; c < ncol && c < n_src_el; ++c) {
                const int64_t flat = (int64_t)k * n_src_el + c;
                if (flat < (int64_t)src_rows * src_cols) tab[(size_t)k * ncol + c] = term[flat];
            }
        return tab;
    }
};

extern "C" {

const char *ts_adj_last_error(void) { return g_adj_error.c_str(); }

void ts_adj_destroy(ts_adj *a) {
    if (!a) return;
    cudaSetDevice(a->device);
    cudaDeviceSynchronize();  // work may be in flight on any stream
    for (void *d : a->allocs) cudaFree(d);
    delete a;
}

int ts_adj_create(const ts_desc *d, int32_t checkpoint_every, ts_adj **out) {
    if (!d || !out) return afail(TS_E_ARG, "null argument");
    *out = nullptr;
    if (d->abi_version != TS_ABI_VERSION) return afail(TS_E_ARG, "abi_version mismatch");
    if (d->family != TS_WGSL2D) return afail(TS_E_ARG, "the adjoint supports the TS_WGSL2D family");
    if (d->ord < 2 || d->ord > kMaxOrd) return afail(TS_E_ARG, "ord must be in [2, 6]");
    if (d->nz != 1 || d->nx < 2 * d->ord + 1 || d->ny < 2 * d->ord + 1) return afail(TS_E_ARG, "bad grid");
    if (d->n_steps < 1) return afail(TS_E_ARG, "n_steps must be >= 1");
    if (d->visco && (d->n_sls < 1 || d->n_sls > kMaxSls)) return afail(TS_E_ARG, "n_sls must be in [1, 8]");
    if (checkpoint_every < 0) return afail(TS_E_ARG, "checkpoint_every must be >= 0");
    if (!d->pos_sources || (d->n_rec > 0 && (!d->info_rec_pt || !d->offset_sensors || !d->delay_rec)))
        return afail(TS_E_ARG, "missing source or receiver tables");
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return afail(TS_E_CUDA, "cudaGetDevice");
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return afail(TS_E_CUDA, "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3)) return afail(TS_E_NODEV, "this library is built for sm_103a only");

    ts_adj *a = new ts_adj();
    auto bail = [&](int rc) {
        ts_adj_destroy(a);
        return rc;
    };
    a->device = device;
    a->rows = d->n_steps;
    a->nx = d->nx;
    a->ny = d->ny;
    a->ord = d->ord;
    a->P = round_up(d->ny, 32);
    a->G = (int64_t)a->nx * a->P;
    a->src_rows = d->src_rows;
    a->src_cols = d->src_cols;
    a->n_src_el = d->n_src_el;
    a->zm = !d->visco ? 0 : (d->g_p ? 2 : 1);
    a->n_rec = d->n_rec;
    const int64_t G = a->G;
    StepParams &sp = a->sp;
    AdjState &as = a->as;
    sp.family = TS_WGSL2D;
    // the forward kernels: the stepper's choice at order 2 (one or two), two above
    sp.tx = d->ord == 2 ? std::min(2, nodes_per_thread_2d((int64_t)d->nx * d->ny)) : 2;
    sp.nx = a->nx;
    sp.ny = a->ny;
    sp.nz = 1;
    sp.pitch = a->P;
    sp.plane = a->P;
    sp.grid_elems = G;
    as.nx = a->nx;
    as.ny = a->ny;
    as.P = a->P;
    as.G = G;
    const float steps[2] = {d->dx, d->dy};
    for (int ax = 0; ax < 2; ++ax)
        for (int c = 0; c < kMaxOrd; ++c) sp.cd[ax][c] = as.cd[ax][c] = c < d->ord ? d->coefs[c] / steps[ax] : 0.f;
    sp.zen = as.zen = zener_constants(d);
    int rc;
    Axis axes[2] = {make_axis(a->nx, d->ord, d->a_x, d->b_x, d->k_x, d->a_xh, d->b_xh, d->k_xh),
                    make_axis(a->ny, d->ord, d->a_y, d->b_y, d->k_y, d->a_yh, d->b_yh, d->k_yh)};
    for (int ax = 0; ax < 2; ++ax) {
        Cpml *f = nullptr, *h = nullptr;
        if ((rc = a->upload(&f, axes[ax].full)) || (rc = a->upload(&h, axes[ax].half))) return bail(rc);
        sp.tab_f[ax] = as.tab_f[ax] = f;
        sp.tab_h[ax] = as.tab_h[ax] = h;
        sp.strip[ax] = as.strip[ax] = axes[ax].strip;
    }
    // state blocks: 5 fields, 3 x L memory variables, 8 strip memories (each
    // rounded to 64 floats); the adjoint block adds the 8 stencil-output adjoints
    const int64_t xs = (int64_t)sp.strip[0].width * a->P, ys = (int64_t)a->nx * sp.strip[1].width;
    const int L = d->visco ? d->n_sls : 0;
    const int64_t psz[8] = {xs, xs, ys, ys, xs, xs, ys, ys};
    auto r64 = [](int64_t n) { return (n + 63) / 64 * 64; };
    int64_t n_state = 5 * G + 3 * (int64_t)L * G;
    for (int k = 0; k < 8; ++k) n_state += r64(psz[k]);
    a->state_floats = n_state;
    a->adj_floats = n_state + 8 * G;
    if ((rc = a->alloc(&a->state, (size_t)a->state_floats)) || (rc = a->alloc(&a->astate, (size_t)a->adj_floats)))
        return bail(rc);
    {
        float *q = a->state;
        sp.v[0] = q, q += G;
        sp.v[1] = q, q += G;
        sp.s[0] = q, q += G;
        sp.s[1] = q, q += G;
        sp.s[3] = q, q += G;
        for (int m = 0; m < 3; ++m) sp.r[m] = L ? q + (int64_t)m * L * G : nullptr;
        q += 3 * (int64_t)L * G;
        for (int k = 0; k < 8; ++k) sp.psi[k] = q, q += r64(psz[k]);
        q = a->astate;
        float **a5[5] = {&as.avx, &as.avy, &as.asxx, &as.asyy, &as.asxy};
        for (auto f : a5) *f = q, q += G;
        for (int m = 0; m < 3; ++m) as.ar[m] = L ? q + (int64_t)m * L * G : nullptr;
        q += 3 * (int64_t)L * G;
        for (int k = 0; k < 8; ++k) as.apsi[k] = q, q += r64(psz[k]);
        for (int k = 0; k < 4; ++k) as.dv[k] = q, q += G;
        for (int k = 0; k < 4; ++k) as.ds[k] = q, q += G;
    }
    if ((rc = a->alloc(&a->coefs, (size_t)7 * G))) return bail(rc);
    sp.lam_dt = as.L = a->coefs;
    sp.mu_dt = as.M = a->coefs + G;
    sp.mus_dt[0] = as.Ms = a->coefs + 2 * G;
    sp.dtr[0] = as.Bx = a->coefs + 3 * G;
    sp.dtr[1] = as.By = a->coefs + 4 * G;
    sp.g_p = as.gp = a->coefs + 5 * G;
    sp.g_s = as.gs = a->coefs + 6 * G;
    // sources: every node of the source map, column = its source index,
    // binned by the block that updates it (forward and adjoint block shapes);
    // scales (= By at the node) are set by each forward
    a->n_blocks = blocks_2d(sp);
    const int gx = (a->ny + kBX2 - 1) / kBX2;
    const int n_blocks_adj = gx * ((a->nx + kBY2 * kAdjTx - 1) / (kBY2 * kAdjTx));
    {
        std::vector<std::pair<int64_t, int>> nodes;   // (cell, column) in (x, y) order
        int ncol = 0;
        for (int x = 0; x < a->nx; ++x)
            for (int y = 0; y < a->ny; ++y) {
                const int idx = d->pos_sources[(int64_t)x * a->ny + y];
                if (idx < 0) continue;
                nodes.push_back({(int64_t)x * a->P + y, idx});
                ncol = std::max(ncol, idx + 1);
            }
        auto binned = [&](int tx, int n_blocks, Source **dsrc, int **dstart) {
            struct Cand {
                int blk;
                Source s;
            };
            std::vector<Cand> cands;
            for (const auto &nd : nodes) {
                const int x = (int)(nd.first / a->P), y = (int)(nd.first % a->P);
                cands.push_back({(x / (kBY2 * tx)) * gx + y / kBX2, Source{nd.first, nd.second, 0.f}});
            }
            std::stable_sort(cands.begin(), cands.end(), [](const Cand &p, const Cand &q) { return p.blk < q.blk; });
            std::vector<Source> list;
            std::vector<int> start(n_blocks + 1, 0);
            for (const Cand &c : cands) {
                list.push_back(c.s);
                start[c.blk + 1]++;
            }
            for (int b = 0; b < n_blocks; ++b) start[b + 1] += start[b];
            int r = a->upload(dsrc, list);
            return r ? r : a->upload(dstart, start);
        };
        int *dstart = nullptr, *astart = nullptr;
        Source *asrc = nullptr;
        if ((rc = binned(sp.tx, a->n_blocks, &a->src, &dstart)) || (rc = binned(kAdjTx, n_blocks_adj, &asrc, &astart)))
            return bail(rc);
        a->n_src = (int)nodes.size();
        sp.src = a->src;
        sp.src_block_start = dstart;
        as.src = asrc;
        as.src_block_start = astart;
        sp.src_rows = as.src_rows = a->rows;
        sp.src_ncol = as.src_ncol = std::max(1, ncol);
        if ((rc = a->alloc(&a->src_tab, (size_t)a->rows * sp.src_ncol))) return bail(rc);
        sp.src_tab = as.src_tab = a->src_tab;
        if (d->source_term) {
            if ((rc = ts_adj_set_sources(a, d->source_term))) return bail(rc);
        } else if (cudaMemset(a->src_tab, 0, (size_t)a->rows * sp.src_ncol * 4) != cudaSuccess) {
            return bail(afail(TS_E_CUDA, "memset"));
        }
    }
    // receivers: nodes of each receiver in info_rec_pt order (shader_webgpu_viscoelastic.wgsl:1118-1134)
    {
        if ((int64_t)d->n_rec > (int64_t)std::min(a->n_blocks, n_blocks_adj) * kBX2 * kBY2)
            return bail(afail(TS_E_ARG, "more receivers than threads of a step launch"));
        std::vector<int> start(1, 0), first(std::max(1, d->n_rec), 0);
        std::vector<int64_t> cells;
        const int rec_groups = receiver_groups(d, 3);
        for (int r = 0; r < d->n_rec; ++r) {
            for (int pt = receiver_first_point(d, r, rec_groups); pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * 3 + 2] == r;
                 ++pt) {
                const int x = d->info_rec_pt[pt * 3], y = d->info_rec_pt[pt * 3 + 1];
                if (x >= 0 && x < a->nx && y >= 0 && y < a->ny) cells.push_back((int64_t)x * a->P + y);
            }
            start.push_back((int)cells.size());
            first[r] = d->delay_rec[r];
        }
        int *ds = nullptr, *df = nullptr;
        int64_t *dc = nullptr;
        if ((rc = a->upload(&ds, start)) || (rc = a->upload(&df, first)) || (rc = a->upload(&dc, cells))) return bail(rc);
        sp.rec_start = as.rec_start = ds;
        sp.rec_first_step = as.rec_first = df;
        sp.rec_cell = as.rec_cell = dc;
        as.n_rec = d->n_rec;
    }
    // stability bookkeeping of the forward kernels (not reported here)
    float *bm = nullptr;
    if ((rc = a->alloc(&bm, (size_t)a->n_blocks)) || (rc = a->alloc(&a->scalars, 2))) return bail(rc);
    sp.v2_threshold = FLT_MAX;
    sp.block_max = bm;
    sp.first_bad = a->scalars;
    sp.step_base = a->scalars + 1;
    // record: every step, or one K-step segment with checkpoints every K
    a->ckpt = checkpoint_every >= a->rows ? 0 : checkpoint_every;
    a->n_record_steps = a->ckpt > 0 ? a->ckpt : a->rows;
    if ((rc = a->alloc(&a->record, (size_t)a->n_record_steps * kFeat * G)))
        return bail(afail(rc, g_adj_error + " (adjoint record; a checkpoint interval keeps less)"));
    if (a->ckpt > 0) {
        a->n_ckpt = (a->rows + a->ckpt - 1) / a->ckpt;
        if ((rc = a->alloc(&a->checkpoints, (size_t)a->n_ckpt * a->state_floats))) return bail(rc);
    }
    *out = a;
    return TS_OK;
}

int ts_adj_pitch(const ts_adj *a, int32_t *pitch) {
    if (!a || !pitch) return afail(TS_E_ARG, "null argument");
    *pitch = a->P;
    return TS_OK;
}

int ts_adj_set_sources(ts_adj *a, const float *source_term) {
    if (!a || !source_term) return afail(TS_E_ARG, "null argument");
    const std::vector<float> tab = a->source_table(source_term);
    cudaSetDevice(a->device);
    // ordered after every call already enqueued on any stream
    if (cudaDeviceSynchronize() != cudaSuccess) return afail(TS_E_CUDA, "synchronize");
    if (cudaMemcpy(a->src_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return afail(TS_E_CUDA, "cudaMemcpy");
    return TS_OK;
}

int ts_adj_read_field(ts_adj *a, int32_t what, void *host_dst, size_t bytes) {
    if (!a || !host_dst) return afail(TS_E_ARG, "null argument");
    const StepParams &p = a->sp;
    const float *src = what == TS_VX ? p.v[0] : what == TS_VY ? p.v[1] : what == TS_SXX ? p.s[0]
                     : what == TS_SYY ? p.s[1] : what == TS_SXY ? p.s[3] : nullptr;
    if (!src) return afail(TS_E_ARG, "no such field (2D: TS_VX, TS_VY, TS_SXX, TS_SYY, TS_SXY)");
    const size_t need = (size_t)a->nx * a->ny * sizeof(float);
    if (bytes < need) return afail(TS_E_ARG, "destination too small for the field");
    cudaSetDevice(a->device);
    if (cudaDeviceSynchronize() != cudaSuccess) return afail(TS_E_CUDA, "synchronize");
    if (cudaMemcpy2D(host_dst, a->ny * sizeof(float), src, a->P * sizeof(float), a->ny * sizeof(float), a->nx,
                     cudaMemcpyDeviceToHost) != cudaSuccess)
        return afail(TS_E_CUDA, "cudaMemcpy2D");
    return TS_OK;
}

int ts_adj_set_record_segments(ts_adj *a, int32_t segments) {
    if (!a) return afail(TS_E_ARG, "null handle");
    if (a->ckpt <= 0) return afail(TS_E_STATE, "every step is recorded already (checkpoint_every = 0)");
    if (segments < 1 || segments > a->n_ckpt) return afail(TS_E_ARG, "segments must be in [1, number of segments]");
    if (segments == a->rec_segs) return TS_OK;
    cudaSetDevice(a->device);
    cudaDeviceSynchronize();  // the record may be in use by enqueued work
    float *fresh = nullptr;
    const size_t n = (size_t)a->ckpt * segments * kFeat * a->G;
    if (cudaMalloc(&fresh, n * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return afail(TS_E_NOMEM, "record of the trailing segments");
    }
    for (auto &d : a->allocs)
        if (d == a->record) {
            cudaFree(d);
            d = fresh;
        }
    a->record = fresh;
    a->n_record_steps = a->ckpt * segments;
    a->rec_segs = segments;
    a->tail_recorded = 0;
    a->forward_done = 0;   // the next backward needs a forward that fills the new record
    return TS_OK;
}

int ts_adj_launch_count(const ts_adj *a, int64_t *launches) {
    if (!a || !launches) return afail(TS_E_ARG, "null argument");
    *launches = a->launches;
    return TS_OK;
}

int ts_adj_forward(ts_adj *a, const ts_adj_coefs *c, float *traces, void *stream) {
    if (!a || !c || !traces || !c->L || !c->M || !c->Ms || !c->Bx || !c->By) return afail(TS_E_ARG, "null argument");
    if (a->zm == 2 && (!c->g_p || !c->g_s)) return afail(TS_E_ARG, "per-cell Q scales g_p, g_s required");
    cudaSetDevice(a->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    const int64_t G = a->G;
    const float *src[7] = {c->L, c->M, c->Ms, c->Bx, c->By, c->g_p, c->g_s};
    for (int q = 0; q < (a->zm == 2 ? 7 : 5); ++q)
        if (cudaMemcpyAsync(a->coefs + q * G, src[q], G * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return afail(TS_E_CUDA, "coefficient copy");
    if (cudaMemsetAsync(a->state, 0, a->state_floats * 4, st) != cudaSuccess ||
        cudaMemsetAsync(traces, 0, (size_t)a->rows * std::max(1, a->n_rec) * 4, st) != cudaSuccess)
        return afail(TS_E_CUDA, "memset");
    if (a->n_src > 0) k_source_scales<<<(a->n_src + 127) / 128, 128, 0, st>>>(a->src, a->n_src, a->as.By);
    launch_reset_scalars(a->sp.first_bad, const_cast<int *>(a->sp.step_base), st);
    a->launches += 2;
    a->sp.n_rec = a->n_rec;
    a->sp.traces = traces;
    int rc;
    for (int k = 0; k < a->rows; ++k) {
        if (a->ckpt > 0 && k % a->ckpt == 0 &&
            (rc = a->copy_state(a->checkpoints + (int64_t)(k / a->ckpt) * a->state_floats, true, st)))
            return rc;
        // The trailing segments record as they go: their adjoint sweeps come
        // first and need no recomputation.
        const int t0 = a->tail0();
        float *rec = a->ckpt <= 0 ? a->record_of(k) : (k >= t0 ? a->record_of(k - t0) : nullptr);
        a->forward_step(k, rec, st);
    }
    a->tail_recorded = a->ckpt > 0;
    a->sp.n_rec = 0;
    a->sp.traces = nullptr;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(TS_E_CUDA, cudaGetErrorString(e));
    a->forward_done = 1;
    return TS_OK;
}

int ts_adj_backward(ts_adj *a, const float *residual, const ts_adj_grads *g, void *stream) {
    if (!a || !residual || !g || !g->gL || !g->gM || !g->gMs || !g->gBx || !g->gBy) return afail(TS_E_ARG, "null argument");
    if (!a->forward_done) return afail(TS_E_STATE, "ts_adj_forward must run first");
    cudaSetDevice(a->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    const int64_t G = a->G;
    AdjState &as = a->as;
    as.res = residual;
    as.gL = g->gL;
    as.gM = g->gM;
    as.gMs = g->gMs;
    as.gBx = g->gBx;
    as.gBy = g->gBy;
    if (cudaMemsetAsync(a->astate, 0, a->adj_floats * 4, st) != cudaSuccess) return afail(TS_E_CUDA, "memset");
    for (float *q : {g->gL, g->gM, g->gMs, g->gBx, g->gBy})
        if (cudaMemsetAsync(q, 0, (size_t)G * 4, st) != cudaSuccess) return afail(TS_E_CUDA, "memset");
    int rc;
    if (a->ckpt <= 0) {
        for (int k = a->rows - 1; k >= 0; --k) a->adjoint_step(k, a->record_of(k), st);
    } else {
        // (recomputing segment s-1 on a second stream while segment s is swept
        // was measured no faster: both passes share the same memory system)
        const int first_tail = a->n_ckpt - std::min(a->rec_segs, a->n_ckpt);
        for (int s = a->n_ckpt - 1; s >= 0; --s) {
            if (s >= first_tail && a->tail_recorded) {
                a->sweep(s, a->tail0(), st);
            } else {
                if ((rc = a->recompute(s, st))) return rc;
                a->tail_recorded = 0;   // the recomputed segment overwrote the start of the record
                a->sweep(s, s * a->ckpt, st);
            }
        }
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(TS_E_CUDA, cudaGetErrorString(e));
    return TS_OK;
}

}  // extern "C"
