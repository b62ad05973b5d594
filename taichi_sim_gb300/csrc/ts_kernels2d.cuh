// 2D staggered-grid (visco)elastic step kernels on sm_103a (internal header,
// included by the translation units that instantiate them).
//
// One time step = two launches on one stream:
//   k_stress2d   : sxx, syy (normal node) and sxy (shear node) from the
//                  velocities, with the CPML convolution in the boundary
//                  strips and the Zener memory-variable update fused in;
//   k_velocity2d : vx, vy from the stresses, with CPML, Dirichlet zeroing,
//                  source injection, receiver sampling of syy and the
//                  stability bookkeeping fused in.
//
// Thread (tx, ty) of block (bx, by) owns column y = 32 bx + tx and updates
// TX consecutive nodes x = TX (8 by + ty) + t: a warp reads 128 contiguous
// bytes per row (y is the contiguous axis).  Marching along x, the x-stencil
// values sit in a register window that takes one new row per node, and the
// index, region and bookkeeping work is paid once per TX nodes; these kernels
// are otherwise limited by the instructions they issue per node.  Within a
// node every load is issued before the first store, so one memory latency is
// paid per node.
//
// With FEAT the kernels also record, per node, the quantities the adjoint
// multiplies the coefficients by (slots of StepParams::feat, see
// ts_internal.cuh): at the normal node (dx~ + dy~ + Sxx/2),
// (2 dx~ + Sxx/2 + Syy) and (2 dy~ + Sxx/2 - Syy), at the shear node
// (e + Sxy/2), at the velocity nodes the CPML-corrected stress divergences.
//
// Semantics follow the reference (family TS_TAICHI2D:
// sim_taichi_elastic.py:138-309; family TS_WGSL2D:
// shader_webgpu_viscoelastic.wgsl:829-1072 and :1118-1134).  Family
// TS_WGSL2D replaces the divisions by dx/dy/rho/k with multiplications by
// precomputed reciprocals and contracts a*b+c to fma: it agrees with the
// reference's float arithmetic to rounding.  Family TS_TAICHI2D keeps the
// reference's operation order with every operation rounded on its own
// (taichi_* in ts_internal.cuh): bit for bit the strict-IEEE oracle.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>
#include "ts_internal.cuh"

namespace ts {
namespace {

// Arithmetic families of the 2D kernels: kTaichi keeps the Taichi kernels'
// operation order exactly (coefficient arrays hold lambda, mu, rho); kWgsl
// is the WGSL semantics with the grid-step and density divisions done once
// per derivative and per update, each rounded as a division (coefficient
// arrays hold lambda, mu, rho; sums contract to fma), so no step of the
// update carries a rounding bias that repeats at every node and time step;
// kWgslFolded is the WGSL semantics with dt, 1/dx and 1/rho folded into the
// coefficients (arrays hold lambda dt, mu dt, dt / rho), the form the
// adjoint differentiates (ts_adjoint.cu); kTaichiU is the Taichi kernels'
// semantics (update regions, the source inside the velocity update) in
// kWgsl's unbiased arithmetic.
constexpr int kTaichi = 0, kWgslFolded = 1, kWgsl = 2, kTaichiU = 3;
// the Taichi kernels' update regions and source injection
constexpr bool taichi_semantics(int fam) { return fam == kTaichi || fam == kTaichiU; }
// the unbiased arithmetic: raw coefficients, sums times 1/d as a pair, updates times dt, divisions by rho
constexpr bool unbiased(int fam) { return fam == kWgsl || fam == kTaichiU; }

// weight of derivative term c along axis a: coef / d (folded) or coef
template <int FAM>
__device__ __forceinline__ float dw(const StepParams &p, int a, int c) {
    return unbiased(FAM) ? p.coef[c] : p.cd[a][c];
}
// a derivative's sum of weighted differences, divided by the grid step (kWgsl)
template <int FAM>
__device__ __forceinline__ float dfin(float s, const StepParams &p, int a) {
    // kTaichiU: times the reference's own rounded 1/d, as the Taichi kernels
    // scale every term (their constant's rounding is part of what they compute)
    return FAM == kWgsl ? dscale(s, p.od[a], p.odl[a]) : FAM == kTaichiU ? s * p.od[a] : s;
}

// Loads.  ldg: data no kernel writes (coefficients, tables), through the
// read-only path.  ldf: fields the previous kernel of the stream wrote.  With
// programmatic dependent launch that kernel's lifetime overlaps this one's,
// so its output is not read-only for this kernel's lifetime and must not be
// read through the non-coherent path (doing so returned stale values):
// ld.global.ca, cached in L1 and coherent after griddepcontrol.wait.
__device__ __forceinline__ float ldg(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const float *p) { return __ldca(p); }

// b * psi + a * d, then d / k + psi
__device__ __forceinline__ float cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = fmaf(t.b, psi_old, t.a * d);
    return fmaf(d, t.ik, psi_new);
}

// CPML update in the family's arithmetic
template <int FAM>
__device__ __forceinline__ float cpmlf(float d, float psi_old, float &psi_new, const Cpml &t) {
    if (FAM == kTaichi) return taichi_cpml(d, psi_old, psi_new, t);
    if (unbiased(FAM)) {
        psi_new = fmaf(t.b, psi_old, t.a * d);
        return qdiv(d, t.k, t.ik) + psi_new;
    }
    return cpml(d, psi_old, psi_new, t);
}

// Window of 2*ORD rows of one field at column y, first row `r0`; rows
// outside the grid read 0 (they are only used by nodes outside the regions).
// CHECK = false: every row is known to lie inside the grid.
template <int ORD, bool CHECK = true>
__device__ __forceinline__ void load_window(float (&w)[2 * ORD], const float *f, int r0, int nx, int P, int y) {
#pragma unroll
    for (int j = 0; j < 2 * ORD; ++j) {
        const int r = r0 + j;
        w[j] = (!CHECK || (r >= 0 && r < nx)) ? ldf(f + (int64_t)r * P + y) : 0.f;
    }
}

template <int ORD, bool CHECK = true>
__device__ __forceinline__ void shift_window(float (&w)[2 * ORD], const float *f, int r_new, int nx, int P, int y) {
#pragma unroll
    for (int j = 0; j < 2 * ORD - 1; ++j) w[j] = w[j + 1];
    w[2 * ORD - 1] = (!CHECK || (r_new >= 0 && r_new < nx)) ? ldf(f + (int64_t)r_new * P + y) : 0.f;
}

// A warp whose TX-node chunk lies wholly in the interior (every node inside
// the update regions of both kernels, outside the CPML strips, window rows
// inside the grid) sweeps without per-node region, strip or bounds tests.
// Evaluated by all 32 lanes before any of them returns.
template <int ORD, int TX, typename Params>
__device__ __forceinline__ bool interior_warp(const Params &p, int y, int x0, int sy) {
    const bool lane = y < p.ny && sy < 0 && y >= ORD && y < p.ny - ORD && x0 >= ORD && x0 >= p.strip[0].lo &&
                      x0 + TX + ORD <= p.nx && x0 + TX <= p.strip[0].hi;
    return __all_sync(0xffffffffu, lane);
}

// PAL: the node's coefficients (lambda, mu, its Q scales; mu at the shear
// node) come from p.pal[p.pal_idx[node]] (one 16-bit index per node into the
// model's distinct coefficient tuples, loaded first; its table entry after
// every other load) instead of five arrays.
template <int ORD, int FAM, int ZM, int NS, int TX, bool FEAT = false, int MINB = 0, bool PAL = false>
__global__ void __launch_bounds__(kBX2 *kBY2, MINB) k_stress2d(const StepParams p) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x0 = (blockIdx.y * kBY2 + threadIdx.y) * TX;
    const int sy = y < p.ny ? strip_index(p.strip[1], y) : -1;
    const bool fast = interior_warp<ORD, TX>(p, y, x0, sy);
    if (y >= p.ny || x0 >= p.nx) return;
    const int P = p.pitch, nx = p.nx;
    const float *__restrict__ vx = p.v[0];   // read with ldf only
    const float *__restrict__ vy = p.v[1];
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    constexpr int R = NS > 0 ? NS : 1;
    const bool yn = y >= ORD && y < p.ny - ORD + 1;   // normal-stress rows in y
    const bool ys = y >= ORD - 1 && y < p.ny - ORD;   // shear-stress rows in y
    pdl_wait();
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // vx rows [x-ORD+1, x+ORD] (normal x-derivative), vy rows [x-ORD, x+ORD-1] (shear)
        float wvx[2 * ORD], wvy[2 * ORD];
        load_window<ORD, !FAST>(wvx, vx, x0 - ORD + 1, nx, P, y);
        load_window<ORD, !FAST>(wvy, vy, x0 - ORD, nx, P, y);

#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (!FAST && x >= nx) break;
            const int64_t i = (int64_t)x * P + y;
            const bool in_n = FAST || (yn && x >= ORD - 1 && x < nx - ORD);
            const bool in_s = FAST || (ys && x >= ORD && x < nx - ORD + 1);
            if (in_n || in_s) {
                const int sx = FAST ? -1 : strip_index(p.strip[0], x);
                const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + syl;
                // ---- loads ----
                float L = 0.f, M = 0.f, Ms = 0.f, gp = 1.f, gs = 1.f, sxx = 0.f, syy = 0.f, sxy = 0.f;
                float ny_lo[ORD], ny_hi[ORD - 1 > 0 ? ORD - 1 : 1], sx_lo[ORD - 1 > 0 ? ORD - 1 : 1], sx_hi[ORD];
                float rxx[R], ryy[R], rxy[R];
                float pn0 = 0.f, pn1 = 0.f, ps0 = 0.f, ps1 = 0.f;
                const uint16_t pidx = PAL ? __ldg(p.pal_idx + i) : 0;
                if (in_n) {
                    if (!PAL) {
                        L = ldg(p.lam_dt + i);
                        M = ldg(p.mu_dt + i);
                        if (ZM == 2) gp = ldg(p.g_p + i);
                    }
#pragma unroll
                    for (int c = 0; c < ORD; ++c) ny_lo[c] = ldf(vy + i - c - 1);   // vy[y-c-1]
#pragma unroll
                    for (int c = 1; c < ORD; ++c) ny_hi[c - 1] = ldf(vy + i + c);   // vy[y+c], c >= 1
                    sxx = p.s[0][i];
                    syy = p.s[1][i];
                    if (sx >= 0) pn0 = p.psi[0][ix];
                    if (syl >= 0) pn1 = p.psi[2][iy];
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) {
                                rxx[l] = p.r[0][l * p.grid_elems + i];
                                ryy[l] = p.r[1][l * p.grid_elems + i];
                            }
                    }
                }
                if (in_s) {
                    if (!PAL) Ms = ldg(p.mus_dt[0] + i);
#pragma unroll
                    for (int c = 0; c < ORD; ++c) sx_hi[c] = ldf(vx + i + c + 1);   // vx[y+c+1]
#pragma unroll
                    for (int c = 1; c < ORD; ++c) sx_lo[c - 1] = ldf(vx + i - c);   // vx[y-c], c >= 1
                    sxy = p.s[3][i];
                    if (sx >= 0) ps0 = p.psi[1][ix];
                    if (syl >= 0) ps1 = p.psi[3][iy];
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) rxy[l] = p.r[2][l * p.grid_elems + i];
                    }
                }
                if (ZM == 2 && !PAL) gs = ldg(p.g_s + i);
                if (PAL) {
                    const float4 cn = __ldg(&p.pal[pidx].normal), cs = __ldg(&p.pal[pidx].shear);
                    L = cn.x;
                    M = cn.y;
                    gp = cn.z;
                    gs = cn.w;
                    Ms = cs.x;
                }
                // ---- normal stresses ----
                if (in_n) {
                    float ddx = 0.f, ddy = 0.f, np_;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        const float hi = c == 0 ? wvy[ORD] : ny_hi[c > 0 ? c - 1 : 0];
                        if (FAM == kTaichi) {
                            ddx = taichi_term(ddx, p.coef[c], wvx[c + ORD], wvx[ORD - 1 - c], p.od[0]);
                            ddy = taichi_term(ddy, p.coef[c], hi, ny_lo[c], p.od[1]);
                        } else {
                            ddx = fmaf(dw<FAM>(p, 0, c), wvx[c + ORD] - wvx[ORD - 1 - c], ddx);
                            ddy = fmaf(dw<FAM>(p, 1, c), hi - ny_lo[c], ddy);
                        }
                    }
                    ddx = dfin<FAM>(ddx, p, 0);
                    ddy = dfin<FAM>(ddy, p, 1);
                    if (sx >= 0) {
                        ddx = cpmlf<FAM>(ddx, pn0, np_, p.tab_h[0][x]);
                        p.psi[0][ix] = np_;
                    }
                    if (syl >= 0) {
                        ddy = cpmlf<FAM>(ddy, pn1, np_, p.tab_f[1][y]);
                        p.psi[2][iy] = np_;
                    }
                    if (FAM == kTaichi) {
                        const float dl = __fmul_rn(L, __fadd_rn(ddx, ddy));
                        sxx = taichi_normal(sxx, dl, M, ddx, p.dt);
                        syy = taichi_normal(syy, dl, M, ddy, p.dt);
                    } else if (FAM == kTaichiU) {
                        // (lambda div + 2 mu d) dt with no per-node constant folded (lambda + 2 mu
                        // rounded once per node would bias every step alike)
                        const float dl = L * (ddx + ddy);
                        sxx += fmaf(2.f * M, ddx, dl) * p.dt;
                        syy += fmaf(2.f * M, ddy, dl) * p.dt;
                    } else {
                        const float L2M = fmaf(2.f, M, L);
                        float ux = fmaf(L2M, ddx, L * ddy), uy = fmaf(L, ddx, L2M * ddy);
                        float srxx = 0.f, sryy = 0.f;
                        if (ZM != 0) {
                            const float dsum = ddx + ddy, ddif = 0.5f * (ddx - ddy);
#pragma unroll
                            for (int l = 0; l < R; ++l)
                                if (l < n_mech) {
                                    const float a = fmaf(p.zen.Ap[l], rxx[l], (p.zen.Bp[l] * gp) * dsum);
                                    const float b = fmaf(p.zen.As[l], ryy[l], (p.zen.Bs[l] * gs) * ddif);
                                    srxx += rxx[l] + a;
                                    sryy += ryy[l] + b;
                                    p.r[0][l * p.grid_elems + i] = a;
                                    p.r[1][l * p.grid_elems + i] = b;
                                }
                            const float hl = 0.5f * (L + M);
                            ux = fmaf(hl, srxx, fmaf(M, sryy, ux));
                            uy = fmaf(hl, srxx, fmaf(-M, sryy, uy));
                        }
                        if (unbiased(FAM)) {   // (...) dt, wgsl:915-916
                            sxx += ux * p.dt;
                            syy += uy * p.dt;
                        } else {
                            sxx += ux;
                            syy += uy;
                        }
                        if (FEAT) {
                            const float h = 0.5f * srxx;
                            p.feat[kFeatLam * p.grid_elems + i] = ddx + ddy + h;
                            p.feat[kFeatMuX * p.grid_elems + i] = fmaf(2.f, ddx, h + sryy);
                            p.feat[kFeatMuY * p.grid_elems + i] = fmaf(2.f, ddy, h - sryy);
                        }
                    }
                    p.s[0][i] = sxx;
                    p.s[1][i] = syy;
                }
                // ---- shear stress ----
                if (in_s) {
                    float a = 0.f, b = 0.f, np_;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        const float lo = c == 0 ? wvx[ORD - 1] : sx_lo[c > 0 ? c - 1 : 0];
                        if (FAM == kTaichi) {
                            a = taichi_term(a, p.coef[c], wvy[c + ORD], wvy[ORD - 1 - c], p.od[0]);
                            b = taichi_term(b, p.coef[c], sx_hi[c], lo, p.od[1]);
                        } else {
                            a = fmaf(dw<FAM>(p, 0, c), wvy[c + ORD] - wvy[ORD - 1 - c], a);
                            b = fmaf(dw<FAM>(p, 1, c), sx_hi[c] - lo, b);
                        }
                    }
                    a = dfin<FAM>(a, p, 0);
                    b = dfin<FAM>(b, p, 1);
                    if (sx >= 0) {
                        a = cpmlf<FAM>(a, ps0, np_, p.tab_f[0][x]);
                        p.psi[1][ix] = np_;
                    }
                    if (syl >= 0) {
                        b = cpmlf<FAM>(b, ps1, np_, p.tab_h[1][y]);
                        p.psi[3][iy] = np_;
                    }
                    if (FAM == kTaichi) {
                        p.s[3][i] = taichi_shear(sxy, __fadd_rn(a, b), Ms, p.dt);
                    } else {
                        const float e = a + b;
                        float u = Ms * e, sr = 0.f;
                        if (ZM != 0) {
#pragma unroll
                            for (int l = 0; l < R; ++l)
                                if (l < n_mech) {
                                    const float n_ = fmaf(p.zen.As[l], rxy[l], (p.zen.Bs[l] * gs) * e);
                                    sr += rxy[l] + n_;
                                    p.r[2][l * p.grid_elems + i] = n_;
                                }
                            u = fmaf(0.5f * Ms, sr, u);
                        }
                        if (FEAT) p.feat[kFeatShear * p.grid_elems + i] = fmaf(0.5f, sr, e);
                        p.s[3][i] = unbiased(FAM) ? sxy + u * p.dt : sxy + u;
                    }
                }
            }
            if (t + 1 < TX) {
                shift_window<ORD, !FAST>(wvx, vx, x + ORD + 1, nx, P, y);
                shift_window<ORD, !FAST>(wvy, vy, x + ORD, nx, P, y);
            }
        }
    };
    if (fast) sweep(std::true_type{});
    else sweep(std::false_type{});
    pdl_trigger();
}

template <int ORD, int FAM, int TX, bool FEAT = false, int MINB = 0>
__global__ void __launch_bounds__(kBX2 *kBY2, MINB) k_velocity2d(const StepParams p, const int j) {
    const int y = blockIdx.x * kBX2 + threadIdx.x;
    const int x0 = (blockIdx.y * kBY2 + threadIdx.y) * TX;
    const int tid = threadIdx.y * kBX2 + threadIdx.x;
    const int blk = blockIdx.y * gridDim.x + blockIdx.x;
    const int P = p.pitch, nx = p.nx;
    const bool live_col = y < p.ny;
    const float *__restrict__ sxx = p.s[0];  // read with ldf only
    const float *__restrict__ syy = p.s[1];
    const float *__restrict__ sxy = p.s[3];
    const int sy = live_col ? strip_index(p.strip[1], y) : -1;
    // y-part of the regions
    const bool yvy = y >= ORD - 1 && y < p.ny - ORD;
    const bool yvx = taichi_semantics(FAM) ? (y >= ORD && y < p.ny - ORD + 1) : (yvy && y >= ORD);
    const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
    const bool fast = interior_warp<ORD, TX>(p, y, x0, sy) && q0 == q1;   // no source node in the block
    pdl_wait();
    const int k = *p.step_base + j;
    unsigned vmax = 0u;  // max |v|^2 as float bits (v2 >= 0 or NaN: NaN ranks highest)
    bool bad = false;

    // The interior sweep issues every load of the thread's TX nodes before
    // the first update (one memory latency per thread, not per node): sxx
    // rows x0-ORD .. x0+TX+ORD-2, sxy rows x0-ORD+1 .. x0+TX+ORD-1, and per
    // node the y-neighbours of sxy and syy, vx, vy and dt/rho.
    auto interior = [&]() {
        constexpr int NR = TX + 2 * ORD - 1;
        float rxx[NR], rxy[NR];
        float bl[TX][ORD], bh[TX][ORD - 1 > 0 ? ORD - 1 : 1], by[TX][2 * ORD];
        float vx0[TX], vy0[TX], dx0[TX], dy0[TX];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            rxx[r] = ldf(sxx + (int64_t)(x0 - ORD + r) * P + y);
            rxy[r] = ldf(sxy + (int64_t)(x0 - ORD + 1 + r) * P + y);
        }
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int64_t i = (int64_t)(x0 + t) * P + y;
#pragma unroll
            for (int c = 0; c < ORD; ++c) bl[t][c] = ldf(sxy + i - c - 1);   // sxy[y-c-1]
#pragma unroll
            for (int c = 1; c < ORD; ++c) bh[t][c - 1] = ldf(sxy + i + c);   // sxy[y+c], c >= 1
#pragma unroll
            for (int c = 0; c < 2 * ORD; ++c) by[t][c] = ldf(syy + i - ORD + 1 + c);   // syy[y-ORD+1 .. y+ORD]
            vx0[t] = p.v[0][i];
            vy0[t] = p.v[1][i];
            dx0[t] = ldg(p.dtr[0] + i);
            dy0[t] = ldg(p.dtr[1] + i);
        }
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int64_t i = (int64_t)(x0 + t) * P + y;
            // rows x+c / x-c-1 of sxx and x+c+1 / x-c of sxy sit at t+ORD+c / t+ORD-1-c; sxy row x at t+ORD-1
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                const float hi = c == 0 ? rxy[t + ORD - 1] : bh[t][c > 0 ? c - 1 : 0];
                if (FAM == kTaichi) {
                    a = taichi_term(a, p.coef[c], rxx[t + ORD + c], rxx[t + ORD - 1 - c], p.od[0]);
                    b = taichi_term(b, p.coef[c], hi, bl[t][c], p.od[1]);
                } else {
                    a = fmaf(dw<FAM>(p, 0, c), rxx[t + ORD + c] - rxx[t + ORD - 1 - c], a);
                    b = fmaf(dw<FAM>(p, 1, c), hi - bl[t][c], b);
                }
            }
            a = dfin<FAM>(a, p, 0);
            b = dfin<FAM>(b, p, 1);
            const float fax = FAM == kTaichi ? __fadd_rn(a, b) : a + b;
            const float vxn = FAM == kTaichi ? taichi_velocity(vx0[t], fax, 0.f, dx0[t], p.dt) : unbiased(FAM) ? wgsl_velocity_rho(vx0[t], fax, dx0[t], p.dt)
                                                   : fmaf(fax, dx0[t], vx0[t]);
            a = 0.f;
            b = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                if (FAM == kTaichi) {
                    a = taichi_term(a, p.coef[c], rxy[t + ORD + c], rxy[t + ORD - 1 - c], p.od[0]);
                    b = taichi_term(b, p.coef[c], by[t][ORD + c], by[t][ORD - 1 - c], p.od[1]);
                } else {
                    a = fmaf(dw<FAM>(p, 0, c), rxy[t + ORD + c] - rxy[t + ORD - 1 - c], a);
                    b = fmaf(dw<FAM>(p, 1, c), by[t][ORD + c] - by[t][ORD - 1 - c], b);
                }
            }
            a = dfin<FAM>(a, p, 0);
            b = dfin<FAM>(b, p, 1);
            const float fay = FAM == kTaichi ? __fadd_rn(a, b) : a + b;
            const float vyn = FAM == kTaichi ? taichi_velocity(vy0[t], fay, 0.f, dy0[t], p.dt) : unbiased(FAM) ? wgsl_velocity_rho(vy0[t], fay, dy0[t], p.dt)
                                                   : fmaf(fay, dy0[t], vy0[t]);
            p.v[0][i] = vxn;
            p.v[1][i] = vyn;
            if (FEAT) {
                p.feat[kFeatVx * p.grid_elems + i] = fax;
                p.feat[kFeatVy * p.grid_elems + i] = fay;
            }
            const float v2 = fmaf(vxn, vxn, vyn * vyn);
            bad |= !(v2 <= p.v2_threshold);
            vmax = max(vmax, __float_as_uint(v2));
        }
    };

    // The general sweep (every region, strip, bounds and source test); the
    // interior sweep above replaces its FAST instantiation.
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // sxx rows [x-ORD, x+ORD-1] (vx), sxy rows [x-ORD+1, x+ORD] (vy; row x also feeds vx's y-derivative)
        float wxx[2 * ORD], wxy[2 * ORD];
        load_window<ORD, !FAST>(wxx, sxx, x0 - ORD, nx, P, y);
        load_window<ORD, !FAST>(wxy, sxy, x0 - ORD + 1, nx, P, y);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (!FAST && x >= nx) break;
            const int64_t i = (int64_t)x * P + y;
            const bool in_vy = FAST || (yvy && x >= ORD - 1 && x < nx - ORD);
            const bool in_vx = FAST || (taichi_semantics(FAM) ? (yvx && x >= ORD && x < nx - ORD + 1) : (yvx && in_vy && x >= ORD));
            const int sx = FAST ? -1 : strip_index(p.strip[0], x);
            const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + syl;
            // ---- loads ----
            float bx_lo[ORD], bx_hi[ORD - 1 > 0 ? ORD - 1 : 1], by[2 * ORD];
            float vx0 = 0.f, vy0 = 0.f, dx0 = 0.f, dy0 = 0.f, pxa = 0.f, pxb = 0.f, pya = 0.f, pyb = 0.f;
            if (in_vx) {
#pragma unroll
                for (int c = 0; c < ORD; ++c) bx_lo[c] = ldf(sxy + i - c - 1);   // sxy[y-c-1]
#pragma unroll
                for (int c = 1; c < ORD; ++c) bx_hi[c - 1] = ldf(sxy + i + c);   // sxy[y+c], c >= 1
                vx0 = p.v[0][i];
                dx0 = ldg(p.dtr[0] + i);
                if (sx >= 0) pxa = p.psi[4][ix];
                if (syl >= 0) pxb = p.psi[6][iy];
            }
            if (in_vy) {
#pragma unroll
                for (int c = 0; c < 2 * ORD; ++c) by[c] = ldf(syy + i - ORD + 1 + c);   // syy[y-ORD+1 .. y+ORD]
                vy0 = p.v[1][i];
                dy0 = ldg(p.dtr[1] + i);
                if (sx >= 0) pya = p.psi[5][ix];
                if (syl >= 0) pyb = p.psi[7][iy];
            }
            // ---- update ----
            float vxn = 0.f, vyn = 0.f, np_, fax = 0.f, fay = 0.f;
            if (in_vx) {
                float a = 0.f, b = 0.f;
#pragma unroll
                for (int c = 0; c < ORD; ++c) {
                    const float hi = c == 0 ? wxy[ORD - 1] : bx_hi[c > 0 ? c - 1 : 0];
                    if (FAM == kTaichi) {
                        a = taichi_term(a, p.coef[c], wxx[c + ORD], wxx[ORD - 1 - c], p.od[0]);
                        b = taichi_term(b, p.coef[c], hi, bx_lo[c], p.od[1]);
                    } else {
                        a = fmaf(dw<FAM>(p, 0, c), wxx[c + ORD] - wxx[ORD - 1 - c], a);
                        b = fmaf(dw<FAM>(p, 1, c), hi - bx_lo[c], b);
                    }
                }
                a = dfin<FAM>(a, p, 0);
                b = dfin<FAM>(b, p, 1);
                if (sx >= 0) {
                    a = cpmlf<FAM>(a, pxa, np_, p.tab_f[0][x]);
                    p.psi[4][ix] = np_;
                }
                if (syl >= 0) {
                    b = cpmlf<FAM>(b, pxb, np_, p.tab_f[1][y]);
                    p.psi[6][iy] = np_;
                }
                fax = FAM == kTaichi ? __fadd_rn(a, b) : a + b;
                vxn = FAM == kTaichi ? taichi_velocity(vx0, fax, 0.f, dx0, p.dt)
                      : unbiased(FAM)  ? wgsl_velocity_rho(vx0, fax, dx0, p.dt)
                                       : fmaf(fax, dx0, vx0);
            }
            if (in_vy) {
                float a = 0.f, b = 0.f;
#pragma unroll
                for (int c = 0; c < ORD; ++c) {
                    if (FAM == kTaichi) {
                        a = taichi_term(a, p.coef[c], wxy[c + ORD], wxy[ORD - 1 - c], p.od[0]);
                        b = taichi_term(b, p.coef[c], by[ORD + c], by[ORD - 1 - c], p.od[1]);
                    } else {
                        a = fmaf(dw<FAM>(p, 0, c), wxy[c + ORD] - wxy[ORD - 1 - c], a);
                        b = fmaf(dw<FAM>(p, 1, c), by[ORD + c] - by[ORD - 1 - c], b);
                    }
                }
                a = dfin<FAM>(a, p, 0);
                b = dfin<FAM>(b, p, 1);
                if (sx >= 0) {
                    a = cpmlf<FAM>(a, pya, np_, p.tab_h[0][x]);
                    p.psi[5][ix] = np_;
                }
                if (syl >= 0) {
                    b = cpmlf<FAM>(b, pyb, np_, p.tab_h[1][y]);
                    p.psi[7][iy] = np_;
                }
                fay = FAM == kTaichi ? __fadd_rn(a, b) : a + b;
                if (FAM == kTaichi) {
                    // the source's force dt / rho joins the update inside it (sim_taichi_elastic.py:294-304)
                    float src = 0.f;
                    if constexpr (!FAST) {
                        for (int q = q0; q < q1; ++q) {
                            const Source s = p.src[q];
                            if (s.cell == i && k < p.src_rows)
                                src = __fdiv_rn(__fmul_rn(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), p.dt), s.scale);
                        }
                    }
                    vyn = taichi_velocity(vy0, fay, src, dy0, p.dt);
                } else if (FAM == kTaichiU) {
                    // the source inside the update, as the Taichi kernel adds it, in the unbiased arithmetic
                    float src = 0.f;
                    if constexpr (!FAST) {
                        for (int q = q0; q < q1; ++q) {
                            const Source s = p.src[q];
                            if (s.cell == i && k < p.src_rows)
                                src = wgsl_source(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, p.dt);
                        }
                    }
                    vyn = dy0 > 0.f ? vy0 + (src + qdiv(fay * p.dt, dy0, __frcp_rn(dy0))) : vy0;
                } else {
                    vyn = FAM == kWgsl ? wgsl_velocity_rho(vy0, fay, dy0, p.dt) : fmaf(fay, dy0, vy0);
                }
            }
            if constexpr (!FAST && !taichi_semantics(FAM)) {
                for (int q = q0; q < q1; ++q) {
                    const Source s = p.src[q];
                    if (s.cell == i && k < p.src_rows)
                        vyn = FAM == kWgsl ? vyn + wgsl_source(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, p.dt)
                                           : fmaf(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, vyn);
                }
            }
            p.v[0][i] = vxn;
            p.v[1][i] = vyn;
            if (FEAT) {
                p.feat[kFeatVx * p.grid_elems + i] = fax;
                p.feat[kFeatVy * p.grid_elems + i] = fay;
            }
            const float v2 = fmaf(vxn, vxn, vyn * vyn);
            bad |= !(v2 <= p.v2_threshold);
            vmax = max(vmax, __float_as_uint(v2));
            if (t + 1 < TX) {
                shift_window<ORD, !FAST>(wxx, sxx, x + ORD, nx, P, y);
                shift_window<ORD, !FAST>(wxy, sxy, x + ORD + 1, nx, P, y);
            }
        }
    };
    if (fast) interior();
    else if (live_col && x0 < nx) sweep(std::false_type{});

    // receivers: global thread g samples receiver g (syy is final for step k)
    const int g = blk * (kBX2 * kBY2) + tid;
    if (g < p.n_rec && k >= __ldg(p.rec_first_step + g) && !(p.rec_chunked && p.rec_chunked[g])) {
        float acc = 0.f;
        for (int q = __ldg(p.rec_start + g); q < __ldg(p.rec_start + g + 1); ++q) acc += ldf(syy + __ldg(p.rec_cell + q));
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }
    warp_stability(__uint_as_float(vmax), bad, reinterpret_cast<unsigned *>(p.block_max) + blk, p.first_bad, k);
    pdl_trigger();
}

}  // namespace
}  // namespace ts
