// Batched 2D (visco)elastic stepping: many shots of several phantoms (grids
// of uneven sizes) advanced together, one launch per kernel per time step.
//
// Layout: per phantom every field is [S/W][nx][ny][W]: blocks of W = 32 or
// 64 shots (S = shots rounded up to W), the shot index innermost.  A warp
// covers the W shots of one grid node (one or two per lane), so every load
// and store is one contiguous 128- or 256-byte row, neighbouring nodes along
// y are W floats apart (immediate offsets), the per-node coefficients
// (lambda, mu, dt/rho, Q scale) are one broadcast load shared by all shots,
// and the region and CPML-strip tests are uniform across the warp.
// Blocks are 32 lanes x CY nodes along y; each thread updates TX consecutive
// nodes along x, keeping the x-stencil rows in a register window (one new
// row per node), for SPT shots.  The flat block index runs over (phantom,
// x-chunk, y-block, shot-block), so phantoms of any size share one launch;
// the stress and velocity launches may use different CY and TX (their own
// block decompositions, Decomp), the shot layout (SPT) being shared.
// Threads whose nodes all lie in the interior (no region, strip, bounds or
// source test can fire) take a sweep with those tests compiled out; the
// velocity kernel's interior sweep issues every load of its nodes first.
// The phantom records are a __grid_constant__ parameter (constant cache, no
// aliasing with the fields) and offsets are 32-bit (checked at creation).
//
// Semantics: the WGSL 2D kernels (shader_webgpu_viscoelastic.wgsl:829-1072
// and :1118-1134) per shot, except for the source columns: shot s injects
// column idx of its own source table (the column the reference's source map
// names), so one-element shots of a full-matrix capture fire the element
// they name.  The arithmetic is the single-shot stepper's (ts_kernels2d.cuh,
// kWgsl): derivative sums times 1 / d as a (hi, lo) pair, updates times dt,
// velocity updates times dt / rho as a pair, so that no rounded constant
// biases every node and step alike.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/taichi_sim_gb300.h"
#include "ts_internal.cuh"
#include "ts_prep.h"

namespace ts {
namespace {

constexpr int kMaxPhantoms = 8;

struct BSrc {
    int cell;     // x * ny + y
    int col;      // source column
    float scale;  // rho at the vy node (the source force is divided by it)
};

// Flat block range of one phantom in one kernel's launch: blocks of 32 lanes
// x CY nodes along y, TX nodes along x per thread.
struct Decomp {
    int block0, xchunks, yblocks;
};

struct BPh {
    int nx, ny, S, W, n_shots;   // S shots padded to a multiple of W (shots per block row: 32 or 64)
    int G;      // nx * ny * S (checked < 2^31 with the memory variables)
    int sblocks;
    Decomp dc[2];  // block decomposition of the stress (0) and velocity (1) launches
    float od[2], odl[2];   // 1 / dx, 1 / dy as (hi, lo): a derivative is its sum times them
    float *v[2], *s[3], *r[3], *psi[8];
    const Cpml *tab_f[2], *tab_h[2];
    Strip strip[2];
    const float *lam, *mu, *mus, *gp, *gs;   // lambda, mu, mu at the shear node (not folded with dt)
    const float2 *dtw0, *dtw1;                // dt / rho at the vx, vy nodes as (hi, lo) pairs
    const BSrc *src;
    const int *src_start;  // [xchunks * yblocks + 1] of the velocity launch
    const float *shot_tab;  // [n_shots][rows][ncol]
    int ncol;
    int n_rec;
    const int *rec_start, *rec_cell, *rec_first;
    float *traces;  // [n_shots][rows][n_rec]
    int rec_work0;
};

// Passed as a __grid_constant__ kernel parameter: the phantom records are read
// through the constant cache and cannot alias the fields the kernels write.
struct BParams {
    int n_ph;
    BPh ph[kMaxPhantoms];
    int block_end[2][kMaxPhantoms];  // exclusive flat block end per kernel and phantom
    Zener zen;
    float coef[kMaxOrd];   // staggered FD coefficients
    float dt;
    int rows;
    float v2_threshold;
    float *block_max;
    int *first_bad;
    const int *step_base;
    int rec_work;
    int prefetch;   // L2 prefetch, before the wait, of each thread's own state (last written two launches back)
};

// b psi + a d, then d / k + psi (the shader's division, rounded as one)
__device__ __forceinline__ float cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = fmaf(t.b, psi_old, t.a * d);
    return qdiv(d, t.k, t.ik) + psi_new;
}

struct Loc {
    const BPh *ph;
    int x0, y, sb, lane, s0, cell0;
    int i0;
    bool live;
};

// Block b of a launch of kernel KIND (0 stress, 1 velocity): phantom, then
// (x-chunk, y-block, shot-block) within it.
// W = 32 * SPT shots per shot block: lane l owns shots SPT l .. SPT l + SPT-1.
template <int KIND, int CY, int TX, int SPT>
__device__ __forceinline__ Loc locate(const BParams &p) {
    constexpr int W = 32 * SPT;
    const int b = blockIdx.x;
    int q = 0;
#pragma unroll 1
    while (q + 1 < p.n_ph && b >= p.block_end[KIND][q]) ++q;
    Loc L;
    L.ph = p.ph + q;
    const BPh &h = *L.ph;
    const Decomp &dc = h.dc[KIND];
    const int local = b - dc.block0;
    L.sb = local % h.sblocks;
    const int t = local / h.sblocks;
    const int yb = t % dc.yblocks;
    L.x0 = (t / dc.yblocks) * TX;
    L.y = yb * CY + threadIdx.y;
    L.lane = threadIdx.x;
    L.s0 = L.sb * W + L.lane * SPT;
    L.live = L.y < h.ny && L.x0 < h.nx;
    L.cell0 = L.x0 * h.ny + L.y;
    L.i0 = ((L.sb * h.nx + L.x0) * h.ny + L.y) * W + L.lane * SPT;
    return L;
}

// SPT consecutive shots of one node.  ldf: a field the previous kernel of the
// stream wrote, read with ld.global.ca, never through the non-coherent path
// (with programmatic dependent launch that kernel overlaps this one's
// lifetime); ldo / sto: the node's own state.
template <int SPT>
__device__ __forceinline__ void ldf(float (&o)[SPT], const float *q) {
    if constexpr (SPT == 2) {
        const float2 v = __ldca(reinterpret_cast<const float2 *>(q));
        o[0] = v.x;
        o[1] = v.y;
    } else {
        o[0] = __ldca(q);
    }
}
template <int SPT>
__device__ __forceinline__ void ldo(float (&o)[SPT], const float *q) {
    if constexpr (SPT == 2) {
        const float2 v = *reinterpret_cast<const float2 *>(q);
        o[0] = v.x;
        o[1] = v.y;
    } else {
        o[0] = *q;
    }
}
template <int SPT>
__device__ __forceinline__ void sto(float *q, const float (&v)[SPT]) {
    if constexpr (SPT == 2) *reinterpret_cast<float2 *>(q) = make_float2(v[0], v[1]);
    else *q = v[0];
}

// Rows r0 .. r0+2*ORD-1 of one field at (y, shots), zero outside the grid.
template <int ORD, int SPT, bool CHECK = true>
__device__ __forceinline__ void bwindow(float (&w)[2 * ORD][SPT], const float *f, int r0, int nx, int X, int col) {
#pragma unroll
    for (int j = 0; j < 2 * ORD; ++j) {
        const int r = r0 + j;
        if (!CHECK || (r >= 0 && r < nx)) ldf<SPT>(w[j], f + r * X + col);
        else
#pragma unroll
            for (int q = 0; q < SPT; ++q) w[j][q] = 0.f;
    }
}

template <int ORD, int SPT, bool CHECK = true>
__device__ __forceinline__ void bshift(float (&w)[2 * ORD][SPT], const float *f, int r_new, int nx, int X, int col) {
#pragma unroll
    for (int j = 0; j < 2 * ORD - 1; ++j)
#pragma unroll
        for (int q = 0; q < SPT; ++q) w[j][q] = w[j + 1][q];
    if (!CHECK || (r_new >= 0 && r_new < nx)) ldf<SPT>(w[2 * ORD - 1], f + r_new * X + col);
    else
#pragma unroll
        for (int q = 0; q < SPT; ++q) w[2 * ORD - 1][q] = 0.f;
}

// Register budget of the stress kernel: 64 per thread for one shot per
// thread, 128 for two.  The velocity kernel takes 128 in both cases: its
// interior sweep holds every load of the thread's nodes at once.
template <int CY, int SPT>
struct MinBlocks {
    static constexpr int v = (SPT == 1 ? 32 : 16) / CY;
};
template <int CY>
struct MinBlocksV {
    static constexpr int v = 16 / CY;
};

template <int ORD, int ZM, int NS, int CY, int TX, int SPT>
__global__ void __launch_bounds__(32 * CY, (MinBlocks<CY, SPT>::v)) k_bstress(const __grid_constant__ BParams p) {
    constexpr int W = 32 * SPT, Y = W;
    const Loc at = locate<0, CY, TX, SPT>(p);
    if (!at.live) return;
    const BPh &h = *at.ph;
    // per-phantom values used at every node, copied to registers once
    const int y = at.y, nx = h.nx, ny = h.ny, G = h.G;
    const int X = ny * W, col = (at.sb * nx * ny + y) * W + at.lane * SPT;
    const bool yn = y >= ORD && y < ny - ORD + 1;
    const bool ys = y >= ORD - 1 && y < ny - ORD;
    const int sy = strip_index(h.strip[1], y);
    const Strip stx = h.strip[0];
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    constexpr int R = NS > 0 ? NS : 1;
    float cdx[ORD], cdy[ORD];
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        cdx[c] = p.coef[c];   // the sums are scaled by 1 / d after (dscale)
        cdy[c] = p.coef[c];
    }
    const float *__restrict__ vx = h.v[0];   // read with ldf only
    const float *__restrict__ vy = h.v[1];
    float *__restrict__ s0 = h.s[0];
    float *__restrict__ s1 = h.s[1];
    float *__restrict__ s2 = h.s[2];
    float *__restrict__ r0 = h.r[0];
    float *__restrict__ r1 = h.r[1];
    float *__restrict__ r2 = h.r[2];
    if (p.prefetch) {   // stresses and memory variables, written by this kernel's previous launch
#pragma unroll
        for (int t = 0; t < TX; ++t)
            if (at.x0 + t < nx) {
                const int i = at.i0 + t * X;
                prefetch_l2(s0 + i);
                prefetch_l2(s1 + i);
                prefetch_l2(s2 + i);
                if (ZM != 0)
                    for (int l = 0; l < n_mech; ++l) {
                        prefetch_l2(r0 + l * G + i);
                        prefetch_l2(r1 + l * G + i);
                        prefetch_l2(r2 + l * G + i);
                    }
            }
    }
    pdl_wait();
    // Interior chunks (every node of the thread inside both update regions and
    // outside the CPML strips, window rows inside the grid) take a sweep with
    // no per-node region, strip or bounds tests.
    const bool fast = sy < 0 && y >= ORD && y < ny - ORD && at.x0 >= ORD && at.x0 >= stx.lo &&
                      at.x0 + TX + ORD <= nx && at.x0 + TX <= stx.hi;
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // vx rows [x-ORD+1, x+ORD] (normal x-derivative), vy rows [x-ORD, x+ORD-1] (shear)
        float wvx[2 * ORD][SPT], wvy[2 * ORD][SPT];
        bwindow<ORD, SPT, !FAST>(wvx, vx, at.x0 - ORD + 1, nx, X, col);
        bwindow<ORD, SPT, !FAST>(wvy, vy, at.x0 - ORD, nx, X, col);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = at.x0 + t;
            if (!FAST && x >= nx) break;
            const int cell = at.cell0 + t * h.ny;
            const int i = at.i0 + t * X;
            const bool in_n = FAST || (yn && x >= ORD - 1 && x < nx - ORD);
            const bool in_s = FAST || (ys && x >= ORD && x < nx - ORD + 1);
            if (in_n || in_s) {
                const int sx = FAST ? -1 : strip_index(stx, x);
                const int ix = ((at.sb * stx.width + sx) * ny + y) * W + at.lane * SPT;
                const int iy = ((at.sb * nx + x) * h.strip[1].width + syl) * W + at.lane * SPT;
                // ---- loads ----
                float L = 0.f, M = 0.f, Ms = 0.f, gp = 1.f, gs = 1.f;
                float sxx[SPT], syy[SPT], sxy[SPT], pn0[SPT], pn1[SPT], ps0[SPT], ps1[SPT];
                float ny_lo[ORD][SPT], ny_hi[ORD][SPT], sx_lo[ORD][SPT], sx_hi[ORD][SPT];
                float rxx[R][SPT], ryy[R][SPT], rxy[R][SPT];
                if (in_n) {
                    L = __ldg(h.lam + cell);
                    M = __ldg(h.mu + cell);
                    if (ZM == 2) gp = __ldg(h.gp + cell);
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        ldf<SPT>(ny_hi[c], vy + i + c * Y);         // vy[y+c]
                        ldf<SPT>(ny_lo[c], vy + i - (c + 1) * Y);   // vy[y-c-1]
                    }
                    ldo<SPT>(sxx, s0 + i);
                    ldo<SPT>(syy, s1 + i);
                    if (sx >= 0) ldo<SPT>(pn0, h.psi[0] + ix);
                    if (syl >= 0) ldo<SPT>(pn1, h.psi[2] + iy);
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) {
                                ldo<SPT>(rxx[l], r0 + l * G + i);
                                ldo<SPT>(ryy[l], r1 + l * G + i);
                            }
                    }
                }
                if (in_s) {
                    Ms = __ldg(h.mus + cell);
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        ldf<SPT>(sx_hi[c], vx + i + (c + 1) * Y);   // vx[y+c+1]
                        ldf<SPT>(sx_lo[c], vx + i - c * Y);         // vx[y-c]
                    }
                    ldo<SPT>(sxy, s2 + i);
                    if (sx >= 0) ldo<SPT>(ps0, h.psi[1] + ix);
                    if (syl >= 0) ldo<SPT>(ps1, h.psi[3] + iy);
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) ldo<SPT>(rxy[l], r2 + l * G + i);
                    }
                }
                if (ZM == 2) gs = __ldg(h.gs + cell);
                // ---- normal stresses ----
                if (in_n) {
                    float ux[SPT], uy[SPT], pn0n[SPT], pn1n[SPT];
                    float ra[R][SPT], rb[R][SPT];
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        float ddx = 0.f, ddy = 0.f;
#pragma unroll
                        for (int c = 0; c < ORD; ++c) {
                            ddx = fmaf(cdx[c], wvx[c + ORD][q] - wvx[ORD - 1 - c][q], ddx);
                            ddy = fmaf(cdy[c], ny_hi[c][q] - ny_lo[c][q], ddy);
                        }
                        ddx = dscale(ddx, h.od[0], h.odl[0]);
                        ddy = dscale(ddy, h.od[1], h.odl[1]);
                        if (sx >= 0) ddx = cpml(ddx, pn0[q], pn0n[q], h.tab_h[0][x]);
                        if (syl >= 0) ddy = cpml(ddy, pn1[q], pn1n[q], h.tab_f[1][y]);
                        const float L2M = fmaf(2.f, M, L);
                        ux[q] = fmaf(L2M, ddx, L * ddy);
                        uy[q] = fmaf(L, ddx, L2M * ddy);
                        if (ZM != 0) {
                            float srxx = 0.f, sryy = 0.f;
                            const float dsum = ddx + ddy, ddif = 0.5f * (ddx - ddy);
#pragma unroll
                            for (int l = 0; l < R; ++l)
                                if (l < n_mech) {
                                    ra[l][q] = fmaf(p.zen.Ap[l], rxx[l][q], (p.zen.Bp[l] * gp) * dsum);
                                    rb[l][q] = fmaf(p.zen.As[l], ryy[l][q], (p.zen.Bs[l] * gs) * ddif);
                                    srxx += rxx[l][q] + ra[l][q];
                                    sryy += ryy[l][q] + rb[l][q];
                                }
                            const float hl = 0.5f * (L + M);
                            ux[q] = fmaf(hl, srxx, fmaf(M, sryy, ux[q]));
                            uy[q] = fmaf(hl, srxx, fmaf(-M, sryy, uy[q]));
                        }
                        ux[q] = sxx[q] + ux[q] * p.dt;   // (...) dt, wgsl:915-916
                        uy[q] = syy[q] + uy[q] * p.dt;
                    }
                    if (sx >= 0) sto<SPT>(h.psi[0] + ix, pn0n);
                    if (syl >= 0) sto<SPT>(h.psi[2] + iy, pn1n);
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) {
                                sto<SPT>(r0 + l * G + i, ra[l]);
                                sto<SPT>(r1 + l * G + i, rb[l]);
                            }
                    }
                    sto<SPT>(s0 + i, ux);
                    sto<SPT>(s1 + i, uy);
                }
                // ---- shear stress ----
                if (in_s) {
                    float u[SPT], ps0n[SPT], ps1n[SPT], rn[R][SPT];
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        float a = 0.f, b = 0.f;
#pragma unroll
                        for (int c = 0; c < ORD; ++c) {
                            a = fmaf(cdx[c], wvy[c + ORD][q] - wvy[ORD - 1 - c][q], a);
                            b = fmaf(cdy[c], sx_hi[c][q] - sx_lo[c][q], b);
                        }
                        a = dscale(a, h.od[0], h.odl[0]);
                        b = dscale(b, h.od[1], h.odl[1]);
                        if (sx >= 0) a = cpml(a, ps0[q], ps0n[q], h.tab_f[0][x]);
                        if (syl >= 0) b = cpml(b, ps1[q], ps1n[q], h.tab_h[1][y]);
                        const float e = a + b;
                        u[q] = Ms * e;
                        if (ZM != 0) {
                            float sr = 0.f;
#pragma unroll
                            for (int l = 0; l < R; ++l)
                                if (l < n_mech) {
                                    rn[l][q] = fmaf(p.zen.As[l], rxy[l][q], (p.zen.Bs[l] * gs) * e);
                                    sr += rxy[l][q] + rn[l][q];
                                }
                            u[q] = fmaf(0.5f * Ms, sr, u[q]);
                        }
                        u[q] = sxy[q] + u[q] * p.dt;
                    }
                    if (sx >= 0) sto<SPT>(h.psi[1] + ix, ps0n);
                    if (syl >= 0) sto<SPT>(h.psi[3] + iy, ps1n);
                    if (ZM != 0) {
#pragma unroll
                        for (int l = 0; l < R; ++l)
                            if (l < n_mech) sto<SPT>(r2 + l * G + i, rn[l]);
                    }
                    sto<SPT>(s2 + i, u);
                }
            }
            if (t + 1 < TX) {
                bshift<ORD, SPT, !FAST>(wvx, vx, x + ORD + 1, nx, X, col);
                bshift<ORD, SPT, !FAST>(wvy, vy, x + ORD, nx, X, col);
            }
        }
    };
    if (fast) sweep(std::true_type{});
    else sweep(std::false_type{});
    pdl_trigger();
}

template <int ORD, int CY, int TX, int SPT>
__global__ void __launch_bounds__(32 * CY, (MinBlocksV<CY>::v)) k_bvelocity(const __grid_constant__ BParams p,
                                                                              const int j) {
    constexpr int W = 32 * SPT, Y = W;
    const Loc at = locate<1, CY, TX, SPT>(p);
    const BPh &h = *at.ph;
    // per-phantom values used at every node, copied to registers once
    const int y = at.y, nx = h.nx, ny = h.ny;
    const int X = ny * W, col = (at.sb * nx * ny + y) * W + at.lane * SPT;
    const bool yvy = y >= ORD - 1 && y < ny - ORD;
    const bool yvx = yvy && y >= ORD;
    const int sy = at.live ? strip_index(h.strip[1], y) : -1;
    const Strip stx = h.strip[0];
    float cdx[ORD], cdy[ORD];
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        cdx[c] = p.coef[c];   // the sums are scaled by 1 / d after (dscale)
        cdy[c] = p.coef[c];
    }
    const float *__restrict__ sxx = h.s[0];  // read with ldf only
    const float *__restrict__ syy = h.s[1];
    const float *__restrict__ sxy = h.s[2];
    const float2 *__restrict__ dtw0 = h.dtw0;
    const float2 *__restrict__ dtw1 = h.dtw1;
    float *__restrict__ v0 = h.v[0];
    float *__restrict__ v1 = h.v[1];
    if (p.prefetch && at.live) {   // velocities (this kernel's previous launch) and dt / rho
#pragma unroll
        for (int t = 0; t < TX; ++t)
            if (at.x0 + t < nx) {
                const int i = at.i0 + t * X, cell = at.cell0 + t * ny;
                prefetch_l2(v0 + i);
                prefetch_l2(v1 + i);
                prefetch_l2(dtw0 + cell);
                prefetch_l2(dtw1 + cell);
            }
    }
    pdl_wait();
    const int k = *p.step_base + j;
    // source nodes among this thread's TX nodes: one bin per (x-chunk, y-block)
    int q0 = 0, q1 = 0;
    if (at.live && k < p.rows) {
        const int bin = (at.x0 / TX) * h.dc[1].yblocks + y / CY;
        q0 = __ldg(h.src_start + bin);
        q1 = __ldg(h.src_start + bin + 1);
    }
    unsigned vmax = 0u;  // max |v|^2 as float bits (v2 >= 0 or NaN: NaN ranks highest)
    bool bad = false;
    // Interior chunks (every node inside both update regions, outside the
    // CPML strips, window rows inside the grid, no source node) take a sweep
    // with no per-node region, strip, bounds or source tests.
    const bool fast = at.live && sy < 0 && q0 == q1 && y >= ORD && y < ny - ORD && at.x0 >= ORD &&
                      at.x0 >= stx.lo && at.x0 + TX + ORD <= nx && at.x0 + TX <= stx.hi;
    // The interior sweep issues every load of the thread's TX nodes before
    // the first update, so the thread waits for memory once, not once per
    // node: x rows x0-ORD .. x0+TX+ORD-2 of sxx and x0-ORD+1 .. x0+TX+ORD-1
    // of sxy, and per node the y-neighbours of sxy and syy, vx, vy, dt/rho.
    auto interior = [&]() {
        constexpr int NR = TX + 2 * ORD - 1;
        float rxx[NR][SPT], rxy[NR][SPT];
        float bxh[TX][ORD][SPT], bxl[TX][ORD][SPT], byh[TX][ORD][SPT], byl[TX][ORD][SPT];
        float vx0[TX][SPT], vy0[TX][SPT];
        float2 dx0[TX], dy0[TX];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            ldf<SPT>(rxx[r], sxx + (at.x0 - ORD + r) * X + col);
            ldf<SPT>(rxy[r], sxy + (at.x0 - ORD + 1 + r) * X + col);
        }
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int i = at.i0 + t * X, cell = at.cell0 + t * ny;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                ldf<SPT>(bxh[t][c], sxy + i + c * Y);         // sxy[y+c]
                ldf<SPT>(bxl[t][c], sxy + i - (c + 1) * Y);   // sxy[y-c-1]
                ldf<SPT>(byh[t][c], syy + i + (c + 1) * Y);   // syy[y+c+1]
                ldf<SPT>(byl[t][c], syy + i - c * Y);         // syy[y-c]
            }
            ldo<SPT>(vx0[t], v0 + i);
            ldo<SPT>(vy0[t], v1 + i);
            dx0[t] = __ldg(dtw0 + cell);
            dy0[t] = __ldg(dtw1 + cell);
        }
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int i = at.i0 + t * X;
            float vxn[SPT], vyn[SPT];
#pragma unroll
            for (int q = 0; q < SPT; ++q) {
                float ax = 0.f, bx = 0.f, ay = 0.f, by = 0.f;
#pragma unroll
                for (int c = 0; c < ORD; ++c) {
                    // rows x+c / x-c-1 of sxx and x+c+1 / x-c of sxy sit at t+ORD+c / t+ORD-1-c
                    ax = fmaf(cdx[c], rxx[t + ORD + c][q] - rxx[t + ORD - 1 - c][q], ax);
                    bx = fmaf(cdy[c], bxh[t][c][q] - bxl[t][c][q], bx);
                    ay = fmaf(cdx[c], rxy[t + ORD + c][q] - rxy[t + ORD - 1 - c][q], ay);
                    by = fmaf(cdy[c], byh[t][c][q] - byl[t][c][q], by);
                }
                ax = dscale(ax, h.od[0], h.odl[0]);
                bx = dscale(bx, h.od[1], h.odl[1]);
                ay = dscale(ay, h.od[0], h.odl[0]);
                by = dscale(by, h.od[1], h.odl[1]);
                vxn[q] = wgsl_velocity(vx0[t][q], ax + bx, dx0[t]);
                vyn[q] = wgsl_velocity(vy0[t][q], ay + by, dy0[t]);
                const float v2 = fmaf(vxn[q], vxn[q], vyn[q] * vyn[q]);
                bad |= !(v2 <= p.v2_threshold);
                vmax = max(vmax, __float_as_uint(v2));
            }
            sto<SPT>(v0 + i, vxn);
            sto<SPT>(v1 + i, vyn);
        }
    };
    // The general sweep (every region, strip, bounds and source test); the
    // interior sweep above replaces its FAST instantiation.
    auto sweep = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        const int syl = FAST ? -1 : sy;
        // sxx rows [x-ORD, x+ORD-1] (vx), sxy rows [x-ORD+1, x+ORD] (vy)
        float wxx[2 * ORD][SPT], wxy[2 * ORD][SPT];
        bwindow<ORD, SPT, !FAST>(wxx, sxx, at.x0 - ORD, nx, X, col);
        bwindow<ORD, SPT, !FAST>(wxy, sxy, at.x0 - ORD + 1, nx, X, col);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = at.x0 + t;
            if (!FAST && x >= nx) break;
            const int cell = at.cell0 + t * h.ny;
            const int i = at.i0 + t * X;
            const bool in_vy = FAST || (yvy && x >= ORD - 1 && x < nx - ORD);
            const bool in_vx = FAST || (yvx && in_vy && x >= ORD);
            const int sx = FAST ? -1 : strip_index(stx, x);
            const int ix = ((at.sb * stx.width + sx) * ny + y) * W + at.lane * SPT;
            const int iy = ((at.sb * nx + x) * h.strip[1].width + syl) * W + at.lane * SPT;
            // ---- loads ----
            float bx_hi[ORD][SPT], bx_lo[ORD][SPT], by_hi[ORD][SPT], by_lo[ORD][SPT];
            float vx0[SPT], vy0[SPT], pxa[SPT], pxb[SPT], pya[SPT], pyb[SPT];
            float2 dx0 = make_float2(0.f, 0.f), dy0 = make_float2(0.f, 0.f);
            if (in_vx) {
#pragma unroll
                for (int c = 0; c < ORD; ++c) {
                    ldf<SPT>(bx_hi[c], sxy + i + c * Y);         // sxy[y+c]
                    ldf<SPT>(bx_lo[c], sxy + i - (c + 1) * Y);   // sxy[y-c-1]
                }
                ldo<SPT>(vx0, v0 + i);
                dx0 = __ldg(dtw0 + cell);
                if (sx >= 0) ldo<SPT>(pxa, h.psi[4] + ix);
                if (syl >= 0) ldo<SPT>(pxb, h.psi[6] + iy);
            }
            if (in_vy) {
#pragma unroll
                for (int c = 0; c < ORD; ++c) {
                    ldf<SPT>(by_hi[c], syy + i + (c + 1) * Y);   // syy[y+c+1]
                    ldf<SPT>(by_lo[c], syy + i - c * Y);         // syy[y-c]
                }
                ldo<SPT>(vy0, v1 + i);
                dy0 = __ldg(dtw1 + cell);
                if (sx >= 0) ldo<SPT>(pya, h.psi[5] + ix);
                if (syl >= 0) ldo<SPT>(pyb, h.psi[7] + iy);
            }
            // ---- update ----
            float vxn[SPT], vyn[SPT], pxan[SPT], pxbn[SPT], pyan[SPT], pybn[SPT];
#pragma unroll
            for (int q = 0; q < SPT; ++q) {
                vxn[q] = 0.f;
                vyn[q] = 0.f;
                if (in_vx) {
                    float a = 0.f, b = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        a = fmaf(cdx[c], wxx[c + ORD][q] - wxx[ORD - 1 - c][q], a);
                        b = fmaf(cdy[c], bx_hi[c][q] - bx_lo[c][q], b);
                    }
                    a = dscale(a, h.od[0], h.odl[0]);
                    b = dscale(b, h.od[1], h.odl[1]);
                    if (sx >= 0) a = cpml(a, pxa[q], pxan[q], h.tab_f[0][x]);
                    if (syl >= 0) b = cpml(b, pxb[q], pxbn[q], h.tab_f[1][y]);
                    vxn[q] = wgsl_velocity(vx0[q], a + b, dx0);
                }
                if (in_vy) {
                    float a = 0.f, b = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        a = fmaf(cdx[c], wxy[c + ORD][q] - wxy[ORD - 1 - c][q], a);
                        b = fmaf(cdy[c], by_hi[c][q] - by_lo[c][q], b);
                    }
                    a = dscale(a, h.od[0], h.odl[0]);
                    b = dscale(b, h.od[1], h.odl[1]);
                    if (sx >= 0) a = cpml(a, pya[q], pyan[q], h.tab_h[0][x]);
                    if (syl >= 0) b = cpml(b, pyb[q], pybn[q], h.tab_h[1][y]);
                    vyn[q] = wgsl_velocity(vy0[q], a + b, dy0);
                }
                const int shot = at.s0 + q;
                if (!FAST && q0 < q1 && shot < h.n_shots)
                    for (int qq = q0; qq < q1; ++qq) {
                        const BSrc s = h.src[qq];
                        if (s.cell == cell)
                            vyn[q] += wgsl_source(__ldg(h.shot_tab + ((int64_t)shot * p.rows + k) * h.ncol + s.col),
                                                  s.scale, p.dt);
                    }
                const float v2 = fmaf(vxn[q], vxn[q], vyn[q] * vyn[q]);
                bad |= !(v2 <= p.v2_threshold);
                vmax = max(vmax, __float_as_uint(v2));
            }
            if (in_vx) {
                if (sx >= 0) sto<SPT>(h.psi[4] + ix, pxan);
                if (syl >= 0) sto<SPT>(h.psi[6] + iy, pxbn);
            }
            if (in_vy) {
                if (sx >= 0) sto<SPT>(h.psi[5] + ix, pyan);
                if (syl >= 0) sto<SPT>(h.psi[7] + iy, pybn);
            }
            sto<SPT>(v0 + i, vxn);
            sto<SPT>(v1 + i, vyn);
            if (t + 1 < TX) {
                bshift<ORD, SPT, !FAST>(wxx, sxx, x + ORD, nx, X, col);
                bshift<ORD, SPT, !FAST>(wxy, sxy, x + ORD + 1, nx, X, col);
            }
        }
    };
    if (fast) interior();
    else if (at.live) sweep(std::false_type{});
    // receivers: flat work item g = (phantom, shot, receiver)
    const int g = blockIdx.x * (32 * CY) + threadIdx.y * 32 + threadIdx.x;
    if (g < p.rec_work) {
        int q = 0;
        while (q + 1 < p.n_ph && g >= p.ph[q + 1].rec_work0) ++q;
        const BPh &r = p.ph[q];
        const int w = g - r.rec_work0, shot = w / r.n_rec, rec = w % r.n_rec;
        if (k >= __ldg(r.rec_first + rec)) {
            float acc = 0.f;
            for (int t = __ldg(r.rec_start + rec); t < __ldg(r.rec_start + rec + 1); ++t)
                acc += __ldca(r.s[1] + ((shot / r.W) * r.nx * r.ny + __ldg(r.rec_cell + t)) * r.W + shot % r.W);
            r.traces[((int64_t)shot * p.rows + k) * r.n_rec + rec] = acc;
        }
    }
    warp_stability(__uint_as_float(vmax), bad, reinterpret_cast<unsigned *>(p.block_max) + blockIdx.x, p.first_bad, k);
    pdl_trigger();
}

template <int ORD, int CY, int TX, int SPT>
void launch_shape(const BParams &p, int n_blocks, int zen_mode, int j, cudaStream_t st, int parts) {
    const dim3 block(32, CY), grid(n_blocks);
    const bool three = p.zen.n == 3;
    if (parts & 1) {
        if (zen_mode == 0) launch_pdl(k_bstress<ORD, 0, 0, CY, TX, SPT>, grid, block, st, p);
        else if (zen_mode == 1 && three) launch_pdl(k_bstress<ORD, 1, 3, CY, TX, SPT>, grid, block, st, p);
        else if (zen_mode == 1) launch_pdl(k_bstress<ORD, 1, kMaxSls, CY, TX, SPT>, grid, block, st, p);
        else if (three) launch_pdl(k_bstress<ORD, 2, 3, CY, TX, SPT>, grid, block, st, p);
        else launch_pdl(k_bstress<ORD, 2, kMaxSls, CY, TX, SPT>, grid, block, st, p);
    }
    if (parts & 2) launch_pdl(k_bvelocity<ORD, CY, TX, SPT>, grid, block, st, p, j);
}

// Launch shapes: blocks of 32 lanes x CY nodes along y, TX nodes per thread
// along x, SPT shots per lane.  Order 2 has every shape of the autotuner; order
// 4 has the default shape only.
template <int ORD>
void launch_ord(const BParams &p, int n_blocks, int cy, int tx, int spt, int zen_mode, int j, cudaStream_t st,
                int parts) {
    if constexpr (ORD == 2) {
        if (spt == 2) {
            if (cy == 4 && tx == 1) return launch_shape<ORD, 4, 1, 2>(p, n_blocks, zen_mode, j, st, parts);
            if (cy == 4 && tx == 2) return launch_shape<ORD, 4, 2, 2>(p, n_blocks, zen_mode, j, st, parts);
            if (cy == 4) return launch_shape<ORD, 4, 4, 2>(p, n_blocks, zen_mode, j, st, parts);
            if (tx == 1) return launch_shape<ORD, 8, 1, 2>(p, n_blocks, zen_mode, j, st, parts);
            if (tx == 2) return launch_shape<ORD, 8, 2, 2>(p, n_blocks, zen_mode, j, st, parts);
            return launch_shape<ORD, 8, 4, 2>(p, n_blocks, zen_mode, j, st, parts);
        }
        if (cy == 4 && tx == 1) return launch_shape<ORD, 4, 1, 1>(p, n_blocks, zen_mode, j, st, parts);
        if (cy == 4 && tx == 2) return launch_shape<ORD, 4, 2, 1>(p, n_blocks, zen_mode, j, st, parts);
        if (cy == 4) return launch_shape<ORD, 4, 4, 1>(p, n_blocks, zen_mode, j, st, parts);
        if (cy == 8 && tx == 1) return launch_shape<ORD, 8, 1, 1>(p, n_blocks, zen_mode, j, st, parts);
        if (cy == 8 && tx == 4) return launch_shape<ORD, 8, 4, 1>(p, n_blocks, zen_mode, j, st, parts);
    }
    launch_shape<ORD, 8, 2, 1>(p, n_blocks, zen_mode, j, st, parts);
}

// One time step: the stress launch (shape 0) then the velocity launch (shape
// 1); `parts` selects them (bit 0 stress, bit 1 velocity).
void launch_batch(const BParams &p, const int (&n_blocks)[2], int ord, const int (&cy)[2], const int (&tx)[2], int spt,
                  int zen_mode, int j, cudaStream_t st, int parts = 3) {
    for (int k = 0; k < 2; ++k) {
        if (!(parts & (1 << k))) continue;
        switch (ord) {
        case 2: launch_ord<2>(p, n_blocks[k], cy[k], tx[k], spt, zen_mode, j, st, 1 << k); break;
        case 4: launch_ord<4>(p, n_blocks[k], cy[k], tx[k], spt, zen_mode, j, st, 1 << k); break;
        default: break;
        }
    }
}

thread_local std::string g_batch_error;

int bfail(int code, const std::string &m) {
    g_batch_error = m;
    return code;
}

}  // namespace
}  // namespace ts

using namespace ts;

struct ts_batch {
    int device = 0, ord = 2, spt = 1, zen_mode = 0, rows = 0;
    int cy[2] = {8, 8}, tx[2] = {2, 2}, n_blocks[2] = {0, 0};  // stress, velocity launch shapes
    int steps_done = 0, n_ph = 0;
    int64_t launches = 0, h2d_bytes = 0, d2h_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<void *> allocs;
    std::vector<std::pair<void *, size_t>> state;
    std::vector<BPh> ph;
    BParams p{};
    std::vector<int> shots, nrec, ncol, cells;

    template <typename T>
    int alloc(T **ptr, size_t n, bool is_state) {
        void *d = nullptr;
        const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&d, bytes);
        if (e != cudaSuccess) return bfail(TS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(d);
        if (is_state) state.push_back({d, bytes});
        *ptr = static_cast<T *>(d);
        return TS_OK;
    }
    template <typename T>
    int upload(T **ptr, const std::vector<T> &h) {
        int rc = alloc(ptr, h.size(), false);
        if (rc) return rc;
        if (!h.empty() && cudaMemcpy(*ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
            return bfail(TS_E_CUDA, "cudaMemcpy");
        h2d_bytes += (int64_t)(h.size() * sizeof(T));
        return TS_OK;
    }
};

extern "C" {

void ts_batch_destroy(ts_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->done) cudaEventSynchronize(b->done);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void *d : b->allocs) cudaFree(d);
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char *ts_batch_last_error(void) { return g_batch_error.c_str(); }

int ts_batch_reset(ts_batch *b, void *stream) {
    if (!b) return bfail(TS_E_ARG, "null handle");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    for (auto &s : b->state)
        if (cudaMemsetAsync(s.first, 0, s.second, st) != cudaSuccess) return bfail(TS_E_CUDA, "cudaMemsetAsync");
    launch_reset_scalars(b->p.first_bad, const_cast<int *>(b->p.step_base), st);
    b->launches += 1;
    if (cudaEventRecord(b->done, st) != cudaSuccess) return bfail(TS_E_CUDA, "cudaEventRecord");
    b->steps_done = 0;
    if (!stream && cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(TS_E_CUDA, "sync");
    return TS_OK;
}

int ts_batch_create(const ts_batch_desc *bd, ts_batch **out) {
    if (!out || !bd) return bfail(TS_E_ARG, "null argument");
    *out = nullptr;
    if (bd->abi_version != TS_ABI_VERSION) return bfail(TS_E_ARG, "abi_version mismatch");
    if (bd->n_phantoms < 1 || bd->n_phantoms > kMaxPhantoms) return bfail(TS_E_ARG, "n_phantoms must be in [1, 8]");
    if (!bd->phantoms || !bd->n_shots || !bd->shot_sources) return bfail(TS_E_ARG, "missing phantom tables");
    const int cells[2] = {bd->block_cells, bd->velocity_block_cells};
    const int nodes[2] = {bd->nodes_per_thread, bd->velocity_nodes_per_thread};
    for (int k = 0; k < 2; ++k) {
        if (!(cells[k] == 0 || cells[k] == 4 || cells[k] == 8))
            return bfail(TS_E_ARG, "block_cells must be 0 (default), 4 or 8");
        if (!(nodes[k] == 0 || nodes[k] == 1 || nodes[k] == 2 || nodes[k] == 4))
            return bfail(TS_E_ARG, "nodes_per_thread must be 0 (default), 1, 2 or 4");
        if (bd->phantoms && bd->phantoms->ord == 4 && !((cells[k] == 0 || cells[k] == 8) && (nodes[k] == 0 || nodes[k] == 2)))
            return bfail(TS_E_ARG, "order-4 batches take the default launch shape (8 cells, 2 nodes, 1 shot per thread)");
    }
    if (!(bd->shots_per_thread == 0 || bd->shots_per_thread == 1 || bd->shots_per_thread == 2))
        return bfail(TS_E_ARG, "shots_per_thread must be 0 (default), 1 or 2");
    if (bd->phantoms && bd->phantoms->ord == 4 && bd->shots_per_thread > 1)
        return bfail(TS_E_ARG, "order-4 batches take the default launch shape (8 cells, 2 nodes, 1 shot per thread)");
    const ts_desc *d0 = bd->phantoms;
    for (int q = 0; q < bd->n_phantoms; ++q) {
        const ts_desc *d = bd->phantoms + q;
        if (d->family != TS_WGSL2D) return bfail(TS_E_ARG, "batched stepping supports the TS_WGSL2D family");
        if (d->ord != 2 && d->ord != 4) return bfail(TS_E_ARG, "batched stepping supports ord 2 and 4");
        if (d->ord != d0->ord || d->dt != d0->dt || d->n_steps != d0->n_steps || d->visco != d0->visco ||
            (d->g_p == nullptr) != (d0->g_p == nullptr) || (d->visco && d->n_sls != d0->n_sls))
            return bfail(TS_E_ARG, "phantoms of one batch must share ord, dt, n_steps and attenuation model");
        if (d->nx < 2 * d->ord + 1 || d->ny < 2 * d->ord + 1 || d->nz != 1) return bfail(TS_E_ARG, "bad grid");
        if (bd->n_shots[q] < 1) return bfail(TS_E_ARG, "every phantom needs at least one shot");
        if (!bd->shot_sources[q]) return bfail(TS_E_ARG, "missing shot source table");
        if (!d->rho || !d->cp || !d->cs || !d->pos_sources || !d->coefs || !d->a_x || !d->a_y || !d->b_x ||
            !d->b_y || !d->k_x || !d->k_y || !d->a_xh || !d->b_xh || !d->k_xh || !d->a_yh || !d->b_yh || !d->k_yh)
            return bfail(TS_E_ARG, "missing table");
        if (d->n_rec > 0 && (!d->info_rec_pt || !d->offset_sensors || !d->delay_rec))
            return bfail(TS_E_ARG, "missing receiver tables");
        if (d->visco && !d->g_p && (!d->tau || !d->sum_alpha)) return bfail(TS_E_ARG, "missing Zener tables");
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return bfail(TS_E_CUDA, "cudaGetDevice");
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bfail(TS_E_CUDA, "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3)) return bfail(TS_E_NODEV, "this library is built for sm_103a only");

    ts_batch *b = new ts_batch();
    auto bail = [&](int rc) {
        ts_batch_destroy(b);
        return rc;
    };
    b->device = device;
    b->ord = d0->ord;
    b->rows = d0->n_steps;
    b->n_ph = bd->n_phantoms;
    b->cy[0] = bd->block_cells ? bd->block_cells : 8;
    b->tx[0] = bd->nodes_per_thread ? bd->nodes_per_thread : 2;
    b->cy[1] = bd->velocity_block_cells ? bd->velocity_block_cells : b->cy[0];
    b->tx[1] = bd->velocity_nodes_per_thread ? bd->velocity_nodes_per_thread : b->tx[0];
    b->spt = bd->shots_per_thread ? bd->shots_per_thread : 1;
    b->zen_mode = !d0->visco ? 0 : (d0->g_p ? 2 : 1);
    b->ph.resize(b->n_ph);
    int block0[2] = {0, 0}, rec0 = 0, rc;
    for (int q = 0; q < b->n_ph; ++q) {
        const ts_desc *d = bd->phantoms + q;
        BPh &h = b->ph[q];
        h = BPh{};
        h.nx = d->nx;
        h.ny = d->ny;
        h.n_shots = bd->n_shots[q];
        h.W = 32 * b->spt;
        h.S = round_up(h.n_shots, h.W);
        if ((int64_t)h.nx * h.ny * h.S * std::max(1, d->visco ? d->n_sls : 1) >= (int64_t)1 << 31)
            return bail(bfail(TS_E_ARG, "phantom too large for one batch (nodes x shots x mechanisms >= 2^31)"));
        h.G = h.nx * h.ny * h.S;

        h.sblocks = h.S / h.W;
        for (int k = 0; k < 2; ++k) {
            Decomp &dc = h.dc[k];
            dc.yblocks = (h.ny + b->cy[k] - 1) / b->cy[k];
            dc.xchunks = (h.nx + b->tx[k] - 1) / b->tx[k];
            dc.block0 = block0[k];
            block0[k] += dc.xchunks * dc.yblocks * h.sblocks;
        }
        const float steps[2] = {d->dx, d->dy};
        for (int a = 0; a < 2; ++a) {
            h.od[a] = 1.f / steps[a];
            h.odl[a] = (float)(1.0 / (double)steps[a] - (double)h.od[a]);
        }
        Axis ax[2] = {make_axis(h.nx, d->ord, d->a_x, d->b_x, d->k_x, d->a_xh, d->b_xh, d->k_xh),
                      make_axis(h.ny, d->ord, d->a_y, d->b_y, d->k_y, d->a_yh, d->b_yh, d->k_yh)};
        for (int a = 0; a < 2; ++a) {
            Cpml *f = nullptr, *hh = nullptr;
            if ((rc = b->upload(&f, ax[a].full)) || (rc = b->upload(&hh, ax[a].half))) return bail(rc);
            h.tab_f[a] = f;
            h.tab_h[a] = hh;
            h.strip[a] = ax[a].strip;
        }
        for (int f = 0; f < 2; ++f)
            if ((rc = b->alloc(&h.v[f], h.G, true))) return bail(rc);
        for (int f = 0; f < 3; ++f)
            if ((rc = b->alloc(&h.s[f], h.G, true))) return bail(rc);
        const int64_t xs = (int64_t)h.strip[0].width * h.ny * h.S, ys = (int64_t)h.nx * h.strip[1].width * h.S;
        const int64_t psz[8] = {xs, xs, ys, ys, xs, xs, ys, ys};
        for (int k = 0; k < 8; ++k)
            if ((rc = b->alloc(&h.psi[k], psz[k], true))) return bail(rc);
        if (d->visco)
            for (int m = 0; m < 3; ++m)
                if ((rc = b->alloc(&h.r[m], (size_t)h.G * d->n_sls, true))) return bail(rc);
        // per-node coefficients, shared by every shot
        const int64_t cells = (int64_t)h.nx * h.ny;
        std::vector<float> lam(cells), mu(cells), mus(cells), dtr0(cells), dtr1(cells), rho_vy(cells);
        for (int x = 0; x < h.nx; ++x)
            for (int y = 0; y < h.ny; ++y) {
                const Coef2D c = coef_2d(d, x, y);
                const int64_t i = (int64_t)x * h.ny + y;
                lam[i] = c.lam_raw;
                mu[i] = c.mu_raw;
                mus[i] = c.mus_raw;
                dtr0[i] = c.rho_vx;
                dtr1[i] = c.rho_vy;
                rho_vy[i] = c.rho_vy;
            }
        float *dev = nullptr;
        if ((rc = b->upload(&dev, lam))) return bail(rc);
        h.lam = dev;
        if ((rc = b->upload(&dev, mu))) return bail(rc);
        h.mu = dev;
        if ((rc = b->upload(&dev, mus))) return bail(rc);
        h.mus = dev;
        for (int c = 0; c < 2; ++c) {   // dt / rho as (hi, lo), computed in double
            const std::vector<float> &rh = c == 0 ? dtr0 : dtr1;
            std::vector<float2> w(rh.size(), make_float2(0.f, 0.f));
            for (size_t i = 0; i < rh.size(); ++i)
                if (rh[i] > 0.f) {
                    const double q = (double)d->dt / (double)rh[i];
                    const float hi = (float)q;
                    w[i] = make_float2(hi, (float)(q - (double)hi));
                }
            float2 *dw = nullptr;
            if ((rc = b->upload(&dw, w))) return bail(rc);
            (c == 0 ? h.dtw0 : h.dtw1) = dw;
        }
        if (b->zen_mode == 2) {
            std::vector<float> gp(d->g_p, d->g_p + cells), gs(d->g_s, d->g_s + cells);
            if ((rc = b->upload(&dev, gp))) return bail(rc);
            h.gp = dev;
            if ((rc = b->upload(&dev, gs))) return bail(rc);
            h.gs = dev;
        }
        // sources: nodes of the source map, binned by (x-chunk, y-block)
        std::vector<std::vector<BSrc>> bins((size_t)h.dc[1].xchunks * h.dc[1].yblocks);
        int maxcol = 0;
        for (int x = 0; x < h.nx; ++x)
            for (int y = 0; y < h.ny; ++y) {
                const int idx = d->pos_sources[(int64_t)x * h.ny + y];
                const float r4 = rho_vy[(int64_t)x * h.ny + y];
                if (idx < 0 || idx >= d->src_cols || !(r4 > 0.f)) continue;
                bins[(size_t)(x / b->tx[1]) * h.dc[1].yblocks + y / b->cy[1]].push_back(BSrc{x * h.ny + y, idx, r4});
                maxcol = std::max(maxcol, idx + 1);
            }
        std::vector<BSrc> list;
        std::vector<int> start(1, 0);
        for (auto &v : bins) {
            list.insert(list.end(), v.begin(), v.end());
            start.push_back((int)list.size());
        }
        BSrc *dsrc = nullptr;
        int *dstart = nullptr;
        if ((rc = b->upload(&dsrc, list)) || (rc = b->upload(&dstart, start))) return bail(rc);
        h.src = dsrc;
        h.src_start = dstart;
        h.ncol = d->src_cols;
        std::vector<float> tab(bd->shot_sources[q], bd->shot_sources[q] + (size_t)h.n_shots * b->rows * d->src_cols);
        float *dtab = nullptr;
        if ((rc = b->upload(&dtab, tab))) return bail(rc);
        h.shot_tab = dtab;
        // receivers (WGSL order over info_rec_pt)
        std::vector<int> rstart(1, 0), rcell, rfirst(std::max(1, d->n_rec), 0);
        const int rec_groups = receiver_groups(d, 3);
        for (int r = 0; r < d->n_rec; ++r) {
            for (int pt = receiver_first_point(d, r, rec_groups); pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * 3 + 2] == r; ++pt) {
                const int x = d->info_rec_pt[pt * 3], y = d->info_rec_pt[pt * 3 + 1];
                if (x >= 0 && x < h.nx && y >= 0 && y < h.ny) rcell.push_back(x * h.ny + y);
            }
            rstart.push_back((int)rcell.size());
            rfirst[r] = d->delay_rec[r];
        }
        int *d1 = nullptr, *d2 = nullptr, *d3 = nullptr;
        if ((rc = b->upload(&d1, rstart)) || (rc = b->upload(&d2, rcell)) || (rc = b->upload(&d3, rfirst))) return bail(rc);
        h.n_rec = d->n_rec;
        h.rec_start = d1;
        h.rec_cell = d2;
        h.rec_first = d3;
        if ((rc = b->alloc(&h.traces, (size_t)h.n_shots * b->rows * std::max(1, d->n_rec), true))) return bail(rc);
        h.rec_work0 = rec0;
        rec0 += h.n_shots * d->n_rec;
        b->shots.push_back(h.n_shots);
        b->nrec.push_back(d->n_rec);
        b->ncol.push_back(d->src_cols);
        b->cells.push_back(h.nx * h.ny);
    }
    BParams &p = b->p;
    p.n_ph = b->n_ph;
    for (int q = 0; q < b->n_ph; ++q) p.ph[q] = b->ph[q];
    for (int k = 0; k < 2; ++k) {
        b->n_blocks[k] = block0[k];
        for (int q = 0; q < kMaxPhantoms; ++q) {
            const Decomp &dc = b->ph[std::min(q, b->n_ph - 1)].dc[k];
            p.block_end[k][q] = q < b->n_ph ? dc.block0 + dc.xchunks * dc.yblocks * b->ph[q].sblocks : block0[k];
        }
    }
    if ((int64_t)rec0 > (int64_t)block0[1] * 32 * b->cy[1])
        return bail(bfail(TS_E_ARG, "more (shot, receiver) pairs than threads of a step launch"));
    p.zen = zener_constants(d0);
    for (int c = 0; c < kMaxOrd; ++c) p.coef[c] = c < d0->ord ? d0->coefs[c] : 0.f;
    p.dt = d0->dt;
    p.rows = b->rows;
    p.v2_threshold = FLT_MAX;
    p.rec_work = rec0;
    // L2 prefetch of each thread's own state before the wait (FMC 46.3 ->
    // 47.6 Gcell/s); TS_BATCH_PREFETCH=0 turns it off
    const char *pf = getenv("TS_BATCH_PREFETCH");
    p.prefetch = !(pf && pf[0] == '0');
    if ((rc = b->alloc(&p.block_max, b->n_blocks[1], true))) return bail(rc);
    int *fb = nullptr, *sb = nullptr;
    if ((rc = b->alloc(&fb, 1, false)) || (rc = b->alloc(&sb, 1, false))) return bail(rc);
    p.first_bad = fb;
    p.step_base = sb;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess)
        return bail(bfail(TS_E_CUDA, "stream/event creation"));
    if ((rc = ts_batch_reset(b, nullptr))) return bail(rc);
    *out = b;
    return TS_OK;
}

int ts_batch_run(ts_batch *b, int32_t n_steps, void *stream) {
    if (!b) return bfail(TS_E_ARG, "null handle");
    if (n_steps < 0 || b->steps_done + (int64_t)n_steps > b->rows) return bfail(TS_E_ARG, "steps beyond n_steps");
    cudaSetDevice(b->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    constexpr int G = 16;
    auto steps = [&](int count, cudaStream_t where) {
        for (int j = 0; j < count; ++j)
            launch_batch(b->p, b->n_blocks, b->ord, b->cy, b->tx, b->spt, b->zen_mode, j, where);
        launch_advance(const_cast<int *>(b->p.step_base), count, where);
    };
    if (!b->graph && n_steps >= G) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return bfail(TS_E_CUDA, "capture");
        steps(G, b->stream);
        if (cudaStreamEndCapture(b->stream, &g) != cudaSuccess) return bfail(TS_E_CUDA, "end capture");
        cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(TS_E_CUDA, std::string("graph: ") + cudaGetErrorString(e));
    }
    int left = n_steps;
    while (left >= G && b->graph) {
        if (cudaGraphLaunch(b->graph, st) != cudaSuccess) return bfail(TS_E_CUDA, "cudaGraphLaunch");
        b->launches += 2 * G + 1;
        left -= G;
    }
    if (left > 0) {
        steps(left, st);
        b->launches += 2 * left + 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return bfail(TS_E_CUDA, cudaGetErrorString(e));
    cudaEventRecord(b->done, st);
    b->steps_done += n_steps;
    return TS_OK;
}

int ts_batch_status(ts_batch *b, int32_t *steps_done, float *max_v2, int32_t *first_unstable) {
    if (!b) return bfail(TS_E_ARG, "null handle");
    cudaEventSynchronize(b->done);
    if (steps_done) *steps_done = b->steps_done;
    if (max_v2) {
        std::vector<unsigned> bm(b->n_blocks[1]);
        if (cudaMemcpy(bm.data(), b->p.block_max, bm.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return bfail(TS_E_CUDA, "cudaMemcpy");
        unsigned m = 0;
        for (unsigned v : bm) m = std::max(m, v);
        float f;
        memcpy(&f, &m, 4);
        *max_v2 = f;
    }
    if (first_unstable) {
        int fb = 0;
        if (cudaMemcpy(&fb, b->p.first_bad, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return bfail(TS_E_CUDA, "cudaMemcpy");
        *first_unstable = fb == 0x7fffffff ? -1 : fb;
    }
    return TS_OK;
}

int ts_batch_read_traces(ts_batch *b, int32_t phantom, void *dst, size_t bytes) {
    if (!b || !dst || phantom < 0 || phantom >= b->n_ph) return bfail(TS_E_ARG, "bad argument");
    cudaEventSynchronize(b->done);
    const size_t need = (size_t)b->shots[phantom] * b->rows * b->nrec[phantom] * 4;
    if (bytes < need) return bfail(TS_E_ARG, "destination too small");
    if (need && cudaMemcpy(dst, b->ph[phantom].traces, need, cudaMemcpyDeviceToHost) != cudaSuccess)
        return bfail(TS_E_CUDA, "cudaMemcpy");
    b->d2h_bytes += (int64_t)need;
    return TS_OK;
}

int ts_batch_read_field(ts_batch *b, int32_t phantom, int32_t what, void *dst, size_t bytes) {
    if (!b || !dst || phantom < 0 || phantom >= b->n_ph) return bfail(TS_E_ARG, "bad argument");
    const BPh &h = b->ph[phantom];
    const float *src = what == TS_VX ? h.v[0] : what == TS_VY ? h.v[1] : what == TS_SXX ? h.s[0]
                     : what == TS_SYY ? h.s[1] : what == TS_SXY ? h.s[2] : nullptr;
    if (!src) return bfail(TS_E_ARG, "no such field");
    cudaEventSynchronize(b->done);
    const size_t need = (size_t)h.nx * h.ny * h.n_shots * 4;
    if (bytes < need) return bfail(TS_E_ARG, "destination too small");
    // device layout [S/W][nx][ny][W] -> host [n_shots][nx][ny]
    std::vector<float> tmp((size_t)h.G);
    if (cudaMemcpy(tmp.data(), src, tmp.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return bfail(TS_E_CUDA, "cudaMemcpy");
    b->d2h_bytes += (int64_t)(tmp.size() * 4);
    float *o = static_cast<float *>(dst);
    const int64_t cells = (int64_t)h.nx * h.ny;
    for (int s = 0; s < h.n_shots; ++s)
        for (int64_t c = 0; c < cells; ++c) o[s * cells + c] = tmp[((s / h.W) * cells + c) * h.W + (s % h.W)];
    return TS_OK;
}

int ts_batch_profile_steps(ts_batch *b, int32_t n_steps, void *stream, float *ms_per_kernel) {
    if (!b || !ms_per_kernel || n_steps < 1 || b->steps_done + (int64_t)n_steps > b->rows)
        return bfail(TS_E_ARG, "bad argument");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    std::vector<cudaEvent_t> ev(2 * n_steps + 1);
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], st);
    for (int j = 0; j < n_steps; ++j)
        for (int part = 0; part < 2; ++part) {
            launch_batch(b->p, b->n_blocks, b->ord, b->cy, b->tx, b->spt, b->zen_mode, j, st, 1 << part);
            cudaEventRecord(ev[2 * j + part + 1], st);
        }
    launch_advance(const_cast<int *>(b->p.step_base), n_steps, st);
    b->launches += 2 * (int64_t)n_steps + 1;
    cudaEventSynchronize(ev.back());
    double tot[2] = {0, 0};
    for (int j = 0; j < n_steps; ++j)
        for (int part = 0; part < 2; ++part) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[2 * j + part], ev[2 * j + part + 1]);
            tot[part] += ms;
        }
    for (auto &e : ev) cudaEventDestroy(e);
    ms_per_kernel[0] = (float)(tot[0] / n_steps);
    ms_per_kernel[1] = (float)(tot[1] / n_steps);
    cudaEventRecord(b->done, st);
    b->steps_done += n_steps;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TS_OK : bfail(TS_E_CUDA, cudaGetErrorString(e));
}

int ts_batch_launch_count(const ts_batch *b, int64_t *n) {
    if (!b || !n) return bfail(TS_E_ARG, "null argument");
    *n = b->launches;
    return TS_OK;
}

int ts_batch_transfer_bytes(const ts_batch *b, int64_t *h2d, int64_t *d2h) {
    if (!b) return bfail(TS_E_ARG, "null handle");
    if (h2d) *h2d = b->h2d_bytes;
    if (d2h) *d2h = b->d2h_bytes;
    return TS_OK;
}

}  // extern "C"
