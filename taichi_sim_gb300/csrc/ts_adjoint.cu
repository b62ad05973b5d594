// Discrete adjoint of the 2D (visco)elastic stepper (family TS_WGSL2D):
// gradient of a receiver-trace misfit with respect to the per-node
// coefficients the stepper uses, L = lambda*dt and M = mu*dt at the normal
// node, Ms = mu*dt at the shear node, Bx = dt/rho at the vx node and
// By = dt/rho at the vy node.  (A caller maps per-cell lambda, mu, rho to
// these with the reference's averaging and chains the gradient back.)
//
// Forward step n (shader_webgpu_viscoelastic.wgsl:829-1072):
//   stress:   d~ = ik d + p',  p' = b p + a d         (CPML, per derivative)
//             r'_l = A_l r_l + C_l g drive,  S = sum_l (r_l + r'_l)
//             sxx' = sxx + (L+2M) dx + L dy + (L+M)/2 Sxx + M Syy
//             syy' = syy + L dx + (L+2M) dy + (L+M)/2 Sxx - M Syy
//             sxy' = sxy + Ms e + Ms/2 Sxy,  e = dvy/dx~ + dvx/dy~
//   velocity: vx' = vx + Bx ax,  vy' = vy + By ay (+ source f_n By),
//             zero outside the vy region
//   receivers: trace_n = sum of syy' over each receiver's nodes.
// The update is linear in the state, so the adjoint runs the transposed
// operators backward in time and needs from the forward pass only the
// "features" that multiply the coefficients: (dx~, dy~, Sxx, Syy) at normal
// nodes, (e, Sxy) at shear nodes, (ax, ay) at velocity nodes - 8 floats per
// node and step.  They are kept for every step when they fit in memory
// (GB300's HBM holds a 512x1024 x 3000-step record in 50 GB), otherwise the
// forward state is checkpointed every K steps and each K-step segment is
// recomputed before its adjoint sweep (revolve-style, K ~ sqrt(steps)).
//
// Adjoint step n, from the adjoints of the state after step n:
//   K_vel(n):    velocity nodes - v^bar of step n+1 gathers the transposed
//                stress stencils of step n+1 (skipped for the last step);
//                then abar = B vbar, gB += vbar * a_feature, CPML adjoint
//                (q = pbar + abar, dbar = ik abar + a q, pbar <- b q) ->
//                dbar arrays; receiver residuals added to syy^bar.
//   K_str(n):    stress nodes - syy/sxx/sxy^bar gather the transposed
//                velocity stencils; gL, gM, gMs accumulate; Zener adjoint
//                (rho_l = rbar_l + Sbar, rbar_l <- A_l rho_l + Sbar,
//                drive^bar += C_l g rho_l); CPML adjoint -> dbar arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/taichi_sim_gb300.h"
#include "ts_internal.cuh"
#include "ts_prep.h"

namespace ts {
namespace {

constexpr int kF = 8;  // features per node and step
// feature slots
enum { F_DX = 0, F_DY, F_SXX, F_SYY, F_E, F_SXY, F_AX, F_AY };

struct AdjParams {
    int nx, ny, P, ord, zm;  // zm: 0 elastic, 1 global Zener, 2 per-cell Q
    int64_t G;               // nx * P
    float cd[2][kMaxOrd];
    Zener zen;
    const Cpml *tab_f[2], *tab_h[2];
    Strip strip[2];
    // coefficients (caller's device arrays, [nx][P])
    const float *L, *M, *Ms, *Bx, *By, *gp, *gs;
    // forward state
    float *vx, *vy, *sxx, *syy, *sxy, *r[3], *psi[8];
    // features of the step being run: [kF][G] (null: not recorded)
    float *feat;
    // sources (plain list; few nodes)
    int n_src;
    const int64_t *src_cell;
    const int *src_col;
    const float *src_tab;  // [rows][ncol]
    int ncol, rows;
    // receivers
    int n_rec;
    const int *rec_start;
    const int64_t *rec_cell;
    const int *rec_first;
    float *traces;  // [rows][n_rec]
    // adjoint state
    float *avx, *avy, *asxx, *asyy, *asxy, *ar[3], *apsi[8];
    float *dv[4];  // stress-node dbar: dx (normal), dy (normal), e_x (shear, dvy/dx), e_y (shear, dvx/dy)
    float *ds[4];  // velocity-node dbar: ax_x, ax_y (vx), ay_x, ay_y (vy)
    float *gL, *gM, *gMs, *gBx, *gBy;
    const float *res;  // [rows][n_rec] trace residuals dJ/dtrace
};

__device__ __forceinline__ float cpml(float d, float p_old, float &p_new, const Cpml &t) {
    p_new = fmaf(t.b, p_old, t.a * d);
    return fmaf(d, t.ik, p_new);
}

// adjoint of cpml(): given dbar~ and the carried adjoint of p', returns dbar
// and replaces pbar by the adjoint of the previous step's p'
__device__ __forceinline__ float cpml_adj(float dt_bar, float &pbar, const Cpml &t) {
    const float q = pbar + dt_bar;
    pbar = t.b * q;
    return fmaf(t.ik, dt_bar, t.a * q);
}

constexpr int BX = 32, BY = 8;

struct Node {
    int x, y;
    int64_t i;
    bool live;
};

__device__ __forceinline__ Node node(const AdjParams &p) {
    Node n;
    n.y = blockIdx.x * BX + threadIdx.x;
    n.x = blockIdx.y * BY + threadIdx.y;
    n.live = n.x < p.nx && n.y < p.ny;
    n.i = (int64_t)n.x * p.P + n.y;
    return n;
}

template <int ORD>
__device__ __forceinline__ bool in_normal(const AdjParams &p, int x, int y) {
    return x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1;
}
template <int ORD>
__device__ __forceinline__ bool in_shear(const AdjParams &p, int x, int y) {
    return x >= ORD && x < p.nx - ORD + 1 && y >= ORD - 1 && y < p.ny - ORD;
}
template <int ORD>
__device__ __forceinline__ bool in_vy(const AdjParams &p, int x, int y) {
    return x >= ORD - 1 && x < p.nx - ORD && y >= ORD - 1 && y < p.ny - ORD;
}
template <int ORD>
__device__ __forceinline__ bool in_vx(const AdjParams &p, int x, int y) {
    return in_vy<ORD>(p, x, y) && x >= ORD && y >= ORD;
}

// ------------------------------------------------------------------ forward
template <int ORD, int ZM>
__global__ void __launch_bounds__(BX *BY) k_fwd_stress(const AdjParams p) {
    const Node n = node(p);
    if (!n.live) return;
    const int x = n.x, y = n.y, P = p.P;
    const int64_t i = n.i;
    const bool nn = in_normal<ORD>(p, x, y), ss = in_shear<ORD>(p, x, y);
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
    const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;
    const int L3 = ZM ? p.zen.n : 0;
    if (nn) {
        float ddx = 0.f, ddy = 0.f, np_;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            ddx = fmaf(p.cd[0][c], p.vx[i + (int64_t)(c + 1) * P] - p.vx[i - (int64_t)c * P], ddx);
            ddy = fmaf(p.cd[1][c], p.vy[i + c] - p.vy[i - c - 1], ddy);
        }
        if (sx >= 0) {
            ddx = cpml(ddx, p.psi[0][ix], np_, p.tab_h[0][x]);
            p.psi[0][ix] = np_;
        }
        if (sy >= 0) {
            ddy = cpml(ddy, p.psi[2][iy], np_, p.tab_f[1][y]);
            p.psi[2][iy] = np_;
        }
        const float L = p.L[i], M = p.M[i], L2M = fmaf(2.f, M, L);
        float ux = fmaf(L2M, ddx, L * ddy), uy = fmaf(L, ddx, L2M * ddy), srx = 0.f, sry = 0.f;
        if (ZM) {
            const float gp = ZM == 2 ? p.gp[i] : 1.f, gs = ZM == 2 ? p.gs[i] : 1.f;
            const float dsum = ddx + ddy, ddif = 0.5f * (ddx - ddy);
            for (int l = 0; l < L3; ++l) {
                float *rx = p.r[0] + l * p.G + i, *ry = p.r[1] + l * p.G + i;
                const float ox = *rx, oy = *ry;
                const float a = fmaf(p.zen.Ap[l], ox, (p.zen.Bp[l] * gp) * dsum);
                const float b = fmaf(p.zen.As[l], oy, (p.zen.Bs[l] * gs) * ddif);
                srx += ox + a;
                sry += oy + b;
                *rx = a;
                *ry = b;
            }
            const float hl = 0.5f * (L + M);
            ux = fmaf(hl, srx, fmaf(M, sry, ux));
            uy = fmaf(hl, srx, fmaf(-M, sry, uy));
        }
        p.sxx[i] += ux;
        p.syy[i] += uy;
        if (p.feat) {
            p.feat[F_DX * p.G + i] = ddx;
            p.feat[F_DY * p.G + i] = ddy;
            p.feat[F_SXX * p.G + i] = srx;
            p.feat[F_SYY * p.G + i] = sry;
        }
    }
    if (ss) {
        float a = 0.f, b = 0.f, np_;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            a = fmaf(p.cd[0][c], p.vy[i + (int64_t)c * P] - p.vy[i - (int64_t)(c + 1) * P], a);
            b = fmaf(p.cd[1][c], p.vx[i + c + 1] - p.vx[i - c], b);
        }
        if (sx >= 0) {
            a = cpml(a, p.psi[1][ix], np_, p.tab_f[0][x]);
            p.psi[1][ix] = np_;
        }
        if (sy >= 0) {
            b = cpml(b, p.psi[3][iy], np_, p.tab_h[1][y]);
            p.psi[3][iy] = np_;
        }
        const float e = a + b, Ms = p.Ms[i];
        float u = Ms * e, sr = 0.f;
        if (ZM) {
            const float gs = ZM == 2 ? p.gs[i] : 1.f;
            for (int l = 0; l < L3; ++l) {
                float *rr = p.r[2] + l * p.G + i;
                const float o = *rr;
                const float n_ = fmaf(p.zen.As[l], o, (p.zen.Bs[l] * gs) * e);
                sr += o + n_;
                *rr = n_;
            }
            u = fmaf(0.5f * Ms, sr, u);
        }
        p.sxy[i] += u;
        if (p.feat) {
            p.feat[F_E * p.G + i] = e;
            p.feat[F_SXY * p.G + i] = sr;
        }
    }
}

template <int ORD>
__global__ void __launch_bounds__(BX *BY) k_fwd_velocity(const AdjParams p, int k) {
    // receivers: global thread g samples receiver g (syy is final for step k;
    // this kernel does not write it).  traces == null: not recorded.
    const int g = (blockIdx.y * gridDim.x + blockIdx.x) * (BX * BY) + threadIdx.y * BX + threadIdx.x;
    if (p.traces && g < p.n_rec && k >= p.rec_first[g]) {
        float acc = 0.f;
        for (int t = p.rec_start[g]; t < p.rec_start[g + 1]; ++t) acc += p.syy[p.rec_cell[t]];
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }
    const Node n = node(p);
    if (!n.live) return;
    const int x = n.x, y = n.y, P = p.P;
    const int64_t i = n.i;
    const bool vy_ = in_vy<ORD>(p, x, y), vx_ = in_vx<ORD>(p, x, y);
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
    const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;
    float vxn = 0.f, vyn = 0.f, ax = 0.f, ay = 0.f, np_;
    if (vx_) {
        float a = 0.f, b = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            a = fmaf(p.cd[0][c], p.sxx[i + (int64_t)c * P] - p.sxx[i - (int64_t)(c + 1) * P], a);
            b = fmaf(p.cd[1][c], p.sxy[i + c] - p.sxy[i - c - 1], b);
        }
        if (sx >= 0) {
            a = cpml(a, p.psi[4][ix], np_, p.tab_f[0][x]);
            p.psi[4][ix] = np_;
        }
        if (sy >= 0) {
            b = cpml(b, p.psi[6][iy], np_, p.tab_f[1][y]);
            p.psi[6][iy] = np_;
        }
        ax = a + b;
        vxn = fmaf(ax, p.Bx[i], p.vx[i]);
    }
    if (vy_) {
        float a = 0.f, b = 0.f;
#pragma unroll
        for (int c = 0; c < ORD; ++c) {
            a = fmaf(p.cd[0][c], p.sxy[i + (int64_t)(c + 1) * P] - p.sxy[i - (int64_t)c * P], a);
            b = fmaf(p.cd[1][c], p.syy[i + c + 1] - p.syy[i - c], b);
        }
        if (sx >= 0) {
            a = cpml(a, p.psi[5][ix], np_, p.tab_h[0][x]);
            p.psi[5][ix] = np_;
        }
        if (sy >= 0) {
            b = cpml(b, p.psi[7][iy], np_, p.tab_h[1][y]);
            p.psi[7][iy] = np_;
        }
        ay = a + b;
        vyn = fmaf(ay, p.By[i], p.vy[i]);
    }
    for (int q = 0; q < p.n_src; ++q)
        if (p.src_cell[q] == i && k < p.rows) vyn = fmaf(p.src_tab[(int64_t)k * p.ncol + p.src_col[q]], p.By[i], vyn);
    p.vx[i] = vxn;
    p.vy[i] = vyn;
    if (p.feat) {
        p.feat[F_AX * p.G + i] = ax;
        p.feat[F_AY * p.G + i] = ay;
    }
}

// ------------------------------------------------------------------ adjoint
// velocity nodes: (1) vbar gathers the transposed stress stencils of step
// k+1 (gather_stress), (2) pointwise velocity adjoint of step k, (3) the
// receiver residuals of step k enter syy^bar.
template <int ORD>
__global__ void __launch_bounds__(BX *BY) k_adj_velocity(const AdjParams p, int k, int gather_stress,
                                                          const float *feat_k) {
    const Node n = node(p);
    const int x = n.x, y = n.y, P = p.P;
    const int64_t i = n.i;
    if (n.live) {
        float avx = p.avx[i], avy = p.avy[i];
        if (gather_stress) {
            // vx from normal dx (x, +) and shear e_y (y, +); vy from normal dy (y, -) and shear e_x (x, -)
            auto dvx_at = [&](int xx, int yy) { return in_normal<ORD>(p, xx, yy) ? p.dv[0][(int64_t)xx * P + yy] : 0.f; };
            auto dvy_at = [&](int xx, int yy) { return in_normal<ORD>(p, xx, yy) ? p.dv[1][(int64_t)xx * P + yy] : 0.f; };
            auto dex_at = [&](int xx, int yy) { return in_shear<ORD>(p, xx, yy) ? p.dv[2][(int64_t)xx * P + yy] : 0.f; };
            auto dey_at = [&](int xx, int yy) { return in_shear<ORD>(p, xx, yy) ? p.dv[3][(int64_t)xx * P + yy] : 0.f; };
            float gx = 0.f, gy = 0.f;
#pragma unroll
            for (int c = 0; c < ORD; ++c) {
                gx = fmaf(p.cd[0][c], dvx_at(x - c - 1, y) - dvx_at(x + c, y), gx);
                gx = fmaf(p.cd[1][c], dey_at(x, y - c - 1) - dey_at(x, y + c), gx);
                gy = fmaf(p.cd[1][c], dvy_at(x, y - c) - dvy_at(x, y + c + 1), gy);
                gy = fmaf(p.cd[0][c], dex_at(x - c, y) - dex_at(x + c + 1, y), gy);
            }
            avx += gx;
            avy += gy;
        }
        // pointwise adjoint of the velocity update of step k
        const bool vy_ = in_vy<ORD>(p, x, y), vx_ = in_vx<ORD>(p, x, y);
        const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
        const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;
        float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
        if (vx_) {
            const float ab = p.Bx[i] * avx;
            p.gBx[i] += avx * feat_k[F_AX * p.G + i];
            d0 = ab;
            d1 = ab;
            if (sx >= 0) d0 = cpml_adj(ab, p.apsi[4][ix], p.tab_f[0][x]);
            if (sy >= 0) d1 = cpml_adj(ab, p.apsi[6][iy], p.tab_f[1][y]);
        }
        if (vy_) {
            const float ab = p.By[i] * avy;
            float gb = avy * feat_k[F_AY * p.G + i];
            for (int q = 0; q < p.n_src; ++q)
                if (p.src_cell[q] == i && k < p.rows) gb = fmaf(avy, p.src_tab[(int64_t)k * p.ncol + p.src_col[q]], gb);
            p.gBy[i] += gb;
            d2 = ab;
            d3 = ab;
            if (sx >= 0) d2 = cpml_adj(ab, p.apsi[5][ix], p.tab_h[0][x]);
            if (sy >= 0) d3 = cpml_adj(ab, p.apsi[7][iy], p.tab_h[1][y]);
        } else if (p.n_src > 0) {
            // outside the vy region a source node is overwritten, not updated
            float gb = 0.f;
            for (int q = 0; q < p.n_src; ++q)
                if (p.src_cell[q] == i && k < p.rows) gb = fmaf(avy, p.src_tab[(int64_t)k * p.ncol + p.src_col[q]], gb);
            p.gBy[i] += gb;
        }
        p.ds[0][i] = d0;
        p.ds[1][i] = d1;
        p.ds[2][i] = d2;
        p.ds[3][i] = d3;
        // v^bar of the state before step k: identity inside the updated
        // regions; outside the vy region the update overwrites v (adjoint 0)
        p.avx[i] = vy_ ? avx : 0.f;
        p.avy[i] = vy_ ? avy : 0.f;
    }
    // receiver residuals of step k into syy^bar (no other writer in this kernel)
    const int g = (blockIdx.y * gridDim.x + blockIdx.x) * (BX * BY) + threadIdx.y * BX + threadIdx.x;
    if (g < p.n_rec && k >= p.rec_first[g]) {
        const float r = p.res[(int64_t)k * p.n_rec + g];
        for (int t = p.rec_start[g]; t < p.rec_start[g + 1]; ++t) atomicAdd(p.asyy + p.rec_cell[t], r);
    }
}

template <int ORD, int ZM>
__global__ void __launch_bounds__(BX *BY) k_adj_stress(const AdjParams p, const float *feat_k) {
    const Node n = node(p);
    if (!n.live) return;
    const int x = n.x, y = n.y, P = p.P;
    const int64_t i = n.i;
    // transposed velocity stencils: gather the velocity-node dbar
    auto ax_x = [&](int xx, int yy) { return in_vx<ORD>(p, xx, yy) ? p.ds[0][(int64_t)xx * P + yy] : 0.f; };
    auto ax_y = [&](int xx, int yy) { return in_vx<ORD>(p, xx, yy) ? p.ds[1][(int64_t)xx * P + yy] : 0.f; };
    auto ay_x = [&](int xx, int yy) { return in_vy<ORD>(p, xx, yy) ? p.ds[2][(int64_t)xx * P + yy] : 0.f; };
    auto ay_y = [&](int xx, int yy) { return in_vy<ORD>(p, xx, yy) ? p.ds[3][(int64_t)xx * P + yy] : 0.f; };
    float sxx = p.asxx[i], syy = p.asyy[i], sxy = p.asxy[i];
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        sxx = fmaf(p.cd[0][c], ax_x(x - c, y) - ax_x(x + c + 1, y), sxx);
        sxy = fmaf(p.cd[1][c], ax_y(x, y - c) - ax_y(x, y + c + 1), sxy);
        sxy = fmaf(p.cd[0][c], ay_x(x - c - 1, y) - ay_x(x + c, y), sxy);
        syy = fmaf(p.cd[1][c], ay_y(x, y - c - 1) - ay_y(x, y + c), syy);
    }
    p.asxx[i] = sxx;
    p.asyy[i] = syy;
    p.asxy[i] = sxy;
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y);
    const int64_t ix = (int64_t)sx * P + y, iy = (int64_t)x * p.strip[1].width + sy;
    const int L3 = ZM ? p.zen.n : 0;
    float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
    if (in_normal<ORD>(p, x, y)) {
        const float L = p.L[i], M = p.M[i], L2M = fmaf(2.f, M, L);
        const float fdx = feat_k[F_DX * p.G + i], fdy = feat_k[F_DY * p.G + i];
        const float fsx = feat_k[F_SXX * p.G + i], fsy = feat_k[F_SYY * p.G + i];
        p.gL[i] += (sxx + syy) * (fdx + fdy + 0.5f * fsx);
        p.gM[i] += sxx * (2.f * fdx + 0.5f * fsx + fsy) + syy * (2.f * fdy + 0.5f * fsx - fsy);
        float bx = fmaf(L2M, sxx, L * syy), by = fmaf(L, sxx, L2M * syy);
        if (ZM) {
            const float gp = ZM == 2 ? p.gp[i] : 1.f, gs = ZM == 2 ? p.gs[i] : 1.f;
            const float Sx = 0.5f * (L + M) * (sxx + syy), Sy = M * (sxx - syy);
            float drx = 0.f, dry = 0.f;
            for (int l = 0; l < L3; ++l) {
                float *rx = p.ar[0] + l * p.G + i, *ry = p.ar[1] + l * p.G + i;
                const float qx = *rx + Sx, qy = *ry + Sy;
                *rx = fmaf(p.zen.Ap[l], qx, Sx);
                *ry = fmaf(p.zen.As[l], qy, Sy);
                drx = fmaf(p.zen.Bp[l] * gp, qx, drx);
                dry = fmaf(p.zen.Bs[l] * gs, qy, dry);
            }
            bx += drx + 0.5f * dry;
            by += drx - 0.5f * dry;
        }
        o0 = bx;
        o1 = by;
        if (sx >= 0) o0 = cpml_adj(bx, p.apsi[0][ix], p.tab_h[0][x]);
        if (sy >= 0) o1 = cpml_adj(by, p.apsi[2][iy], p.tab_f[1][y]);
    }
    if (in_shear<ORD>(p, x, y)) {
        const float Ms = p.Ms[i];
        const float fe = feat_k[F_E * p.G + i], fsr = feat_k[F_SXY * p.G + i];
        p.gMs[i] += sxy * (fe + 0.5f * fsr);
        float eb = Ms * sxy;
        if (ZM) {
            const float gs = ZM == 2 ? p.gs[i] : 1.f;
            const float S = 0.5f * Ms * sxy;
            for (int l = 0; l < L3; ++l) {
                float *rr = p.ar[2] + l * p.G + i;
                const float q = *rr + S;
                *rr = fmaf(p.zen.As[l], q, S);
                eb = fmaf(p.zen.Bs[l] * gs, q, eb);
            }
        }
        o2 = eb;
        o3 = eb;
        if (sx >= 0) o2 = cpml_adj(eb, p.apsi[1][ix], p.tab_f[0][x]);
        if (sy >= 0) o3 = cpml_adj(eb, p.apsi[3][iy], p.tab_h[1][y]);
    }
    p.dv[0][i] = o0;
    p.dv[1][i] = o1;
    p.dv[2][i] = o2;
    p.dv[3][i] = o3;
}

template <int ORD>
void launch_fwd(const AdjParams &p, int k, cudaStream_t st) {
    const dim3 block(BX, BY), grid((p.ny + BX - 1) / BX, (p.nx + BY - 1) / BY);
    if (p.zm == 0) k_fwd_stress<ORD, 0><<<grid, block, 0, st>>>(p);
    else if (p.zm == 1) k_fwd_stress<ORD, 1><<<grid, block, 0, st>>>(p);
    else k_fwd_stress<ORD, 2><<<grid, block, 0, st>>>(p);
    k_fwd_velocity<ORD><<<grid, block, 0, st>>>(p, k);
}

template <int ORD>
void launch_adj(const AdjParams &p, int k, int gather, const float *feat_k, cudaStream_t st) {
    const dim3 block(BX, BY), grid((p.ny + BX - 1) / BX, (p.nx + BY - 1) / BY);
    k_adj_velocity<ORD><<<grid, block, 0, st>>>(p, k, gather, feat_k);
    if (p.zm == 0) k_adj_stress<ORD, 0><<<grid, block, 0, st>>>(p, feat_k);
    else if (p.zm == 1) k_adj_stress<ORD, 1><<<grid, block, 0, st>>>(p, feat_k);
    else k_adj_stress<ORD, 2><<<grid, block, 0, st>>>(p, feat_k);
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
    int device = 0, rows = 0, nx = 0, ny = 0, P = 0, ord = 2, ckpt = 0, n_ckpt = 0;
    int src_cols = 0, src_rows = 0, n_src_el = 0;
    int64_t G = 0, state_floats = 0, adj_floats = 0, launches = 0;
    std::vector<void *> allocs;
    AdjParams p{};
    float *state = nullptr;     // forward state, one block: v, s, r, psi
    float *astate = nullptr;    // adjoint state, one block
    float *coefs = nullptr;     // own copy of L, M, Ms, Bx, By, g_p, g_s
    float *features = nullptr;  // [n_feat_steps][kF][G]
    int n_feat_steps = 0;
    float *checkpoints = nullptr;  // [n_ckpt][state_floats]
    std::vector<int> src_col_of_node;  // column (source index) of each source node
    float *src_tab = nullptr;
    int forward_done = 0;

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
    void launch_forward(int k, cudaStream_t st) {
        if (ord == 4) launch_fwd<4>(p, k, st);
        else launch_fwd<2>(p, k, st);
        launches += 2;
    }
    void launch_adjoint(int k, int gather, const float *feat_k, cudaStream_t st) {
        if (ord == 4) launch_adj<4>(p, k, gather, feat_k, st);
        else launch_adj<2>(p, k, gather, feat_k, st);
        launches += 2;
    }
    int copy_state(float *ckpt_slot, bool to_ckpt, cudaStream_t st) {
        cudaError_t e = to_ckpt ? cudaMemcpyAsync(ckpt_slot, state, state_floats * 4, cudaMemcpyDeviceToDevice, st)
                                : cudaMemcpyAsync(state, ckpt_slot, state_floats * 4, cudaMemcpyDeviceToDevice, st);
        return e == cudaSuccess ? TS_OK : afail(TS_E_CUDA, std::string("state copy: ") + cudaGetErrorString(e));
    }
    // source values of every source node for every step, in the reference's
    // flat indexing source_term[k * n_src_el + idx] (shader_webgpu_viscoelastic.wgsl:1050-1060)
    std::vector<float> source_table(const float *term) const {
        const int ncol = p.ncol;
        std::vector<float> tab((size_t)rows * ncol, 0.f);
        for (int k = 0; k < rows; ++k)
            for (int c = 0; c < ncol; ++c) {
                if (c >= n_src_el) continue;
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
    if (d->ord != 2 && d->ord != 4) return afail(TS_E_ARG, "the adjoint supports ord 2 and 4");
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
    AdjParams &p = a->p;
    p.nx = a->nx;
    p.ny = a->ny;
    p.P = a->P;
    p.ord = d->ord;
    p.G = a->G;
    p.zm = !d->visco ? 0 : (d->g_p ? 2 : 1);
    const float steps[2] = {d->dx, d->dy};
    for (int ax = 0; ax < 2; ++ax)
        for (int c = 0; c < kMaxOrd; ++c) p.cd[ax][c] = c < d->ord ? d->coefs[c] / steps[ax] : 0.f;
    p.zen = zener_constants(d);
    int rc;
    Axis axes[2] = {make_axis(a->nx, d->ord, d->a_x, d->b_x, d->k_x, d->a_xh, d->b_xh, d->k_xh),
                    make_axis(a->ny, d->ord, d->a_y, d->b_y, d->k_y, d->a_yh, d->b_yh, d->k_yh)};
    for (int ax = 0; ax < 2; ++ax) {
        Cpml *f = nullptr, *h = nullptr;
        if ((rc = a->upload(&f, axes[ax].full)) || (rc = a->upload(&h, axes[ax].half))) return bail(rc);
        p.tab_f[ax] = f;
        p.tab_h[ax] = h;
        p.strip[ax] = axes[ax].strip;
    }
    // state blocks: 5 fields, 3 x L memory variables, 8 strip memories (each
    // rounded to 64 floats); the adjoint block adds the 8 derivative adjoints
    const int64_t G = a->G, xs = (int64_t)p.strip[0].width * a->P, ys = (int64_t)a->nx * p.strip[1].width;
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
        float **f5[5] = {&p.vx, &p.vy, &p.sxx, &p.syy, &p.sxy};
        for (auto f : f5) *f = q, q += G;
        for (int m = 0; m < 3; ++m) p.r[m] = L ? q + (int64_t)m * L * G : nullptr;
        q += 3 * (int64_t)L * G;
        for (int k = 0; k < 8; ++k) p.psi[k] = q, q += r64(psz[k]);
        q = a->astate;
        float **a5[5] = {&p.avx, &p.avy, &p.asxx, &p.asyy, &p.asxy};
        for (auto f : a5) *f = q, q += G;
        for (int m = 0; m < 3; ++m) p.ar[m] = L ? q + (int64_t)m * L * G : nullptr;
        q += 3 * (int64_t)L * G;
        for (int k = 0; k < 8; ++k) p.apsi[k] = q, q += r64(psz[k]);
        for (int k = 0; k < 4; ++k) p.dv[k] = q, q += G;
        for (int k = 0; k < 4; ++k) p.ds[k] = q, q += G;
    }
    if ((rc = a->alloc(&a->coefs, (size_t)7 * G))) return bail(rc);
    p.L = a->coefs;
    p.M = a->coefs + G;
    p.Ms = a->coefs + 2 * G;
    p.Bx = a->coefs + 3 * G;
    p.By = a->coefs + 4 * G;
    p.gp = a->coefs + 5 * G;
    p.gs = a->coefs + 6 * G;
    // sources: every node of the source map, column = its source index
    {
        std::vector<int64_t> cells;
        std::vector<int> cols;
        int ncol = 0;
        for (int x = 0; x < a->nx; ++x)
            for (int y = 0; y < a->ny; ++y) {
                const int idx = d->pos_sources[(int64_t)x * a->ny + y];
                if (idx < 0) continue;
                cells.push_back((int64_t)x * a->P + y);
                cols.push_back(idx);
                ncol = std::max(ncol, idx + 1);
            }
        int64_t *dc = nullptr;
        int *dcol = nullptr;
        if ((rc = a->upload(&dc, cells)) || (rc = a->upload(&dcol, cols))) return bail(rc);
        p.n_src = (int)cells.size();
        p.src_cell = dc;
        p.src_col = dcol;
        p.ncol = std::max(1, ncol);
        p.rows = a->rows;
        if ((rc = a->alloc(&a->src_tab, (size_t)a->rows * p.ncol))) return bail(rc);
        p.src_tab = a->src_tab;
        if (d->source_term && (rc = ts_adj_set_sources(a, d->source_term))) return bail(rc);
        if (!d->source_term && cudaMemset(a->src_tab, 0, (size_t)a->rows * p.ncol * 4) != cudaSuccess)
            return bail(afail(TS_E_CUDA, "memset"));
    }
    // receivers: nodes of each receiver in info_rec_pt order (shader_webgpu_viscoelastic.wgsl:1118-1134)
    {
        std::vector<int> start(1, 0), first(std::max(1, d->n_rec), 0);
        std::vector<int64_t> cells;
        for (int r = 0; r < d->n_rec; ++r) {
            for (int pt = receiver_first_point(d, r, 3); pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * 3 + 2] == r;
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
        p.n_rec = d->n_rec;
        p.rec_start = ds;
        p.rec_first = df;
        p.rec_cell = dc;
    }
    // feature record: every step, or one K-step segment with checkpoints every K
    a->ckpt = checkpoint_every >= a->rows ? 0 : checkpoint_every;
    a->n_feat_steps = a->ckpt > 0 ? a->ckpt : a->rows;
    if ((rc = a->alloc(&a->features, (size_t)a->n_feat_steps * kF * G)))
        return bail(afail(rc, g_adj_error + " (feature record; a checkpoint interval keeps less)"));
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
    if (cudaDeviceSynchronize() != cudaSuccess)
        return afail(TS_E_CUDA, "synchronize");
    if (cudaMemcpy(a->src_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return afail(TS_E_CUDA, "cudaMemcpy");
    return TS_OK;
}

int ts_adj_read_field(ts_adj *a, int32_t what, void *host_dst, size_t bytes) {
    if (!a || !host_dst) return afail(TS_E_ARG, "null argument");
    const AdjParams &p = a->p;
    const float *src = what == TS_VX ? p.vx : what == TS_VY ? p.vy : what == TS_SXX ? p.sxx
                     : what == TS_SYY ? p.syy : what == TS_SXY ? p.sxy : nullptr;
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

int ts_adj_launch_count(const ts_adj *a, int64_t *launches) {
    if (!a || !launches) return afail(TS_E_ARG, "null argument");
    *launches = a->launches;
    return TS_OK;
}

int ts_adj_forward(ts_adj *a, const ts_adj_coefs *c, float *traces, void *stream) {
    if (!a || !c || !traces || !c->L || !c->M || !c->Ms || !c->Bx || !c->By) return afail(TS_E_ARG, "null argument");
    if (a->p.zm == 2 && (!c->g_p || !c->g_s)) return afail(TS_E_ARG, "per-cell Q scales g_p, g_s required");
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    AdjParams &p = a->p;
    const int64_t G = a->G;
    const float *src[7] = {c->L, c->M, c->Ms, c->Bx, c->By, c->g_p, c->g_s};
    for (int q = 0; q < (a->p.zm == 2 ? 7 : 5); ++q)
        if (cudaMemcpyAsync(a->coefs + q * G, src[q], G * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return afail(TS_E_CUDA, "coefficient copy");
    if (cudaMemsetAsync(a->state, 0, a->state_floats * 4, st) != cudaSuccess ||
        cudaMemsetAsync(traces, 0, (size_t)a->rows * std::max(1, p.n_rec) * 4, st) != cudaSuccess)
        return afail(TS_E_CUDA, "memset");
    p.traces = traces;
    int rc;
    for (int k = 0; k < a->rows; ++k) {
        if (a->ckpt > 0 && k % a->ckpt == 0 &&
            (rc = a->copy_state(a->checkpoints + (int64_t)(k / a->ckpt) * a->state_floats, true, st)))
            return rc;
        p.feat = a->ckpt > 0 ? nullptr : a->features + (int64_t)k * kF * G;
        a->launch_forward(k, st);
    }
    p.feat = nullptr;
    p.traces = nullptr;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(TS_E_CUDA, cudaGetErrorString(e));
    a->forward_done = 1;
    return TS_OK;
}

int ts_adj_backward(ts_adj *a, const float *residual, const ts_adj_grads *g, void *stream) {
    if (!a || !residual || !g || !g->gL || !g->gM || !g->gMs || !g->gBx || !g->gBy) return afail(TS_E_ARG, "null argument");
    if (!a->forward_done) return afail(TS_E_STATE, "ts_adj_forward must run first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    AdjParams &p = a->p;
    const int64_t G = a->G;
    p.res = residual;
    p.gL = g->gL;
    p.gM = g->gM;
    p.gMs = g->gMs;
    p.gBx = g->gBx;
    p.gBy = g->gBy;
    p.traces = nullptr;
    if (cudaMemsetAsync(a->astate, 0, a->adj_floats * 4, st) != cudaSuccess) return afail(TS_E_CUDA, "memset");
    for (float *q : {g->gL, g->gM, g->gMs, g->gBx, g->gBy})
        if (cudaMemsetAsync(q, 0, (size_t)G * 4, st) != cudaSuccess) return afail(TS_E_CUDA, "memset");
    int rc;
    if (a->ckpt <= 0) {
        for (int k = a->rows - 1; k >= 0; --k) a->launch_adjoint(k, k < a->rows - 1, a->features + (int64_t)k * kF * G, st);
    } else {
        for (int s = a->n_ckpt - 1; s >= 0; --s) {
            const int k0 = s * a->ckpt, k1 = std::min(a->rows, k0 + a->ckpt);
            // recompute the segment from its checkpoint, recording its features
            if ((rc = a->copy_state(a->checkpoints + (int64_t)s * a->state_floats, false, st))) return rc;
            for (int k = k0; k < k1; ++k) {
                p.feat = a->features + (int64_t)(k - k0) * kF * G;
                a->launch_forward(k, st);
            }
            p.feat = nullptr;
            for (int k = k1 - 1; k >= k0; --k)
                a->launch_adjoint(k, k < a->rows - 1, a->features + (int64_t)(k - k0) * kF * G, st);
        }
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(TS_E_CUDA, cudaGetErrorString(e));
    return TS_OK;
}

}  // extern "C"
