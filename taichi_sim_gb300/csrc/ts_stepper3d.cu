// 3D staggered-grid (visco)elastic time step on sm_103a.
//
// One time step = k_stress3d (sxx, syy, szz, sxy, sxz, syz with CPML strips
// and the Zener update fused) followed by k_velocity3d (vx, vy, vz with
// CPML, Dirichlet zeroing, source injection, receiver sampling of szz and
// stability bookkeeping fused).  Thread (tx, ty, tz) owns node
// (z = 32 bx + tx, y = 4 by + ty, x = 2 bz + tz): z is the contiguous axis.
// As in 2D, every load of a node is issued before its first store so that
// one memory latency is paid per node.
//
// Semantics: family TS_WGSL3D, shader_webgpu_3D_viscoelastic.wgsl:1341-1773
// and :1824-1843, including its quirks (normal stresses use point
// rho/cp/cs, shear moduli average rho and cs over 4 nodes without the
// cs == 0 test, vz uses the vy-node density, all three velocities are zeroed
// outside the vz region, the source drives vz).
#include <cuda_runtime.h>
#include "ts_internal.cuh"

namespace ts {
namespace {

__device__ __forceinline__ float cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = fmaf(t.b, psi_old, t.a * d);
    return fmaf(d, t.ik, psi_new);
}

// Stencil values of one staggered derivative: hi[c] - lo[c] pairs.
// PLUS: f[i + (c+1) s] - f[i - c s]; otherwise f[i + c s] - f[i - (c+1) s].
template <int ORD>
struct Pairs {
    float hi[ORD], lo[ORD];
};

template <int ORD, bool PLUS>
__device__ __forceinline__ Pairs<ORD> load_pairs(const float *__restrict__ f, int64_t i, int64_t s) {
    Pairs<ORD> r;
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        r.hi[c] = __ldg(f + i + (PLUS ? (c + 1) : c) * s);
        r.lo[c] = __ldg(f + i - (PLUS ? c : (c + 1)) * s);
    }
    return r;
}

template <int ORD>
__device__ __forceinline__ float deriv(const Pairs<ORD> &q, const float *cd) {
    float a = 0.f;
#pragma unroll
    for (int c = 0; c < ORD; ++c) a = fmaf(cd[c], q.hi[c] - q.lo[c], a);
    return a;
}

template <int ORD, int ZM, int NS>
__global__ void __launch_bounds__(kBX3 *kBY3 *kBZ3) k_stress3d(const StepParams p) {
    const int z = blockIdx.x * kBX3 + threadIdx.x;
    const int y = blockIdx.y * kBY3 + threadIdx.y;
    const int x = blockIdx.z * kBZ3 + threadIdx.z;
    const bool in_n = x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1 && z >= ORD && z < p.nz - ORD + 1;
    const bool in_xy = x >= ORD && x < p.nx - ORD + 1 && y >= ORD - 1 && y < p.ny - ORD && z >= ORD - 1 && z < p.nz - ORD;
    const bool in_yz = x >= ORD - 1 && x < p.nx - ORD && y >= ORD - 1 && y < p.ny - ORD && z >= ORD - 1 && z < p.nz - ORD;
    if (!in_n && !in_xy && !in_yz) return;
    const int64_t X = p.plane, Y = p.pitch;
    const int64_t i = (int64_t)x * X + y * Y + z;
    const float *vx = p.v[0], *vy = p.v[1], *vz = p.v[2];
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
    const int64_t ix = ((int64_t)sx * p.ny + y) * p.pitch + z;
    const int64_t iy = ((int64_t)x * p.strip[1].width + sy) * p.pitch + z;
    const int64_t iz = ((int64_t)x * p.ny + y) * p.strip[2].width + sz;
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    const int64_t G = p.grid_elems;
    constexpr int R = NS > 0 ? NS : 1;

    // ---------------- loads ----------------
    // per-node coefficients (never written) before waiting for the previous kernel
    float L = 0.f, M = 0.f, gp = 1.f, gs = 1.f, Mxy = 0.f, Mxz = 0.f, Myz = 0.f;
    if (in_n) {
        L = __ldg(p.lam_dt + i);
        M = __ldg(p.mu_dt + i);
        if (ZM == 2) gp = __ldg(p.g_p + i);
    }
    if (in_xy) {
        Mxy = __ldg(p.mus_dt[0] + i);
        Mxz = __ldg(p.mus_dt[1] + i);
    }
    if (in_yz) Myz = __ldg(p.mus_dt[2] + i);
    if (ZM == 2) gs = __ldg(p.g_s + i);
    pdl_wait();
    Pairs<ORD> n_x, n_y, n_z, a_vy, a_vx, b_vz, b_vx, c_vz, c_vy;
    float s_n[3] = {0.f, 0.f, 0.f};
    float s_xy = 0.f, s_xz = 0.f, s_yz = 0.f;
    float psi[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float r0[R], r1[R], r2[R], r3[R], r4[R], r5[R];
    if (in_n) {
        n_x = load_pairs<ORD, true>(vx, i, X);
        n_y = load_pairs<ORD, false>(vy, i, Y);
        n_z = load_pairs<ORD, false>(vz, i, 1);
        s_n[0] = p.s[0][i];
        s_n[1] = p.s[1][i];
        s_n[2] = p.s[2][i];
        if (sx >= 0) psi[0] = p.psi[0][ix];
        if (sy >= 0) psi[1] = p.psi[1][iy];
        if (sz >= 0) psi[2] = p.psi[2][iz];
        if (ZM != 0) {
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) {
                    r0[l] = p.r[0][l * G + i];
                    r1[l] = p.r[1][l * G + i];
                    r2[l] = p.r[2][l * G + i];
                }
        }
    }
    if (in_xy) {
        a_vy = load_pairs<ORD, false>(vy, i, X);
        a_vx = load_pairs<ORD, true>(vx, i, Y);
        b_vz = load_pairs<ORD, false>(vz, i, X);
        b_vx = load_pairs<ORD, true>(vx, i, 1);
        s_xy = p.s[3][i];
        s_xz = p.s[4][i];
        if (sx >= 0) {
            psi[3] = p.psi[3][ix];
            psi[5] = p.psi[5][ix];
        }
        if (sy >= 0) psi[4] = p.psi[4][iy];
        if (sz >= 0) psi[6] = p.psi[6][iz];
        if (ZM != 0) {
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) {
                    r3[l] = p.r[3][l * G + i];
                    r4[l] = p.r[4][l * G + i];
                }
        }
    }
    if (in_yz) {
        c_vz = load_pairs<ORD, true>(vz, i, Y);
        c_vy = load_pairs<ORD, true>(vy, i, 1);
        s_yz = p.s[5][i];
        if (sy >= 0) psi[7] = p.psi[7][iy];
        if (sz >= 0) psi[8] = p.psi[8][iz];
        if (ZM != 0) {
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) r5[l] = p.r[5][l * G + i];
        }
    }

    // ---------------- normal stresses ----------------
    if (in_n) {
        float ddx = deriv(n_x, p.cd[0]), ddy = deriv(n_y, p.cd[1]), ddz = deriv(n_z, p.cd[2]);
        float np_;
        if (sx >= 0) {
            ddx = cpml(ddx, psi[0], np_, p.tab_h[0][x]);
            p.psi[0][ix] = np_;
        }
        if (sy >= 0) {
            ddy = cpml(ddy, psi[1], np_, p.tab_f[1][y]);
            p.psi[1][iy] = np_;
        }
        if (sz >= 0) {
            ddz = cpml(ddz, psi[2], np_, p.tab_f[2][z]);
            p.psi[2][iz] = np_;
        }
        const float L2M = fmaf(2.f, M, L);
        float ux = fmaf(L2M, ddx, L * (ddy + ddz));
        float uy = fmaf(L2M, ddy, L * (ddx + ddz));
        float uz = fmaf(L2M, ddz, L * (ddx + ddy));
        if (ZM != 0) {
            const float div = ddx + ddy + ddz;
            const float third = div * (1.f / 3.f);
            const float dy_ = ddx - third, dz_ = ddy - third;
            float srxx = 0.f, sryy = 0.f, srzz = 0.f;
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) {
                    const float a = fmaf(p.zen.Ap[l], r0[l], (p.zen.Bp[l] * gp) * div);
                    const float b = fmaf(p.zen.As[l], r1[l], (p.zen.Bs[l] * gs) * dy_);
                    const float c = fmaf(p.zen.As[l], r2[l], (p.zen.Bs[l] * gs) * dz_);
                    srxx += r0[l] + a;
                    sryy += r1[l] + b;
                    srzz += r2[l] + c;
                    p.r[0][l * G + i] = a;
                    p.r[1][l * G + i] = b;
                    p.r[2][l * G + i] = c;
                }
            const float hl23 = 0.5f * fmaf(2.f / 3.f, M, L);
            ux = fmaf(hl23, srxx, fmaf(M, sryy, ux));
            uy = fmaf(hl23, srxx, fmaf(M, srzz, uy));
            uz = fmaf(0.5f * L2M, srxx, fmaf(-M * (1.f / 3.f), sryy + srzz, uz));
        }
        p.s[0][i] = s_n[0] + ux;
        p.s[1][i] = s_n[1] + uy;
        p.s[2][i] = s_n[2] + uz;
    }
    // ---------------- sigma_xy, sigma_xz ----------------
    if (in_xy) {
        float a1 = deriv(a_vy, p.cd[0]), a2 = deriv(a_vx, p.cd[1]);
        float b1 = deriv(b_vz, p.cd[0]), b2 = deriv(b_vx, p.cd[2]);
        float np_;
        if (sx >= 0) {
            a1 = cpml(a1, psi[3], np_, p.tab_f[0][x]);
            p.psi[3][ix] = np_;
            b1 = cpml(b1, psi[5], np_, p.tab_f[0][x]);
            p.psi[5][ix] = np_;
        }
        if (sy >= 0) {
            a2 = cpml(a2, psi[4], np_, p.tab_h[1][y]);
            p.psi[4][iy] = np_;
        }
        if (sz >= 0) {
            b2 = cpml(b2, psi[6], np_, p.tab_h[2][z]);
            p.psi[6][iz] = np_;
        }
        const float ea = a1 + a2, eb = b1 + b2;
        float u = Mxy * ea, w = Mxz * eb;
        if (ZM != 0) {
            float sa = 0.f, sb = 0.f;
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) {
                    const float na = fmaf(p.zen.As[l], r3[l], (p.zen.Bs[l] * gs) * ea);
                    const float nb = fmaf(p.zen.As[l], r4[l], (p.zen.Bs[l] * gs) * eb);
                    sa += r3[l] + na;
                    sb += r4[l] + nb;
                    p.r[3][l * G + i] = na;
                    p.r[4][l * G + i] = nb;
                }
            u = fmaf(0.5f * Mxy, sa, u);
            w = fmaf(0.5f * Mxz, sb, w);
        }
        p.s[3][i] = s_xy + u;
        p.s[4][i] = s_xz + w;
    }
    // ---------------- sigma_yz ----------------
    if (in_yz) {
        float a1 = deriv(c_vz, p.cd[1]), a2 = deriv(c_vy, p.cd[2]);
        float np_;
        if (sy >= 0) {
            a1 = cpml(a1, psi[7], np_, p.tab_h[1][y]);
            p.psi[7][iy] = np_;
        }
        if (sz >= 0) {
            a2 = cpml(a2, psi[8], np_, p.tab_h[2][z]);
            p.psi[8][iz] = np_;
        }
        const float e = a1 + a2;
        float u = Myz * e;
        if (ZM != 0) {
            float sr = 0.f;
#pragma unroll
            for (int l = 0; l < R; ++l)
                if (l < n_mech) {
                    const float n_ = fmaf(p.zen.As[l], r5[l], (p.zen.Bs[l] * gs) * e);
                    sr += r5[l] + n_;
                    p.r[5][l * G + i] = n_;
                }
            u = fmaf(0.5f * Myz, sr, u);
        }
        p.s[5][i] = s_yz + u;
    }
    pdl_trigger();
}

template <int ORD>
__global__ void __launch_bounds__(kBX3 *kBY3 *kBZ3) k_velocity3d(const StepParams p, const int j) {
    const int z = blockIdx.x * kBX3 + threadIdx.x;
    const int y = blockIdx.y * kBY3 + threadIdx.y;
    const int x = blockIdx.z * kBZ3 + threadIdx.z;
    const int tid = (threadIdx.z * kBY3 + threadIdx.y) * kBX3 + threadIdx.x;
    const int blk = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const bool live = x < p.nx && y < p.ny && z < p.nz;
    const int64_t X = p.plane, Y = p.pitch;
    const int64_t i = (int64_t)x * X + y * Y + z;
    const float *sxx = p.s[0], *syy = p.s[1], *szz = p.s[2], *sxy = p.s[3], *sxz = p.s[4], *syz = p.s[5];
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
    const int64_t ix = ((int64_t)sx * p.ny + y) * p.pitch + z;
    const int64_t iy = ((int64_t)x * p.strip[1].width + sy) * p.pitch + z;
    const int64_t iz = ((int64_t)x * p.ny + y) * p.strip[2].width + sz;
    // vz region; outside it all three components are zero (wgsl:1754-1758)
    const bool in_vz = live && x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1 && z >= ORD - 1 &&
                       z < p.nz - ORD;
    const bool in_vx = in_vz && x >= ORD && z >= ORD;        // vx region within the vz region
    const bool in_vy = in_vz && y < p.ny - ORD && z >= ORD;  // vy region within the vz region
    const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
    const float dtx = in_vx ? __ldg(p.dtr[0] + i) : 0.f;
    const float dty = in_vz ? __ldg(p.dtr[1] + i) : 0.f;
    pdl_wait();
    const int k = *p.step_base + j;

    // ---------------- loads ----------------
    Pairs<ORD> xa, xb, xe, ya, yb, ye, za, zb, ze;
    float v0[3] = {0.f, 0.f, 0.f};
    float psi[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (in_vx) {
        xa = load_pairs<ORD, false>(sxx, i, X);
        xb = load_pairs<ORD, false>(sxy, i, Y);
        xe = load_pairs<ORD, false>(sxz, i, 1);
        v0[0] = p.v[0][i];
        if (sx >= 0) psi[0] = p.psi[9][ix];
        if (sy >= 0) psi[1] = p.psi[10][iy];
        if (sz >= 0) psi[2] = p.psi[11][iz];
    }
    if (in_vy) {
        ya = load_pairs<ORD, true>(sxy, i, X);
        yb = load_pairs<ORD, true>(syy, i, Y);
        ye = load_pairs<ORD, false>(syz, i, 1);
        v0[1] = p.v[1][i];
        if (sx >= 0) psi[3] = p.psi[12][ix];
        if (sy >= 0) psi[4] = p.psi[13][iy];
        if (sz >= 0) psi[5] = p.psi[14][iz];
    }
    if (in_vz) {
        za = load_pairs<ORD, true>(sxz, i, X);
        zb = load_pairs<ORD, false>(syz, i, Y);
        ze = load_pairs<ORD, true>(szz, i, 1);
        v0[2] = p.v[2][i];
        if (sx >= 0) psi[6] = p.psi[15][ix];
        if (sy >= 0) psi[7] = p.psi[16][iy];
        if (sz >= 0) psi[8] = p.psi[17][iz];
    }

    // ---------------- update ----------------
    float v2 = 0.f;
    if (live) {
        float vxn = 0.f, vyn = 0.f, vzn = 0.f, np_;
        if (in_vx) {
            float a = deriv(xa, p.cd[0]), b = deriv(xb, p.cd[1]), e = deriv(xe, p.cd[2]);
            if (sx >= 0) {
                a = cpml(a, psi[0], np_, p.tab_f[0][x]);
                p.psi[9][ix] = np_;
            }
            if (sy >= 0) {
                b = cpml(b, psi[1], np_, p.tab_f[1][y]);
                p.psi[10][iy] = np_;
            }
            if (sz >= 0) {
                e = cpml(e, psi[2], np_, p.tab_f[2][z]);
                p.psi[11][iz] = np_;
            }
            vxn = fmaf(a + b + e, dtx, v0[0]);
        }
        if (in_vy) {
            float a = deriv(ya, p.cd[0]), b = deriv(yb, p.cd[1]), e = deriv(ye, p.cd[2]);
            if (sx >= 0) {
                a = cpml(a, psi[3], np_, p.tab_h[0][x]);
                p.psi[12][ix] = np_;
            }
            if (sy >= 0) {
                b = cpml(b, psi[4], np_, p.tab_h[1][y]);
                p.psi[13][iy] = np_;
            }
            if (sz >= 0) {
                e = cpml(e, psi[5], np_, p.tab_f[2][z]);
                p.psi[14][iz] = np_;
            }
            vyn = fmaf(a + b + e, dty, v0[1]);
        }
        if (in_vz) {
            float a = deriv(za, p.cd[0]), b = deriv(zb, p.cd[1]), e = deriv(ze, p.cd[2]);
            if (sx >= 0) {
                a = cpml(a, psi[6], np_, p.tab_h[0][x]);
                p.psi[15][ix] = np_;
            }
            if (sy >= 0) {
                b = cpml(b, psi[7], np_, p.tab_f[1][y]);
                p.psi[16][iy] = np_;
            }
            if (sz >= 0) {
                e = cpml(e, psi[8], np_, p.tab_h[2][z]);
                p.psi[17][iz] = np_;
            }
            vzn = fmaf(a + b + e, dty, v0[2]);  // the vy-node density (wgsl3d:1748)
        }
        for (int q = q0; q < q1; ++q) {
            const Source s = p.src[q];
            if (s.cell == i && k < p.src_rows)
                vzn = fmaf(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, vzn);
        }
        p.v[0][i] = vxn;
        p.v[1][i] = vyn;
        p.v[2][i] = vzn;
        v2 = fmaf(vxn, vxn, fmaf(vyn, vyn, vzn * vzn));
    }

    const int g = blk * (kBX3 * kBY3 * kBZ3) + tid;
    if (g < p.n_rec && k >= __ldg(p.rec_first_step + g)) {
        float acc = 0.f;
        for (int q = __ldg(p.rec_start + g); q < __ldg(p.rec_start + g + 1); ++q) acc += p.s[2][__ldg(p.rec_cell + q)];
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }

    warp_stability(v2, live && !(v2 <= p.v2_threshold), reinterpret_cast<unsigned *>(p.block_max) + blk,
                   p.first_bad, k);
    pdl_trigger();
}

template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    dim3 block(kBX3, kBY3, kBZ3);
    dim3 grid((p.nz + kBX3 - 1) / kBX3, (p.ny + kBY3 - 1) / kBY3, (p.nx + kBZ3 - 1) / kBZ3);
    const bool three = p.zen.n == 3;
    if (parts & 1) {
        if (zen_mode == 0) launch_pdl(k_stress3d<ORD, 0, 0>, grid, block, st, p);
        else if (zen_mode == 1 && three) launch_pdl(k_stress3d<ORD, 1, 3>, grid, block, st, p);
        else if (zen_mode == 1) launch_pdl(k_stress3d<ORD, 1, kMaxSls>, grid, block, st, p);
        else if (three) launch_pdl(k_stress3d<ORD, 2, 3>, grid, block, st, p);
        else launch_pdl(k_stress3d<ORD, 2, kMaxSls>, grid, block, st, p);
    }
    if (parts & 2) launch_pdl(k_velocity3d<ORD>, grid, block, st, p, j);
}

}  // namespace

int blocks_3d(const StepParams &p) {
    return ((p.nz + kBX3 - 1) / kBX3) * ((p.ny + kBY3 - 1) / kBY3) * ((p.nx + kBZ3 - 1) / kBZ3);
}

void launch_step_3d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts) {
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
